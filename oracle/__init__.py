"""CPU oracle for the accelerate-fft GPU path.

Test infrastructure only: tests/, ``__graft_entry__.smoke()`` and the CPU
baseline / reference legs of ``bench.py`` may use it, as the checker or as the
timed CPU baseline.  The product path never imports it.

Parity is unpinned for values (the reference ships no golden vectors and
cannot be built here); see adhoc.cpp for what is restated and how it is
checked.
"""
