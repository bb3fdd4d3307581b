"""The allocation-free entry point gbfft_fft_noalloc.

It exists for callers that cannot allocate device memory: a host that owns the
device heap (Accelerate's PTX backend hands the FFI arrays from its own
allocator) or code recording a CUDA graph by stream capture, where cudaMalloc
is not allowed.  Its work area is a fixed __device__ array, so this test calls
it through the C ABI twice in a row (two lengths, so the shared array is
rewritten between calls) and checks each result against the planned entry
point gbfft_fft on the same input, within the Bluestein tolerance the parity
tests use (4e-6 relative L2).  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 4e-6


def _rel(a, b):
    return float(torch.linalg.vector_norm((a - b).to(torch.complex128)) /
                 torch.linalg.vector_norm(b.to(torch.complex128)))


def test_noalloc_matches_planned_entry_point(gbfft_lib):
    from gbfft import _lib as L
    lib = L.lib()
    rng = np.random.default_rng(77)
    cases = [(5003, 3, L.FORWARD), (1009, 4, L.INVERSE), (5003, 3, L.REVERSE)]
    for n, batch, mode in cases:
        x = torch.from_numpy((rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n)))
                             .astype(np.complex64)).cuda()
        y_na = torch.empty_like(x)
        y_ref = torch.empty_like(x)
        st = lib.gbfft_fft_noalloc(mode, n, batch, L.C32, ctypes.c_void_p(x.data_ptr()),
                                   ctypes.c_void_p(y_na.data_ptr()), None)
        assert st == L.OK, L.error_string(st)
        dims = (ctypes.c_int64 * 2)(batch, n)
        st = lib.gbfft_fft(mode, 2, dims, L.KIND_MANY, L.C32, ctypes.c_void_p(x.data_ptr()),
                           ctypes.c_void_p(y_ref.data_ptr()), None)
        assert st == L.OK
        torch.cuda.synchronize()
        assert _rel(y_na, y_ref) < TOL, (n, batch, mode, _rel(y_na, y_ref))


def test_noalloc_rejects_sizes_beyond_its_work_area(gbfft_lib):
    from gbfft import _lib as L
    lib = L.lib()
    x = torch.zeros(16, dtype=torch.complex64, device="cuda")
    y = torch.zeros(16, dtype=torch.complex64, device="cuda")
    # 4096 rows of length 4096: 2 * 4096 * 8192 * 8 bytes of work > 16 MiB
    st = lib.gbfft_fft_noalloc(L.FORWARD, 4096, 4096, L.C32, ctypes.c_void_p(x.data_ptr()),
                               ctypes.c_void_p(y.data_ptr()), None)
    assert st == L.ERR_TOO_LARGE
    assert "fixed work area" in L.error_string(st)
    st = lib.gbfft_fft_noalloc(L.FORWARD, 1 << 25, 1, L.C32, ctypes.c_void_p(x.data_ptr()),
                               ctypes.c_void_p(y.data_ptr()), None)
    assert st == L.ERR_TOO_LARGE
