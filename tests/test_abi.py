"""CPU tests of the C ABI boundary: libgbfft.so builds, loads, exports every
function include/gbfft.h declares, and its host-only planner picks the
expected passes (no GPU call)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def header_functions():
    src = open(os.path.join(ROOT, "include", "gbfft.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbfft_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(gbfft_lib):
    from gbfft import _lib as L
    lib = L.lib()
    names = header_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
        assert n in L.SIGNATURES, "python binding lacks " + n


def test_error_strings_and_version(gbfft_lib):
    from gbfft import _lib as L
    lib = L.lib()
    assert lib.gbfft_version() >= 100
    for st in range(8):
        assert lib.gbfft_error_string(st)
    assert lib.gbfft_error_string(99) == b"unknown status"


def explain(dims, kind=1, dtype=0, precision=0):
    from gbfft import _lib as L
    buf = ctypes.create_string_buffer(8192)
    d = (ctypes.c_int64 * len(dims))(*dims)
    st = L.lib().gbfft_plan_explain(len(dims), d, kind, dtype, precision, buf, 8192)
    return st, buf.value.decode()


def test_planner_choices(gbfft_lib):
    st, s = explain((4096, 4096))
    assert st == 0 and "launches=2" in s and "scratch=0" in s
    st, s = explain((65536, 1000), kind=0)
    assert st == 0 and "[n=1000 r=10.10.10 es=1 row" in s and "launches=1" in s
    st, s = explain((4096, 1009), kind=0)
    assert st == 0 and "bluestein m=2048" in s and "launches=1" in s
    st, s = explain((65536,))
    assert st == 0 and "four-step" in s and "launches=2" in s and "scratch=0" in s
    st, s = explain((65521,))
    assert st == 0 and "bluestein m=131072" in s and "3-pass" in s and "launches=3" in s
    st, s = explain((8192,), dtype=1)  # Complex Double: four-step above 4096
    assert st == 0 and "four-step" in s
    st, s = explain((256, 256, 256))
    assert st == 0 and "launches=3" in s
    st, s = explain((1, 1, 1))
    assert st == 0 and "launches=0" in s


@pytest.mark.parametrize("n,radices", [(4096, "16.16.16"), (2048, "16.16.8"), (512, "16.16.2"),
                                       (243, "9.9.3"), (250, "10.5.5"), (210, "15.14"), (189, "9.7.3"),
                                       (105, "15.7"), (343, "7.7.7"), (2025, "15.15.9"), (12, "12"),
                                       (6, "6"), (3 * 2048, "16.16.12.2")])
def test_stage_radices(gbfft_lib, n, radices):
    """Powers of two keep radix 16 then 8/4/2 (the register kernels' lists);
    lengths with odd factors take the fewest stages over radices up to 16,
    composite 6/9/10/12/14/15 included, larger radices first."""
    st, s = explain((4, n), kind=0)
    assert st == 0 and ("r=%s " % radices) in s, s


def test_planner_rejects_bad_arguments(gbfft_lib):
    assert explain((4, -1))[0] == 1
    assert explain((4, 4), kind=9)[0] == 1
    assert explain((4, 4), dtype=5)[0] == 1


def test_tune_file_parser(gbfft_lib, tmp_path):
    """The autotuner's JSON-lines cache file loads without a GPU; malformed
    lines are skipped."""
    from gbfft import _lib as L
    lib = L.lib()
    f = tmp_path / "tune.jsonl"
    f.write_text(
        '{"key": "devA|2|4096x4096|1|0|0", "row_variant": 1, "row_tma": 1, "col_variant": 9, '
        '"split_rank": 0, "str_tma": 1, "ms": 0.15}\n'
        'not json at all\n'
        '{"key": "devA|1|65536|0|0|0", "row_variant": 0, "row_tma": 0, "col_variant": 14, '
        '"split_rank": 2, "str_tma": 0, "ms": 0.5}\n'
        '{"key": "devA|1|7|0|0|0", "row_variant": 1}\n')
    lib.gbfft_tune_clear()
    assert lib.gbfft_tune_count() == 0
    assert lib.gbfft_tune_load(str(f).encode()) == 2
    assert lib.gbfft_tune_count() == 2
    assert lib.gbfft_tune_load(str(tmp_path / "missing.jsonl").encode()) == 0
    lib.gbfft_tune_clear()
    assert lib.gbfft_tune_count() == 0


def test_argument_checks_need_no_device(gbfft_lib):
    """Entry points reject bad arguments before touching CUDA: the fused
    centre/shift execution, the Centre.hs kernels and the bandwidth probe."""
    from gbfft import _lib as L
    lib = L.lib()
    vp = ctypes.c_void_p
    assert lib.gbfft_exec_ex(None, L.FORWARD, None, None, None, L.OPT_SHIFT_OUT) == L.ERR_NULL_PLAN
    d3 = (ctypes.c_int64 * 4)(2, 3, 4, 5)
    assert lib.gbfft_centre(4, d3, L.C32, vp(16), vp(32), None) == L.ERR_INVALID_ARG  # rank 1..3
    assert lib.gbfft_centre(2, d3, 7, vp(16), vp(32), None) == L.ERR_INVALID_ARG  # element type
    assert lib.gbfft_shift(2, d3, L.C32, 0, vp(16), vp(16), None) == L.ERR_INVALID_ARG  # in place
    z = (ctypes.c_int64 * 2)(0, 5)
    assert lib.gbfft_shift(2, z, L.C32, 1, None, None, None) == L.OK  # empty: nothing to do
    assert lib.gbfft_probe_tile_copy(300, 256, 24, vp(16), vp(4096), None) == L.ERR_INVALID_ARG
    assert lib.gbfft_probe_tile_copy(300, 256, 3, vp(16), vp(4096), None) == L.ERR_INVALID_ARG
    assert lib.gbfft_probe_tile_copy(4, 4, 2, None, None, None) == L.ERR_INVALID_ARG
    assert lib.gbfft_probe_tile_copy(4, 4, 2, vp(8), vp(4096), None) == L.ERR_INVALID_ARG  # 16-byte aligned
