"""The allocation-free entry point gbfft_fft_noalloc.

It exists for callers that cannot allocate device memory, such as a host that
owns the device heap and keeps its own account of it (Accelerate's PTX backend
hands the FFI arrays from its own allocator).  Its work area is a fixed
__device__ array shared by every call, so these tests call it through the C
ABI several times in a row -- different lengths and both element types, so the
tables held in the array are rewritten between calls -- and check every result
against the planned entry point gbfft_fft on the same input and against an
FP64 FFT, within the tolerances the parity tests use (4e-6 relative L2 for
Complex Float Bluestein, 1e-12 for Complex Double).  One test makes a second
CUDA context (as Accelerate's PTX backend does) and checks that the entry point
uses the array of whichever context is current.  This file is collected last
on purpose.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = {0: 4e-6, 1: 1e-12}  # by dtype: C32, C64


def _rel(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _fp64(mode, x):
    from gbfft import _lib as L
    x = x.astype(np.complex128)
    n = x.shape[-1]
    if mode == L.FORWARD:
        return np.fft.fft(x, axis=-1)
    y = np.fft.ifft(x, axis=-1)
    return y if mode == L.INVERSE else y * n


def _data(rng, batch, n, dtype):
    z = rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))
    return z.astype(np.complex64 if dtype == 0 else np.complex128)


def test_noalloc_matches_planned_entry_point_and_fp64(gbfft_lib):
    from gbfft import _lib as L
    lib = L.lib()
    rng = np.random.default_rng(77)
    # consecutive calls with changing length / type / mode: each one rewrites
    # or reuses the tables held in the shared array
    cases = [(5003, 3, L.FORWARD, L.C32), (1009, 4, L.INVERSE, L.C32), (5003, 3, L.REVERSE, L.C32),
             (1024, 1, L.FORWARD, L.C32), (777, 2, L.INVERSE, L.C64), (777, 5, L.FORWARD, L.C64),
             (1009, 4, L.FORWARD, L.C32)]
    for n, batch, mode, dt in cases:
        xh = _data(rng, batch, n, dt)
        x = torch.from_numpy(xh).cuda()
        y_na = torch.empty_like(x)
        y_ref = torch.empty_like(x)
        st = lib.gbfft_fft_noalloc(mode, n, batch, dt, ctypes.c_void_p(x.data_ptr()),
                                   ctypes.c_void_p(y_na.data_ptr()), None)
        assert st == L.OK, L.error_string(st)
        dims = (ctypes.c_int64 * 2)(batch, n)
        st = lib.gbfft_fft(mode, 2, dims, L.KIND_MANY, dt, ctypes.c_void_p(x.data_ptr()),
                           ctypes.c_void_p(y_ref.data_ptr()), None)
        assert st == L.OK
        torch.cuda.synchronize()
        got = y_na.cpu().numpy()
        assert np.array_equal(x.cpu().numpy(), xh), "input modified"
        e_planned = _rel(got, y_ref.cpu().numpy())
        e_fp64 = _rel(got, _fp64(mode, xh))
        assert e_planned < TOL[dt], (n, batch, mode, dt, e_planned)
        assert e_fp64 < TOL[dt], (n, batch, mode, dt, e_fp64)


class _Driver:
    """The few CUDA driver calls the second-context test needs (ctypes)."""

    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")

    def ok(self, rc, what):
        assert rc == 0, "%s failed: CUresult %d" % (what, rc)

    def create_context(self, ordinal):
        cu = self.cu
        self.ok(cu.cuInit(0), "cuInit")
        dev = ctypes.c_int()
        self.ok(cu.cuDeviceGet(ctypes.byref(dev), ordinal), "cuDeviceGet")
        ctx = ctypes.c_void_p()
        if hasattr(cu, "cuCtxCreate_v2"):
            rc = cu.cuCtxCreate_v2(ctypes.byref(ctx), ctypes.c_uint(0), dev)
        else:
            rc = cu.cuCtxCreate_v4(ctypes.byref(ctx), None, ctypes.c_uint(0), dev)
        self.ok(rc, "cuCtxCreate")  # the new context is now current on this thread
        return ctx

    def alloc(self, nbytes):
        p = ctypes.c_uint64()
        self.ok(self.cu.cuMemAlloc_v2(ctypes.byref(p), ctypes.c_size_t(nbytes)), "cuMemAlloc")
        return p.value

    def free(self, p):
        self.ok(self.cu.cuMemFree_v2(ctypes.c_uint64(p)), "cuMemFree")

    def h2d(self, dst, arr):
        self.ok(self.cu.cuMemcpyHtoD_v2(ctypes.c_uint64(dst), arr.ctypes.data_as(ctypes.c_void_p),
                                        ctypes.c_size_t(arr.nbytes)), "cuMemcpyHtoD")

    def d2h(self, arr, src):
        self.ok(self.cu.cuMemcpyDtoH_v2(arr.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint64(src),
                                        ctypes.c_size_t(arr.nbytes)), "cuMemcpyDtoH")

    def sync(self):
        self.ok(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")

    def pop_and_destroy(self, ctx):
        old = ctypes.c_void_p()
        self.ok(self.cu.cuCtxPopCurrent_v2(ctypes.byref(old)), "cuCtxPopCurrent")
        self.ok(self.cu.cuCtxDestroy_v2(ctx), "cuCtxDestroy")


def test_noalloc_in_a_second_context(gbfft_lib):
    from gbfft import _lib as L
    lib = L.lib()
    rng = np.random.default_rng(78)
    n, batch = 1009, 3
    xh = _data(rng, batch, n, L.C32)
    want = _fp64(L.FORWARD, xh)

    # the primary context (torch's) first, so its array holds these tables
    x = torch.from_numpy(xh).cuda()
    y = torch.empty_like(x)
    st = lib.gbfft_fft_noalloc(L.FORWARD, n, batch, L.C32, ctypes.c_void_p(x.data_ptr()),
                               ctypes.c_void_p(y.data_ptr()), None)
    assert st == L.OK, L.error_string(st)
    torch.cuda.synchronize()
    assert _rel(y.cpu().numpy(), want) < TOL[L.C32]

    # a context of the caller's own on the same device: its own copy of the
    # array, set up and filled on this first call there
    drv = _Driver()
    ctx = drv.create_context(torch.cuda.current_device())
    try:
        din = drv.alloc(xh.nbytes)
        dout = drv.alloc(xh.nbytes)
        drv.h2d(din, xh)
        for mode in (L.FORWARD, L.INVERSE):
            st = lib.gbfft_fft_noalloc(mode, n, batch, L.C32, ctypes.c_void_p(din), ctypes.c_void_p(dout),
                                       None)
            assert st == L.OK, L.error_string(st)
            drv.sync()
            got = np.empty_like(xh)
            drv.d2h(got, dout)
            assert _rel(got, _fp64(mode, xh)) < TOL[L.C32], mode
        drv.free(din)
        drv.free(dout)
    finally:
        drv.pop_and_destroy(ctx)

    # back in the primary context: another length, then the first one again
    for nn in (333, n):
        xx = _data(rng, batch, nn, L.C32)
        xt = torch.from_numpy(xx).cuda()
        yt = torch.empty_like(xt)
        st = lib.gbfft_fft_noalloc(L.REVERSE, nn, batch, L.C32, ctypes.c_void_p(xt.data_ptr()),
                                   ctypes.c_void_p(yt.data_ptr()), None)
        assert st == L.OK, L.error_string(st)
        torch.cuda.synchronize()
        assert _rel(yt.cpu().numpy(), _fp64(L.REVERSE, xx)) < TOL[L.C32], nn


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
    # Complex Double doubles the work: 400 rows of 5003 (m = 10125 or more) no longer fit
    st = lib.gbfft_fft_noalloc(L.FORWARD, 5003, 400, L.C64, ctypes.c_void_p(x.data_ptr()),
                               ctypes.c_void_p(y.data_ptr()), None)
    assert st == L.ERR_TOO_LARGE
