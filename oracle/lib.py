"""ctypes front end of the oracle library (see adhoc.cpp).

Functions mirror accelerate-fft's API: ``fft`` (innermost axis, FFT.hs:63-84),
``fft1D`` / ``fft2D`` / ``fft3D`` (FFT.hs:92-173) with Mode Forward / Reverse /
Inverse, in the precision of the input (complex64 -> Float, complex128 ->
Double); plus ``dft_naive`` (an FP64 per-row DFT), ``dftG`` / ``dftGS`` and
``roots_of_unity`` as the reference writes them (DFT.hs:68-111, Roots.hs:26-51),
``centre`` / ``shift`` (Centre.hs:36-164) and ``ceiling5_smooth``
(Adhoc.hs:289-313).
"""
import ctypes
import os

import numpy as np

from . import build as _build

FORWARD, REVERSE, INVERSE = 0, 1, 2
_KIND = {"fft": 0, "fft1D": 1, "fft2D": 2, "fft3D": 3}
_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = ctypes.CDLL(path)
        i64p = ctypes.POINTER(ctypes.c_int64)
        for name in ("oracle_fft_f32", "oracle_fft_f64"):
            f = getattr(_lib, name)
            f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, i64p, ctypes.c_void_p,
                          ctypes.c_void_p, ctypes.c_int]
            f.restype = ctypes.c_int
        _lib.oracle_dft_naive_f64.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int64,
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        _lib.oracle_dft_naive_f64.restype = ctypes.c_int
        _lib.oracle_ceiling5_smooth.argtypes = [ctypes.c_int64]
        _lib.oracle_ceiling5_smooth.restype = ctypes.c_int64
        for name in ("oracle_dftg_f32", "oracle_dftg_f64"):
            f = getattr(_lib, name)
            f.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                          ctypes.c_int]
            f.restype = ctypes.c_int
        _lib.oracle_dftgs_f64.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p]
        _lib.oracle_dftgs_f64.restype = ctypes.c_int
    return _lib


def _mode_index(mode):
    if isinstance(mode, str):
        return {"forward": 0, "reverse": 1, "inverse": 2}[mode.lower()]
    return int(mode)


def run(kind, mode, x, threads=None):
    x = np.ascontiguousarray(x)
    if x.dtype == np.complex64:
        f = lib().oracle_fft_f32
    elif x.dtype == np.complex128:
        f = lib().oracle_fft_f64
    else:
        raise TypeError("oracle: complex64 or complex128 input required")
    if threads is None:
        threads = os.cpu_count() or 1
    out = np.empty_like(x)
    dims = (ctypes.c_int64 * x.ndim)(*x.shape)
    st = f(_mode_index(mode), _KIND[kind], x.ndim, dims, x.ctypes.data, out.ctypes.data, int(threads))
    if st != 0:
        raise ValueError("oracle: bad arguments for %s on shape %s" % (kind, x.shape))
    return out


def fft(mode, x, threads=None):
    return run("fft", mode, x, threads)


def fft1D(mode, x, threads=None):
    return run("fft1D", mode, x, threads)


def fft2D(mode, x, threads=None):
    return run("fft2D", mode, x, threads)


def fft3D(mode, x, threads=None):
    return run("fft3D", mode, x, threads)


def dft_naive(sign, x, threads=None):
    """O(n^2) FP64 DFT along the innermost axis; sign -1 forward, +1 inverse roots (unnormalised)."""
    x = np.ascontiguousarray(x, dtype=np.complex128)
    n = x.shape[-1]
    rows = x.size // max(n, 1)
    out = np.empty_like(x)
    if threads is None:
        threads = os.cpu_count() or 1
    st = lib().oracle_dft_naive_f64(int(sign), rows, n, x.ctypes.data, out.ctypes.data, int(threads))
    if st != 0:
        raise ValueError("oracle: bad arguments for dft_naive")
    return out


def roots_of_unity(shape, inverse=False, dtype=np.complex128):
    """rootsOfUnity / inverseRootsOfUnity (Roots.hs:26-51): element
    (sh :. i) = cos t :+ (-+ sin t), t = 2*pi*i/n, in the element precision."""
    n = shape[-1]
    real = np.float32 if dtype == np.complex64 else np.float64
    t = (real(2) * real(np.pi) * np.arange(n, dtype=real)) / real(n)
    r = (np.cos(t) + (1j if inverse else -1j) * np.sin(t)).astype(dtype)
    return np.ascontiguousarray(np.broadcast_to(r, shape))


def dftG(roots, x, threads=None):
    """dftG as written (DFT.hs:68-92): every output row is the sum over all
    input elements (sh :. n) of x * roots[sh :. (k*n) mod l]."""
    x = np.ascontiguousarray(x)
    roots = np.ascontiguousarray(roots, dtype=x.dtype)
    if roots.shape != x.shape:
        raise ValueError("oracle: roots and input shapes differ")
    f = lib().oracle_dftg_f32 if x.dtype == np.complex64 else lib().oracle_dftg_f64
    l = x.shape[-1]
    rows = x.size // max(l, 1)
    out = np.empty_like(x)
    if threads is None:
        threads = os.cpu_count() or 1
    if f(rows, l, roots.ctypes.data, x.ctypes.data, out.ctypes.data, int(threads)) != 0:
        raise ValueError("oracle: bad arguments for dftG")
    return out


def dftGS(k, roots, x):
    """dftGS (DFT.hs:95-111) in FP64: one bin, summed over every row."""
    x = np.ascontiguousarray(x, dtype=np.complex128)
    roots = np.ascontiguousarray(roots, dtype=np.complex128)
    l = x.shape[-1]
    rows = x.size // max(l, 1)
    out = np.empty(1, np.complex128)
    if lib().oracle_dftgs_f64(int(k), rows, l, roots.ctypes.data, x.ctypes.data, out.ctypes.data) != 0:
        raise ValueError("oracle: bad arguments for dftGS")
    return out[0]


def centre(x):
    """centre1D/2D/3D (Centre.hs:36-67): element ix times (-1) ** (sum of ix)."""
    x = np.asarray(x)
    idx = np.indices(x.shape).sum(axis=0)
    return np.where(idx % 2 == 0, x, -x).astype(x.dtype)


def shift(x, inverse=False):
    """shift1D/2D/3D and ishift1D/2D/3D (Centre.hs:70-164): backpermute with
    index (i + s) mod n per axis, s = n `quot` 2 + (odd n) for shift, n `quot` 2
    for ishift."""
    x = np.asarray(x)
    out = x
    for ax, n in enumerate(x.shape):
        s = n // 2 + (0 if inverse else n % 2)
        out = np.take(out, (np.arange(n) + s) % n, axis=ax)
    return out


def ceiling5_smooth(n):
    return int(lib().oracle_ceiling5_smooth(int(n)))
