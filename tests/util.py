"""Shared helpers for the test suite: seeded inputs shaped like the
reference's generators (test/Test/Base.hs:35-61) and error metrics."""
import numpy as np


def uniform_complex(rng, shape, dtype=np.complex128):
    """Components i.i.d. uniform on [-1, 1] (test/Test/Base.hs:35-39)."""
    x = rng.uniform(-1.0, 1.0, shape) + 1j * rng.uniform(-1.0, 1.0, shape)
    return x.astype(dtype)


def normal_complex(rng, shape, dtype=np.complex64):
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    return x.astype(dtype)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    nb = np.linalg.norm(b)
    if nb == 0:
        return float(np.linalg.norm(a))
    return float(np.linalg.norm(a - b) / nb)


def np_reference(kind, mode, x):
    """Independent FP64 FFT (numpy's pocketfft) with the reference's mode
    conventions (Mode.hs:21-26, FFT.hs normalisation)."""
    x = np.asarray(x, dtype=np.complex128)
    mode = {"forward": 0, "reverse": 1, "inverse": 2}.get(str(mode).lower(), mode)
    if kind in ("fft", "fft1D"):
        axes = (-1,)
    else:
        axes = tuple(range(x.ndim))
    if mode == 0:
        return np.fft.fftn(x, axes=axes)
    y = np.fft.ifftn(x, axes=axes)
    if mode == 1:
        y = y * np.prod([x.shape[a] for a in axes])
    return y


# Shape generators mirroring test/Test/Base.hs:44-58.
def dim1(rng):
    return (int(rng.integers(1, 1025)),)


def dim2(rng):
    return (int(rng.integers(1, 49)), int(rng.integers(1, 129)))


def dim3(rng):
    return (int(rng.integers(1, 17)), int(rng.integers(1, 33)), int(rng.integers(1, 65)))
