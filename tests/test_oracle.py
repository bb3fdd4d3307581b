"""CPU tests of the oracle (the C++ restatement of the reference's
pure-Accelerate transform, oracle/adhoc.cpp): against an independent FP64 FFT
(numpy), analytic known answers, and the reference's own seven property tests
(test/Test/FFT.hs:112-236) over its shape generators (test/Test/Base.hs:44-58).
"""
import numpy as np
import pytest

from oracle import lib as O
from util import dim1, dim2, dim3, np_reference, rel_l2, uniform_complex

TOL = {np.complex64: 5e-4, np.complex128: 1e-10}


def smooth5(n):
    while n % 2 == 0:
        n //= 2
    for p in (3, 5):
        while n % p == 0:
            n //= p
    return n == 1


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_fft1d_all_small_lengths_vs_numpy(dtype):
    rng = np.random.default_rng(1)
    for n in list(range(1, 130)) + [243, 256, 500, 625, 1000, 1009, 1024, 2048]:
        x = uniform_complex(rng, (n,), dtype)
        for mode in (0, 1, 2):
            y = O.fft1D(mode, x)
            err = rel_l2(y, np_reference("fft1D", mode, x))
            # the Float Bluestein forms pi*k^2/n in single precision (Adhoc.hs:264-265)
            tol = 1e-12 if dtype == np.complex128 else (5e-6 if smooth5(n) else 5e-4)
            assert err < tol, (n, mode, err)


def test_fp64_error_of_float_paths_is_as_expected():
    # split radix / dit235 in Float are accurate; Bluestein in Float is not
    rng = np.random.default_rng(2)
    x = uniform_complex(rng, (1009,), np.complex64)
    err = rel_l2(O.fft1D(0, x), np.fft.fft(x.astype(np.complex128)))
    assert 1e-6 < err < 1e-3
    x = uniform_complex(rng, (1000,), np.complex64)
    assert rel_l2(O.fft1D(0, x), np.fft.fft(x.astype(np.complex128))) < 2e-6


def test_known_answers():
    for n in (1, 2, 3, 5, 7, 8, 12, 97, 1000, 1024):
        d = np.zeros(n, np.complex128)
        d[0] = 1
        assert np.allclose(O.fft1D(0, d), np.ones(n), atol=1e-12)
        one = np.ones(n, np.complex128)
        ref = np.zeros(n, np.complex128)
        ref[0] = n
        assert np.allclose(O.fft1D(0, one), ref, atol=1e-9 * n)
        k0 = min(3, n - 1)
        e = np.exp(2j * np.pi * k0 * np.arange(n) / n)
        ref = np.zeros(n, np.complex128)
        ref[k0] = n
        assert np.allclose(O.fft1D(0, e), ref, atol=1e-9 * n)


def test_naive_dft_matches_numpy():
    rng = np.random.default_rng(3)
    for n in (1, 2, 7, 64, 100, 257):
        x = uniform_complex(rng, (5, n))
        assert rel_l2(O.dft_naive(-1, x), np.fft.fft(x, axis=-1)) < 1e-13
        assert rel_l2(O.dft_naive(1, x), np.fft.ifft(x, axis=-1) * n) < 1e-13


def test_ceiling5_smooth_padded_length():
    # the intended 2^i2 * 3^i3 * 5^i5 (Adhoc.hs:289-313) for the Bluestein sizes used
    assert O.ceiling5_smooth(2 * 1009) == 2025
    for n in range(7, 4000, 13):
        p = O.ceiling5_smooth(2 * n)
        assert p >= 2 * n and smooth5(p)
        exact = next(m for m in range(2 * n, 4 * n + 2) if smooth5(m))
        # the reference's grid stops below ceiling(logBase 5 n) and
        # ceiling(logBase 3 n), so a pure power of 3 or 5 can be skipped
        # (2n = 612: 640, not 625); it never exceeds twice the minimum
        assert exact <= p < 2 * exact, (n, p, exact)


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_rank_2_3_and_innermost_vs_numpy(dtype):
    rng = np.random.default_rng(4)
    tol = 1e-11 if dtype == np.complex128 else 5e-4
    for _ in range(6):
        for gen, kind in ((dim2, "fft2D"), (dim3, "fft3D")):
            sh = gen(rng)
            x = uniform_complex(rng, sh, dtype)
            for mode in (0, 1, 2):
                assert rel_l2(O.run(kind, mode, x), np_reference(kind, mode, x)) < tol
                assert rel_l2(O.fft(mode, x), np_reference("fft", mode, x)) < tol


# ---- the reference's property suite, test/Test/FFT.hs:112-236 ---------------
def _transform(kind):
    return {"fft1D": O.fft1D, "fft2D": O.fft2D, "fft3D": O.fft3D, "fft": O.fft}[kind]


def _reverse(x):
    # k -> (-k) mod n on the innermost axis (test/Test/FFT.hs:86-94)
    n = x.shape[-1]
    return x[..., (-np.arange(n)) % n]


CASES = [("DIM1", dim1, "fft1D", "fft1D"), ("DIM2", dim2, "fft2D", "fft"), ("DIM3", dim3, "fft3D", "fft")]


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
@pytest.mark.parametrize("dim,gen,full,inner", CASES)
def test_reference_properties(dtype, dim, gen, full, inner):
    rng = np.random.default_rng(hash((dim, str(dtype))) % 2**32)
    tol = TOL[dtype]
    F, G = _transform(full), _transform(inner)
    for _ in range(4):
        sh = gen(rng)
        mode = int(rng.integers(0, 3))
        x = uniform_complex(rng, sh, dtype)
        y = uniform_complex(rng, sh, dtype)
        a = uniform_complex(rng, (), dtype)
        # homogeneity / additivity / inverse use the full transform
        assert rel_l2(F(mode, (a * x).astype(dtype)), a * F(mode, x)) < tol
        assert rel_l2(F(mode, (x + y).astype(dtype)), F(mode, x) + F(mode, y)) < tol
        assert rel_l2(F(2, F(0, x)), x) < tol
        # reverse / conjugate / isometry / unitarity use the innermost transform
        assert rel_l2(_reverse(G(mode, x)), G(mode, _reverse(x))) < tol
        assert rel_l2(np.conj(G(mode, x)), G(mode, np.conj(_reverse(x)).astype(dtype))) < tol
        m2 = int(rng.integers(0, 2))  # Forward or Reverse
        n = sh[-1]
        fx, fy = G(m2, x), G(m2, y)
        nx = np.linalg.norm(fx.astype(np.complex128), axis=-1)
        assert rel_l2(nx, np.sqrt(n) * np.linalg.norm(x.astype(np.complex128), axis=-1)) < tol
        d1 = np.sum(fx.astype(np.complex128) * np.conj(fy), axis=-1)
        d2 = n * np.sum(x.astype(np.complex128) * np.conj(y), axis=-1)
        assert rel_l2(d1, d2) < 10 * tol


def test_centre_and_shift_restatement():
    """Centre.hs restated: shift then ishift is the identity, and for even
    lengths centring before a DFT equals shifting after it."""
    import numpy as np
    from oracle import lib as O
    rng = np.random.default_rng(60)
    for shape in [(8,), (7,), (4, 6), (5, 3), (2, 4, 6), (3, 5, 7)]:
        x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        assert np.array_equal(O.shift(O.shift(x), inverse=True), x)
        if all(n % 2 == 0 for n in shape):
            assert np.allclose(np.fft.fftn(O.centre(x)), O.shift(np.fft.fftn(x)), atol=1e-9)
    assert np.array_equal(O.centre(np.ones(5)), np.array([1, -1, 1, -1, 1.0]))
    assert np.array_equal(O.shift(np.arange(5)), np.array([3, 4, 0, 1, 2]))
    assert np.array_equal(O.shift(np.arange(5), inverse=True), np.array([2, 3, 4, 0, 1]))
