"""GPU tests of the naive DFT with caller-supplied roots (Math.DFT: dft, idft,
dftG, dftGS; DFT.hs:37-111) against the oracle's restatement, which keeps the
reference's summation over every element for rank > 1 (each output row holds
the transform of the rows' sum), and against an FP64 FFT for vectors."""
import numpy as np
import pytest
import torch

from oracle import lib as O
from util import rel_l2, uniform_complex

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,tol", [(np.complex64, 3e-5), (np.complex128, 1e-12)])
def test_dft_vectors(gbfft_lib, dtype, tol):
    g = gbfft_lib
    rng = np.random.default_rng(50)
    tdt = torch.complex64 if dtype == np.complex64 else torch.complex128
    for n in list(range(1, 40)) + [97, 256, 1000, 1009]:
        x = uniform_complex(rng, (n,), dtype)
        xt = torch.from_numpy(x).cuda()
        y = g.dft(xt).cpu().numpy()
        assert rel_l2(y, np.fft.fft(x.astype(np.complex128))) < tol, n
        z = g.idft(xt).cpu().numpy()
        assert rel_l2(z, np.fft.ifft(x.astype(np.complex128))) < tol, n
        # same roots as the oracle's restatement of rootsOfUnity
        r = O.roots_of_unity((n,), dtype=dtype)
        assert np.allclose(g.roots_of_unity((n,), dtype=tdt).cpu().numpy(), r, atol=4 * np.finfo(dtype).eps)


@pytest.mark.parametrize("shape", [(3, 64), (2, 3, 40), (5, 7), (2, 2, 2, 2, 12)])
@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_dftG_all_rows_as_the_reference(gbfft_lib, shape, dtype):
    g = gbfft_lib
    rng = np.random.default_rng(51)
    x = uniform_complex(rng, shape, dtype)
    # roots that differ from row to row, to see each row weighted by its own
    roots = uniform_complex(rng, shape, dtype)
    ref64 = O.dftG(roots.astype(np.complex128), x.astype(np.complex128))
    y = g.dftG(torch.from_numpy(roots).cuda(), torch.from_numpy(x).cuda()).cpu().numpy()
    tol = 3e-5 if dtype == np.complex64 else 1e-12
    assert rel_l2(y, ref64) < tol
    rows = y.reshape(-1, shape[-1])
    assert np.array_equal(rows, np.broadcast_to(rows[0], rows.shape))  # every row the same, as written
    for k in (0, 1, shape[-1] - 1, 2 * shape[-1] + 3):
        v = g.dftGS(k, torch.from_numpy(roots).cuda(), torch.from_numpy(x).cuda()).item()
        r = O.dftGS(k, roots, x)
        assert abs(v - r) <= tol * max(1.0, abs(r)) * 10, (k, v, r)


def test_dft_empty_and_errors(gbfft_lib):
    g = gbfft_lib
    from gbfft import _lib as L
    e = torch.zeros((0, 5), dtype=torch.complex64, device="cuda")
    assert g.dftG(e, e).shape == (0, 5)
    v = g.dftGS(2, e, e)
    assert v.item() == 0
    with pytest.raises(ValueError):
        g.dftG(torch.zeros(4, dtype=torch.complex64, device="cuda"),
               torch.zeros(5, dtype=torch.complex64, device="cuda"))
    import ctypes
    dims = (ctypes.c_int64 * 1)(4)
    assert L.lib().gbfft_dftG(1, dims, 7, None, None, None, None) == L.ERR_INVALID_ARG
