"""GPU tests of the naive DFT with caller-supplied roots (Math.DFT: dft, idft,
dftG, dftGS; DFT.hs:37-111) against the oracle's restatement, which keeps the
reference's summation over every element for rank > 1 (each output row holds
the transform of the rows' sum), and against an FP64 FFT for vectors."""
import numpy as np
import pytest
import torch

from oracle import lib as O
from util import np_reference, rel_l2, uniform_complex

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


@pytest.mark.parametrize("shape", [(8,), (7,), (4, 6), (5, 3), (2, 4, 6), (3, 5, 7), (64, 63)])
@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_centre_and_shift(gbfft_lib, shape, dtype):
    g = gbfft_lib
    rng = np.random.default_rng(61)
    x = uniform_complex(rng, shape, dtype)
    xt = torch.from_numpy(x).cuda()
    assert np.array_equal(g.centre(xt).cpu().numpy(), O.centre(x))
    assert np.array_equal(g.shift(xt).cpu().numpy(), O.shift(x))
    assert np.array_equal(g.shift(xt, inverse=True).cpu().numpy(), O.shift(x, inverse=True))


# shapes that route each axis through every kind of final pass: register
# rows (1024, 1000), one-pass and multi-pass Bluestein (1009, 65521), row
# four-step (65536), strided/pencil columns (64x63, 3-D), the clustered
# 4096 column kernel (4096x4096), and a strided four-step axis (8192x8),
# whose last pass cannot rotate and takes the one-pass fallback
FUSED_SHAPES = [(1024,), (1000,), (1009,), (65536,), (65521,), (64, 63), (8192, 8), (6, 10, 12),
                (4096, 4096), (128, 128, 128)]


@pytest.mark.parametrize("shape", FUSED_SHAPES)
@pytest.mark.parametrize("mode", ["forward", "inverse", "reverse"])
def test_fused_shift_centre(gbfft_lib, shape, mode):
    """gbfft_exec_ex: a transform with shiftND / ishiftND of the result and
    centreND of the input (Centre.hs:36-164).  The output rotation only moves
    stores, so shift / ishift are bit-identical to shifting the plain result;
    centring an even-length input is the output rotated by n/2 (shift
    theorem), compared against a transform of the centred input."""
    g = gbfft_lib
    rng = np.random.default_rng(70)
    dtype = np.complex64
    x = uniform_complex(rng, shape, dtype)
    xt = torch.from_numpy(x).cuda()
    plan = g.Plan(shape, kind="full", dtype=torch.complex64)
    y = plan(mode, xt).cpu().numpy()
    assert np.array_equal(plan(mode, xt, shift_out="shift").cpu().numpy(), O.shift(y)), "shift"
    assert np.array_equal(plan(mode, xt, shift_out="ishift").cpu().numpy(), O.shift(y, inverse=True)), "ishift"
    yc = plan(mode, xt, centre_in=True).cpu().numpy()
    ref = np_reference("fft2D", mode, O.centre(x))
    assert rel_l2(yc, ref) < 2e-6 * max(1.0, np.log2(x.size)), "centre"
    ycs = plan(mode, xt, centre_in=True, shift_out="shift").cpu().numpy()
    assert np.array_equal(ycs, O.shift(yc)), "centre+shift"
    plan.close()


@pytest.mark.parametrize("colv", ["9", "16", "17", "18", "19"])
def test_fused_shift_cluster_column_variants(gbfft_lib, monkeypatch, colv):
    """The 4096-point cluster column kernels store the rotated output on their
    own store path (scaled and conjugated for Inverse / Reverse): shift and
    ishift stay bit-identical to shifting the plain result."""
    g = gbfft_lib
    monkeypatch.setenv("GBFFT_COL_VARIANT", colv)
    rng = np.random.default_rng(72)
    x = uniform_complex(rng, (4096, 4096), np.complex64)
    xt = torch.from_numpy(x).cuda()
    plan = g.Plan((4096, 4096), kind="full", dtype=torch.complex64)
    for mode in ("forward", "inverse", "reverse"):
        y = plan(mode, xt).cpu().numpy()
        assert rel_l2(y, np_reference("fft2D", mode, x)) < 2e-6 * np.log2(x.size), (colv, mode)
        assert np.array_equal(plan(mode, xt, shift_out="shift").cpu().numpy(), O.shift(y)), (colv, mode)
        assert np.array_equal(plan(mode, xt, shift_out="ishift").cpu().numpy(), O.shift(y, inverse=True)), \
            (colv, mode)
    plan.close()


@pytest.mark.parametrize("shape", [(7,), (5, 3), (3, 5, 7), (12, 9)])
def test_fused_centre_odd_and_double(gbfft_lib, shape):
    """Odd extents: centring is not a rotation; the input pass runs first and
    the result equals the plain transform of the centred input bit for bit."""
    g = gbfft_lib
    rng = np.random.default_rng(71)
    for dtype, tdt in ((np.complex64, torch.complex64), (np.complex128, torch.complex128)):
        x = uniform_complex(rng, shape, dtype)
        xt = torch.from_numpy(x).cuda()
        plan = g.Plan(shape, kind="full", dtype=tdt)
        want = plan("forward", g.centre(xt)).cpu().numpy()
        assert np.array_equal(plan("forward", xt, centre_in=True).cpu().numpy(), want)
        want_s = O.shift(plan("inverse", xt).cpu().numpy())
        assert np.array_equal(plan("inverse", xt, shift_out="shift").cpu().numpy(), want_s)
        plan.close()


def test_fused_shift_split_fp16_and_errors(gbfft_lib):
    """Split-FP16 plans mark no rotatable pass: the shift runs as one pass
    after the transform.  MANY plans, rank > 3 and shift together with
    ishift are refused."""
    g = gbfft_lib
    from gbfft import _lib as L
    import ctypes
    rng = np.random.default_rng(72)
    x = uniform_complex(rng, (3, 256, 256), np.complex64)
    xt = torch.from_numpy(x).cuda()
    plan = g.Plan((3, 256, 256), kind="full", dtype=torch.complex64, precision="split_fp16")
    assert np.array_equal(plan("forward", xt, shift_out="shift").cpu().numpy(), O.shift(plan("forward", xt).cpu().numpy()))
    plan.close()
    many = g.Plan((4, 64), kind="many", dtype=torch.complex64)
    e = torch.zeros((4, 64), dtype=torch.complex64, device="cuda")
    o = torch.empty_like(e)
    rc = L.lib().gbfft_exec_ex(many.handle, L.FORWARD, ctypes.c_void_p(e.data_ptr()), ctypes.c_void_p(o.data_ptr()),
                               None, L.OPT_SHIFT_OUT)
    assert rc == L.ERR_INVALID_ARG
    many.close()
    full = g.Plan((4, 64), kind="full", dtype=torch.complex64)
    rc = L.lib().gbfft_exec_ex(full.handle, L.FORWARD, ctypes.c_void_p(e.data_ptr()), ctypes.c_void_p(o.data_ptr()),
                               None, L.OPT_SHIFT_OUT | L.OPT_ISHIFT_OUT)
    assert rc == L.ERR_INVALID_ARG
    rc = L.lib().gbfft_exec_ex(full.handle, L.FORWARD, ctypes.c_void_p(e.data_ptr()), ctypes.c_void_p(o.data_ptr()),
                               None, 64)
    assert rc == L.ERR_INVALID_ARG
    full.close()
