"""GPU tests of the spectral convolution and its hand-written adjoint:
forward and gradients against compositions of the oracle's own fft3D (the
reference-composed gradient), against torch autograd through an FP64 FFT,
and against FP64 central finite differences on a 32^3 sub-problem.

Tolerances: complex64 forward / adjoint vs FP64 compositions 2e-6 relative
L2; finite differences 1e-5 relative (the bar of the specification)."""
import numpy as np
import pytest
import torch

from oracle import lib as O
from util import rel_l2

pytestmark = pytest.mark.gpu


def fields(rng, shape, dtype):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(dtype)


def oracle_forward(x, H):
    # y_b = fft3D Inverse (fft3D Forward x_b * H), composed from the oracle's fft3D
    return np.stack([O.fft3D(2, O.fft3D(0, xb) * H) for xb in x])


def oracle_adjoint(x, H, gy):
    N = x[0].size
    gY = np.stack([O.fft3D(0, g) / N for g in gy])
    X = np.stack([O.fft3D(0, xb) for xb in x])
    gH = np.sum(np.conj(X) * gY, axis=0)
    gx = np.stack([O.fft3D(1, np.conj(H) * g) for g in gY])  # Reverse = unnormalised inverse
    return gx, gH


@pytest.mark.parametrize("shape,plane", [((2, 16, 32, 64), ""), ((3, 8, 8, 8), ""), ((1, 32, 32, 32), ""),
                                         ((2, 3, 256, 256), ""), ((2, 3, 256, 256), "plane")])
@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_forward_and_adjoint_vs_oracle(gbfft_lib, shape, plane, dtype, monkeypatch):
    # plane: 256 x 256 planes as one cluster pass each (GBFFT_ENABLE=plane)
    monkeypatch.setenv("GBFFT_ENABLE", plane)
    g = gbfft_lib
    rng = np.random.default_rng(sum(shape))
    x = fields(rng, shape, np.complex128)
    H = fields(rng, shape[1:], np.complex128) / np.sqrt(2)
    gy = fields(rng, shape, np.complex128)
    tdt = torch.complex64 if dtype == np.complex64 else torch.complex128
    plan = g.SpecConvPlan(*shape, dtype=tdt)
    xt = torch.from_numpy(x.astype(dtype)).cuda()
    Ht = torch.from_numpy(H.astype(dtype)).cuda()
    gyt = torch.from_numpy(gy.astype(dtype)).cuda()
    y = plan.forward(xt, Ht).cpu().numpy()
    gx, gH = plan.backward(xt, Ht, gyt)
    tol = 2e-6 if dtype == np.complex64 else 1e-12
    assert rel_l2(y, oracle_forward(x, H)) < tol
    rgx, rgH = oracle_adjoint(x, H, gy)
    assert rel_l2(gx.cpu().numpy(), rgx) < tol
    assert rel_l2(gH.cpu().numpy(), rgH) < tol


def test_autograd_function_matches_torch_fp64(gbfft_lib):
    from gbfft.autograd import spectral_conv3d
    rng = np.random.default_rng(3)
    shape = (2, 16, 16, 32)
    x = torch.from_numpy(fields(rng, shape, np.complex64)).cuda().requires_grad_()
    H = torch.from_numpy(fields(rng, shape[1:], np.complex64)).cuda().requires_grad_()
    y = spectral_conv3d(x, H)
    loss = 0.5 * (y.abs() ** 2).sum()
    loss.backward()
    x64 = x.detach().to(torch.complex128).requires_grad_()
    H64 = H.detach().to(torch.complex128).requires_grad_()
    y64 = torch.fft.ifftn(torch.fft.fftn(x64, dim=(1, 2, 3)) * H64, dim=(1, 2, 3))
    (0.5 * (y64.abs() ** 2).sum()).backward()
    assert rel_l2(y.detach().cpu().numpy(), y64.detach().cpu().numpy()) < 2e-6
    assert rel_l2(x.grad.cpu().numpy(), x64.grad.cpu().numpy()) < 2e-6
    assert rel_l2(H.grad.cpu().numpy(), H64.grad.cpu().numpy()) < 2e-6


def test_adjoint_vs_fp64_finite_differences_32cubed(gbfft_lib):
    g = gbfft_lib
    rng = np.random.default_rng(32)
    shape = (2, 32, 32, 32)
    x = fields(rng, shape, np.complex128)
    H = fields(rng, shape[1:], np.complex128) / np.sqrt(2)
    p64 = g.SpecConvPlan(*shape, dtype=torch.complex128)
    p32 = g.SpecConvPlan(*shape, dtype=torch.complex64)

    def loss64(xa, Ha):
        y = p64.forward(torch.from_numpy(xa).cuda(), torch.from_numpy(Ha).cuda())
        return 0.5 * float((y.abs() ** 2).sum())

    xt = torch.from_numpy(x.astype(np.complex64)).cuda()
    Ht = torch.from_numpy(H.astype(np.complex64)).cuda()
    y = p32.forward(xt, Ht)
    gx, gH = p32.backward(xt, Ht, y)  # L = 1/2 ||y||^2  =>  g_y = y
    gx = gx.cpu().numpy().astype(np.complex128)
    gH = gH.cpu().numpy().astype(np.complex128)
    eps = 1e-6
    for k in range(4):
        v = fields(rng, shape, np.complex128)
        u = fields(rng, shape[1:], np.complex128)
        fd = (loss64(x + eps * v, H + eps * u) - loss64(x - eps * v, H - eps * u)) / (2 * eps)
        an = float(np.real(np.vdot(gx, v)) + np.real(np.vdot(gH, u)))
        assert abs(fd - an) / abs(fd) < 1e-5, (k, fd, an)


def test_config5_full_size_properties(gbfft_lib):
    # 8 fields of 256^3 and a 256^3 filter: H = 1 is the identity, and the
    # adjoint identity <A x, gy> = <x, A^H gy> holds at full size
    g = gbfft_lib
    shape = (8, 256, 256, 256)
    gen = torch.Generator(device="cuda").manual_seed(5)
    x = torch.complex(torch.randn(shape, device="cuda", generator=gen),
                      torch.randn(shape, device="cuda", generator=gen))
    plan = g.SpecConvPlan(*shape)
    ones = torch.ones(shape[1:], dtype=torch.complex64, device="cuda")
    y = plan.forward(x, ones)
    assert float(torch.linalg.vector_norm(y - x) / torch.linalg.vector_norm(x)) < 2e-6
    H = torch.complex(torch.randn(shape[1:], device="cuda", generator=gen),
                      torch.randn(shape[1:], device="cuda", generator=gen)) / np.sqrt(2)
    gy = torch.complex(torch.randn(shape, device="cuda", generator=gen),
                       torch.randn(shape, device="cuda", generator=gen))
    y = plan.forward(x, H)
    gx, gH = plan.backward(x, H, gy)
    lhs = torch.vdot(y.flatten().to(torch.complex128), gy.flatten().to(torch.complex128))
    rhs = torch.vdot(x.flatten().to(torch.complex128), gx.flatten().to(torch.complex128))
    assert abs(complex(lhs - rhs)) / abs(complex(lhs)) < 1e-5
