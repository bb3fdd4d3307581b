"""torch.autograd.Function over the spectral-convolution C ABI, for checking
the hand-written adjoint against autograd and finite differences.

Gradients follow PyTorch's convention for complex tensors (the conjugate
Wirtinger derivative scaled so that for a real loss L and a step dz,
dL = Re(sum(conj(grad) * dz))): grad_x = A^H grad_y for the linear map A.
"""
import torch

from .fft import SpecConvPlan

_plans = {}


def _plan(x):
    key = (tuple(x.shape), x.dtype, x.device.index)
    p = _plans.get(key)
    if p is None:
        p = SpecConvPlan(*x.shape, dtype=x.dtype)
        _plans[key] = p
    return p


class SpectralConv3d(torch.autograd.Function):
    """y_b = fft3D Inverse (fft3D Forward (x_b) * H) for x of shape (B, D, H, W)."""

    @staticmethod
    def forward(ctx, x, H):
        x = x.contiguous()
        H = H.contiguous()
        ctx.save_for_backward(x, H)
        return _plan(x).forward(x, H)

    @staticmethod
    def backward(ctx, gy):
        x, H = ctx.saved_tensors
        gx, gH = _plan(x).backward(x, H, gy.contiguous())
        return gx, gH


def spectral_conv3d(x, H):
    return SpectralConv3d.apply(x, H)
