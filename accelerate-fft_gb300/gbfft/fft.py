"""The accelerate-fft API over the C ABI.

``fft`` transforms the innermost axis of a rank >= 1 array (FFT.hs:63-84; the
PTX path's "cuda.fft2.many" / "cuda.fft3.many", PTX.hs:52-61); ``fft1D``,
``fft2D``, ``fft3D`` transform every axis (FFT.hs:92-173, PTX.hs:63-70).
Inverse is normalised by the innermost length for ``fft`` and by the array
size for the others, as in FFT.hs:69,98,125,155 -- but inside the kernel, so
no extra elementwise pass runs.  Results are new tensors; inputs are never
modified.
"""
import ctypes
import enum

import torch

from . import _lib as L


class Mode(enum.IntEnum):
    """src/Data/Array/Accelerate/Math/FFT/Mode.hs:15-26."""
    Forward = L.FORWARD
    Reverse = L.REVERSE
    Inverse = L.INVERSE


def mode_code(mode):
    if isinstance(mode, str):
        return int(Mode[mode.capitalize()])
    m = int(mode)
    if m not in (L.FORWARD, L.REVERSE, L.INVERSE):
        raise ValueError("mode must be Forward, Reverse or Inverse")
    return m


def _dtype_code(t):
    if t.dtype == torch.complex64:
        return L.C32
    if t.dtype == torch.complex128:
        return L.C64
    raise TypeError("gbfft: complex64 or complex128 tensor required, got %s" % t.dtype)


def _stream(stream):
    if stream is None:
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, torch.cuda.Stream):
        return ctypes.c_void_p(stream.cuda_stream)
    return ctypes.c_void_p(int(stream))


def _dims(shape):
    return (ctypes.c_int64 * len(shape))(*[int(s) for s in shape])


def autotune(shape, kind="full", dtype=torch.complex64, precision="plain", stream=None):
    """Times the candidate plans of this transform (gbfft_autotune) and caches
    the fastest for later plan creations; returns the per-candidate report."""
    buf = ctypes.create_string_buffer(16384)
    shape = tuple(int(s) for s in shape)
    L.check(L.lib().gbfft_autotune(len(shape), _dims(shape), L.KIND_FULL if kind == "full" else L.KIND_MANY,
                                   L.C64 if dtype == torch.complex128 else L.C32,
                                   L.SPLIT_FP16 if precision == "split_fp16" else L.PLAIN,
                                   _stream(stream), buf, 16384), "gbfft_autotune%s" % (shape,))
    return buf.value.decode()


class Plan:
    """An owned plan (gbfft_plan_create / gbfft_exec / gbfft_plan_destroy)."""

    def __init__(self, shape, kind="full", dtype=torch.complex64, precision="plain"):
        self.shape = tuple(int(s) for s in shape)
        self.kind = L.KIND_FULL if kind == "full" else L.KIND_MANY
        self.dtype = dtype
        self.dtype_code = L.C64 if dtype == torch.complex128 else L.C32
        self.precision = L.SPLIT_FP16 if precision == "split_fp16" else L.PLAIN
        h = ctypes.c_void_p()
        L.check(L.lib().gbfft_plan_create(ctypes.byref(h), len(self.shape), _dims(self.shape),
                                          self.kind, self.dtype_code, self.precision),
                "gbfft_plan_create%s" % (self.shape,))
        self.handle = h

    def exec_ptr(self, mode, in_ptr, out_ptr, stream=None, opts=0):
        if opts:
            L.check(L.lib().gbfft_exec_ex(self.handle, mode_code(mode), ctypes.c_void_p(in_ptr),
                                          ctypes.c_void_p(out_ptr), _stream(stream), int(opts)), "gbfft_exec_ex")
            return
        L.check(L.lib().gbfft_exec(self.handle, mode_code(mode), ctypes.c_void_p(in_ptr),
                                   ctypes.c_void_p(out_ptr), _stream(stream)), "gbfft_exec")

    def __call__(self, mode, x, out=None, stream=None, centre_in=False, shift_out=None):
        """Transform x.  centre_in multiplies the input by (-1)^(sum of
        indices) first; shift_out="shift" / "ishift" rolls the result like
        shiftND / ishiftND (Centre.hs:36-164) -- both fused into the passes
        where the lengths allow (gbfft_exec_ex)."""
        if not x.is_cuda or not x.is_contiguous():
            raise ValueError("gbfft: contiguous CUDA tensor required")
        if tuple(x.shape) != self.shape or x.dtype != self.dtype:
            raise ValueError("gbfft: tensor does not match the plan")
        if out is None:
            out = torch.empty_like(x)
        opts = (L.OPT_CENTRE_IN if centre_in else 0) | {None: 0, "shift": L.OPT_SHIFT_OUT,
                                                       "ishift": L.OPT_ISHIFT_OUT}[shift_out]
        self.exec_ptr(mode, x.data_ptr(), out.data_ptr(), stream, opts)
        return out

    @property
    def info(self):
        ws = ctypes.c_size_t()
        n = ctypes.c_int()
        L.check(L.lib().gbfft_plan_info(self.handle, ctypes.byref(ws), ctypes.byref(n)))
        return {"workspace_bytes": ws.value, "launches": n.value}

    def describe(self):
        buf = ctypes.create_string_buffer(4096)
        L.check(L.lib().gbfft_plan_describe(self.handle, buf, 4096))
        return buf.value.decode()

    def pass_kernels(self):
        """CUDA kernel name of each launch of one exec, in order."""
        out = []
        for i in range(self.info["launches"]):
            buf = ctypes.create_string_buffer(128)
            L.check(L.lib().gbfft_plan_pass_kernel(self.handle, i, buf, 128))
            out.append(buf.value.decode())
        return out

    def close(self):
        if getattr(self, "handle", None):
            L.lib().gbfft_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _run(kind, mode, arr, stream=None):
    if not isinstance(arr, torch.Tensor) or not arr.is_cuda:
        raise TypeError("gbfft: a CUDA tensor is required")
    dt = _dtype_code(arr)
    x = arr.contiguous()
    out = torch.empty_like(x)
    shape = tuple(x.shape)
    if x.numel() == 0:
        return out
    L.check(L.lib().gbfft_fft(mode_code(mode), len(shape), _dims(shape), kind, dt,
                              ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                              _stream(stream)), "gbfft_fft%s" % (shape,))
    return out


def fft(mode, arr, stream=None):
    """DFT along the innermost axis (FFT.hs:63-84); any rank >= 1."""
    if arr.dim() < 1:
        raise ValueError("fft: rank >= 1 required")
    if arr.dim() > 5:
        # rank 6+: the batched-innermost plan over the flattened outer axes
        flat = arr.contiguous().reshape(-1, arr.shape[-1])
        return _run(L.KIND_MANY, mode, flat, stream).reshape(arr.shape)
    return _run(L.KIND_MANY, mode, arr, stream)


def fft1D(mode, arr, stream=None):
    """DFT of a vector (FFT.hs:92-111)."""
    if arr.dim() != 1:
        raise ValueError("fft1D: rank 1 required")
    return _run(L.KIND_FULL, mode, arr, stream)


def fft2D(mode, arr, stream=None):
    """DFT of a matrix (FFT.hs:119-142)."""
    if arr.dim() != 2:
        raise ValueError("fft2D: rank 2 required")
    return _run(L.KIND_FULL, mode, arr, stream)


def fft3D(mode, arr, stream=None):
    """DFT of a 3D array (FFT.hs:150-173)."""
    if arr.dim() != 3:
        raise ValueError("fft3D: rank 3 required")
    return _run(L.KIND_FULL, mode, arr, stream)


def roots_of_unity(shape, inverse=False, dtype=torch.complex64, device="cuda"):
    """rootsOfUnity / inverseRootsOfUnity (Roots.hs:26-51): element (sh :. i)
    = cos t :+ (-+ sin t), t = 2*pi*i/n, computed in the element precision."""
    n = int(shape[-1])
    real = torch.float64 if dtype == torch.complex128 else torch.float32
    t = (2 * torch.tensor(torch.pi, dtype=real) * torch.arange(n, dtype=real)) / n
    r = torch.complex(torch.cos(t), torch.sin(t) if inverse else -torch.sin(t))
    return r.expand(tuple(int(s) for s in shape)).contiguous().to(device)


def dftG(roots, arr, stream=None):
    """Math.DFT.dftG (DFT.hs:68-92) on the GPU, summing over every element as
    the reference does (for rank > 1 every output row holds the same values)."""
    if roots.shape != arr.shape or roots.dtype != arr.dtype:
        raise ValueError("dftG: roots and input must have the same shape and type")
    x = arr.contiguous()
    out = torch.empty_like(x)
    L.check(L.lib().gbfft_dftG(x.dim(), _dims(x.shape), _dtype_code(x), ctypes.c_void_p(roots.contiguous().data_ptr()),
                               ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()), _stream(stream)),
            "gbfft_dftG")
    return out


def dftGS(k, roots, arr, stream=None):
    """Math.DFT.dftGS (DFT.hs:95-111): bin k of dftG, a 0-d tensor."""
    x = arr.contiguous()
    out = torch.empty((), dtype=x.dtype, device=x.device)
    L.check(L.lib().gbfft_dftGS(x.dim(), _dims(x.shape), _dtype_code(x), int(k),
                                ctypes.c_void_p(roots.contiguous().data_ptr()), ctypes.c_void_p(x.data_ptr()),
                                ctypes.c_void_p(out.data_ptr()), _stream(stream)), "gbfft_dftGS")
    return out


def dft(arr, stream=None):
    """Math.DFT.dft (DFT.hs:37-41): dftG with rootsOfUnity."""
    return dftG(roots_of_unity(arr.shape, False, arr.dtype, arr.device), arr, stream)


def idft(arr, stream=None):
    """Math.DFT.idft (DFT.hs:44-53): dftG with inverseRootsOfUnity, then / n."""
    return dftG(roots_of_unity(arr.shape, True, arr.dtype, arr.device), arr, stream) / arr.shape[-1]


def centre(arr, stream=None):
    """Math.DFT.Centre.centre1D/2D/3D (Centre.hs:36-67): (-1)^(sum of indices) * arr."""
    x = arr.contiguous()
    out = torch.empty_like(x)
    L.check(L.lib().gbfft_centre(x.dim(), _dims(x.shape), _dtype_code(x), ctypes.c_void_p(x.data_ptr()),
                                 ctypes.c_void_p(out.data_ptr()), _stream(stream)), "gbfft_centre")
    return out


def shift(arr, inverse=False, stream=None):
    """Math.DFT.Centre.shift1D/2D/3D, or ishift*D with inverse=True
    (Centre.hs:70-164): roll every axis by n/2 (+1 for odd n when shifting)."""
    x = arr.contiguous()
    out = torch.empty_like(x)
    L.check(L.lib().gbfft_shift(x.dim(), _dims(x.shape), _dtype_code(x), 1 if inverse else 0,
                                ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()), _stream(stream)),
            "gbfft_shift")
    return out


def ragged_autotune(lengths, modes, offsets=None, dtype=torch.complex64, stream=None):
    """Times candidate ragged plans for these lengths and modes
    (gbfft_ragged_autotune) and caches the fastest; returns the report."""
    import numpy as np
    lengths = np.ascontiguousarray(np.asarray(lengths, dtype=np.int64))
    modes = np.ascontiguousarray(np.asarray([mode_code(m) for m in modes], dtype=np.int32))
    off = None
    if offsets is not None:
        offsets = np.ascontiguousarray(np.asarray(offsets, dtype=np.int64))
        off = offsets.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    buf = ctypes.create_string_buffer(8192)
    L.check(L.lib().gbfft_ragged_autotune(len(lengths), lengths.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                          off, modes.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                          L.C64 if dtype == torch.complex128 else L.C32, _stream(stream),
                                          buf, 8192), "gbfft_ragged_autotune")
    return buf.value.decode()


class RaggedPlan:
    """Many 1D transforms of uneven lengths and modes over one flat buffer,
    run by one persistent launch (gbfft_ragged_plan_create / _exec)."""

    def __init__(self, lengths, modes, offsets=None, dtype=torch.complex64):
        import numpy as np
        self.lengths = np.ascontiguousarray(np.asarray(lengths, dtype=np.int64))
        self.modes = np.ascontiguousarray(np.asarray([mode_code(m) for m in modes], dtype=np.int32))
        self.count = len(self.lengths)
        if offsets is None:
            self.offsets = np.concatenate([[0], np.cumsum(self.lengths)[:-1]]).astype(np.int64) \
                if self.count else np.zeros(0, np.int64)
            off_arg = None
        else:
            self.offsets = np.ascontiguousarray(np.asarray(offsets, dtype=np.int64))
            off_arg = self.offsets.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        self.total = int((self.offsets + self.lengths).max()) if self.count else 0
        self.dtype = dtype
        h = ctypes.c_void_p()
        L.check(L.lib().gbfft_ragged_plan_create(
            ctypes.byref(h), self.count, self.lengths.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
            off_arg, self.modes.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
            L.C64 if dtype == torch.complex128 else L.C32), "gbfft_ragged_plan_create")
        self.handle = h

    def exec_ptr(self, in_ptr, out_ptr, stream=None, per_transform=False):
        f = L.lib().gbfft_ragged_exec_per_transform if per_transform else L.lib().gbfft_ragged_exec
        L.check(f(self.handle, ctypes.c_void_p(in_ptr), ctypes.c_void_p(out_ptr), _stream(stream)),
                "gbfft_ragged_exec")

    def __call__(self, x, out=None, stream=None, per_transform=False):
        if out is None:
            out = torch.zeros_like(x)
        self.exec_ptr(x.data_ptr(), out.data_ptr(), stream, per_transform)
        return out

    def status(self, stream=None):
        return L.lib().gbfft_ragged_status(self.handle, _stream(stream))

    def close(self):
        if getattr(self, "handle", None):
            L.lib().gbfft_ragged_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SpecConvPlan:
    """Spectral convolution y_b = fft3D Inverse (fft3D Forward (x_b) * H) over a
    batch of d x h x w fields, with its adjoint (gbfft_specconv_*)."""

    def __init__(self, batch, d, h, w, dtype=torch.complex64):
        self.shape = (int(batch), int(d), int(h), int(w))
        self.dtype = dtype
        hd = ctypes.c_void_p()
        L.check(L.lib().gbfft_specconv_plan_create(ctypes.byref(hd), *self.shape,
                                                   L.C64 if dtype == torch.complex128 else L.C32),
                "gbfft_specconv_plan_create")
        self.handle = hd

    def _check(self, t, shape):
        if not t.is_cuda or not t.is_contiguous() or tuple(t.shape) != shape or t.dtype != self.dtype:
            raise ValueError("gbfft specconv: expected contiguous %s CUDA tensor of shape %s"
                             % (self.dtype, shape))

    def forward(self, x, H, out=None, stream=None):
        self._check(x, self.shape)
        self._check(H, self.shape[1:])
        y = torch.empty_like(x) if out is None else out
        L.check(L.lib().gbfft_specconv_fwd(self.handle, ctypes.c_void_p(x.data_ptr()),
                                           ctypes.c_void_p(H.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                           _stream(stream)), "gbfft_specconv_fwd")
        return y

    def backward(self, x, H, gy, stream=None):
        self._check(x, self.shape)
        self._check(H, self.shape[1:])
        self._check(gy, self.shape)
        gx = torch.empty_like(x)
        gH = torch.empty_like(H)
        L.check(L.lib().gbfft_specconv_bwd(self.handle, ctypes.c_void_p(x.data_ptr()),
                                           ctypes.c_void_p(H.data_ptr()), ctypes.c_void_p(gy.data_ptr()),
                                           ctypes.c_void_p(gx.data_ptr()), ctypes.c_void_p(gH.data_ptr()),
                                           _stream(stream)), "gbfft_specconv_bwd")
        return gx, gH

    def close(self):
        if getattr(self, "handle", None):
            L.lib().gbfft_specconv_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
