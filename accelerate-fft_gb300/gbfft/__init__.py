"""gbfft: GB300-native FFT engine behind accelerate-fft's GPU interface.

Python mirror of Data.Array.Accelerate.Math.FFT (src/Data/Array/Accelerate/
Math/FFT.hs:25-35): ``Mode``, ``fft``, ``fft1D``, ``fft2D``, ``fft3D`` over
complex64 (Complex Float) and complex128 (Complex Double) CUDA tensors, all
served by libgbfft.so through its C ABI (include/gbfft.h).
"""
from ._lib import GbfftError, lib, error_string  # noqa: F401
from .fft import (Mode, Plan, RaggedPlan, SpecConvPlan, autotune, centre, dft, dftG, dftGS,  # noqa: F401
                  fft, fft1D, fft2D, fft3D, idft, mode_code, ragged_autotune, roots_of_unity, shift)
