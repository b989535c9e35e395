"""fftwpp_gb300: FFTW++'s hybrid dealiased convolution, GB300-native.

* ``fftwpp_gb300.gpu.HybridConvolution`` -- device tensors, any padded
  transform kind per axis, FP64 or FP32-compensated.
* ``fftwpp_gb300.fftwpp`` -- the reference's Python wrapper interface
  (``Convolution``, ``HConvolution``) over host numpy arrays.
* ``lib_fftwpp.so`` -- the C ABI (include/cfftw++.h, include/fftwpp_gb300.h).
"""
from ._native import CENTERED, HERMITIAN, PAD, REAL  # noqa: F401

__version__ = "0.1.0"
