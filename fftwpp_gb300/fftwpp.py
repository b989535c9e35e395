"""Python interface of FFTW++'s wrappers/fftwpp.py, served by lib_fftwpp.so.

Same names, arguments and in-place semantics as the reference module
(wrappers/fftwpp.py:15-351): ``complex_align``, ``fftwpp_set_maxthreads``,
``fftwpp_get_maxthreads``, ``Convolution(shape)`` and
``HConvolution(shape)`` with ``.convolve(f, g)`` overwriting ``f``.  The
arrays stay host numpy arrays; each call copies them to the GB300, runs the
sm_103a kernels and copies the result back.

The reference module itself also runs unchanged against this library: copy
or symlink ``lib_fftwpp.so`` next to it (it loads ``lib_fftwpp.so`` from its
own directory, fftwpp.py:26-27).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native

__all__ = ["Convolution", "HConvolution", "complex_align",
           "fftwpp_set_maxthreads", "fftwpp_get_maxthreads",
           "set_drop_in_precision"]


def complex_align(shape):
    """A complex128 array of `shape` whose data is 16-byte aligned
    (fftwpp.py:15-20)."""
    dtype = np.dtype(np.complex128)
    nbytes = int(np.prod(shape)) * dtype.itemsize
    buf = np.empty(nbytes + 16, dtype=np.uint8)
    start = -buf.ctypes.data % 16
    return buf[start:start + nbytes].view(dtype).reshape(shape)


def fftwpp_set_maxthreads(nthreads):
    _native.load().set_fftwpp_maxthreads(nthreads)


def fftwpp_get_maxthreads():
    return _native.load().get_fftwpp_maxthreads()


def set_drop_in_precision(precision: str = "f64"):
    """Arithmetic of convolutions created afterwards (their arrays stay
    complex128): "f64" (default) or "ff" (float-float, FP64-grade accuracy,
    about 3x faster on GB300).  Not in the reference module."""
    code = {"f64": _native.F64, "ff": _native.FF}.get(precision)
    if code is None or _native.load().fgb_set_drop_in_precision(code) != 0:
        raise ValueError("precision must be 'f64' or 'ff'")


def _check(a, shape):
    if not isinstance(a, np.ndarray) or a.dtype != np.complex128:
        raise TypeError("arrays must be numpy complex128")
    if a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("arrays must be C-contiguous")


class Convolution:
    """Implicitly dealiased complex convolution of 1, 2 or 3 dimensions
    (fftwpp.py:84-223); `shape` is the data shape."""

    def __init__(self, shape):
        if isinstance(shape, int):
            shape = (shape,)
        self.dim = len(shape)
        self.shape = tuple(int(s) for s in shape)
        lib = _native.load()
        if self.dim == 1:
            create, self._convolve, self._delete = (
                lib.fftwpp_create_conv1d, lib.fftwpp_conv1d_convolve,
                lib.fftwpp_conv1d_delete)
        elif self.dim == 2:
            create, self._convolve, self._delete = (
                lib.fftwpp_create_conv2d, lib.fftwpp_conv2d_convolve,
                lib.fftwpp_conv2d_delete)
        elif self.dim == 3:
            create, self._convolve, self._delete = (
                lib.fftwpp_create_conv3d, lib.fftwpp_conv3d_convolve,
                lib.fftwpp_conv3d_delete)
        else:
            raise ValueError("invalid shape (length/dimension should be 1, "
                             "2, or 3)")
        self.cptr = create(*self.shape)
        if not self.cptr:
            raise RuntimeError(_native.last_error())

    def __del__(self):
        if getattr(self, "cptr", None):
            self._delete(self.cptr)
            self.cptr = None

    def convolve(self, f, g):
        """Compute the convolution of f and g in place (f is overwritten)."""
        _check(f, self.shape)
        _check(g, self.shape)
        self._convolve(self.cptr, f.ctypes.data, g.ctypes.data)


class HConvolution:
    """Implicitly dealiased centred Hermitian convolution
    (fftwpp.py:225-351).  `shape` is the stored shape: the last axis holds
    the non-negative modes (H = ceil(L/2) with L = 2H-1)."""

    def __init__(self, shape):
        if isinstance(shape, int):
            shape = (shape,)
        self.dim = len(shape)
        self.shape = tuple(int(s) for s in shape)
        lib = _native.load()
        self._lib = lib
        if self.dim == 1:
            self.cptr = lib.fftwpp_create_hconv1d(2 * self.shape[0] - 1)
            self._convolve, self._delete = (lib.fftwpp_hconv1d_convolve,
                                            lib.fftwpp_hconv1d_delete)
        elif self.dim == 2:
            self.cptr = lib.fftwpp_create_hconv2d(self.shape[0],
                                                  2 * self.shape[1] - 1)
            self._convolve, self._delete = (lib.fftwpp_hconv2d_convolve,
                                            lib.fftwpp_hconv2d_delete)
        elif self.dim == 3:
            self.cptr = lib.fftwpp_create_hconv3d(self.shape[0], self.shape[1],
                                                  2 * self.shape[2] - 1)
            self._convolve, self._delete = (lib.fftwpp_hconv3d_convolve,
                                            lib.fftwpp_hconv3d_delete)
        else:
            raise ValueError("invalid shape (dimension should be 1, 2, or 3)")
        if not self.cptr:
            raise RuntimeError(_native.last_error())

    def __del__(self):
        if getattr(self, "cptr", None):
            self._delete(self.cptr)
            self.cptr = None

    def _symmetrize(self, a):
        lib = self._lib
        p = ctypes.c_void_p(a.ctypes.data)
        if self.dim == 1:
            lib.fftwpp_HermitianSymmetrize(p)
        elif self.dim == 2:
            Lx = a.shape[0]
            lib.fftwpp_HermitianSymmetrizeX((Lx + 1) // 2, a.shape[1], Lx // 2,
                                            p)
        else:
            Lx, Ly = a.shape[0], a.shape[1]
            lib.fftwpp_HermitianSymmetrizeXY((Lx + 1) // 2, (Ly + 1) // 2,
                                             a.shape[2], Lx // 2, Ly // 2, p)

    def convolve(self, f, g):
        """Enforce Hermitian symmetry on the inputs, then convolve in place
        (f is overwritten), as fftwpp.py:316-349 does."""
        _check(f, self.shape)
        _check(g, self.shape)
        self._symmetrize(f)
        self._symmetrize(g)
        self._convolve(self.cptr, f.ctypes.data, g.ctypes.data)
