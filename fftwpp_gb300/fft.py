"""Plain FFT classes of fftw++.h on the GB300 kernels (CUDA tensors).

The class names and constructor arguments follow fftw++.h (fft1d
fftw++.h:556, mfft1d :827, rcfft1d :917, crfft1d :957, mrcfft1d :1023,
mcrfft1d :1122, fft2d :1199, rcfft2d :1249, crfft2d :1318, fft3d :1390,
rcfft3d / crfft3d after it).  Transforms are unnormalised like FFTW's;
fftNormalized divides by the number of points.  Signs: complex transforms
take +1 or -1, real-to-complex use -1 and complex-to-real +1.  Every pass
runs in the hand-written shared-memory kernels of lib_fftwpp.so through
fgb_fft_* (include/fftwpp_gb300.h); there is no library or CPU fallback.

fft0 / fft0Normalized are the origin-shifted transforms of rcfft2d,
crfft2d, rcfft3d and crfft3d (Fourier origin at (nx/2, 0) or
(nx/2, ny/2, 0)): the forward ones negate the entries with i (+ j) odd of
their real input first, as fftw++ does to its input, the backward ones of
their real output afterwards; the other classes ignore the shift, as in
fftw++.h.

Differences from fftw++.h: arrays are torch CUDA tensors (complex128 /
float64, or complex64 / float32 with precision="f32"); lengths must be
products of 2, 3, 5 and 7 (even for real transforms); real transforms and
interleaved sequences stay within one CTA's shared memory, while complex
sequences of any such length (fft1d, mfft1d with stride 1) take two passes;
complex-to-real transforms leave their input intact.
"""
from __future__ import annotations

import ctypes

from . import _native
from ._native import F32, F64

__all__ = ["fft1d", "mfft1d", "rcfft1d", "crfft1d", "mrcfft1d", "mcrfft1d",
           "fft2d", "rcfft2d", "crfft2d", "fft3d", "rcfft3d", "crfft3d"]

C2C, R2C, C2R = 0, 1, 2


class _Pass:
    """One fgb_fft pass: C interleaved sequences of length n in B batches."""

    def __init__(self, lib, kind, n, sign, C, B, istride, ibatch, ostride,
                 obatch, prec):
        self.lib = lib
        self.handle = lib.fgb_fft_create(kind, n, sign, C, B, istride, ibatch,
                                         ostride, obatch, prec)
        if not self.handle:
            raise ValueError(_native.last_error())

    def run(self, src, dst, stream):
        rc = self.lib.fgb_fft_execute_device(
            self.handle, ctypes.c_void_p(src.data_ptr()),
            ctypes.c_void_p(dst.data_ptr()), ctypes.c_void_p(stream))
        if rc != 0:
            raise RuntimeError(_native.last_error())

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            try:
                self.lib.fgb_fft_destroy(h)
            except Exception:
                pass


class _Plain:
    """Passes applied in order; the first reads `in`, the rest work in place
    on the output (complex-to-real: on a scratch copy of the input, then
    into the output)."""

    def __init__(self, in_shape, in_kind, out_shape, out_kind, passes,
                 npoints, precision, scratch=False):
        import torch
        if precision not in ("f64", "f32"):
            raise ValueError("precision must be 'f64' or 'f32'")
        self.lib = _native.load()
        self.prec = F64 if precision == "f64" else F32
        torch.cuda.current_device()
        cdt = torch.complex128 if self.prec == F64 else torch.complex64
        rdt = torch.float64 if self.prec == F64 else torch.float32
        self.in_shape, self.out_shape = tuple(in_shape), tuple(out_shape)
        self.in_dtype = cdt if in_kind == "c" else rdt
        self.out_dtype = cdt if out_kind == "c" else rdt
        self.passes = [_Pass(self.lib, *p, self.prec) for p in passes]
        self.npoints = npoints
        self.scratch = scratch

    def _check(self, t, shape, dtype, what):
        if (not t.is_cuda or t.dtype != dtype or tuple(t.shape) != shape or
                not t.is_contiguous()):
            raise ValueError(f"{what} must be a contiguous CUDA tensor of "
                             f"shape {shape} and type {dtype}")

    def fft(self, x, out=None, stream=None):
        import torch
        self._check(x, self.in_shape, self.in_dtype, "input")
        if out is None:
            out = torch.empty(self.out_shape, dtype=self.out_dtype,
                              device=x.device)
        self._check(out, self.out_shape, self.out_dtype, "output")
        s = (stream if stream is not None else
             torch.cuda.current_stream()).cuda_stream
        if self.scratch:
            # Complex passes in place on a copy, the last pass into `out`.
            w = x.clone()
            for p in self.passes[:-1]:
                p.run(w, w, s)
            self.passes[-1].run(w, out, s)
            return out
        self.passes[0].run(x, out, s)
        for p in self.passes[1:]:
            p.run(out, out, s)
        return out

    def Normalize(self, out):
        out.div_(self.npoints)
        return out

    def fftNormalized(self, x, out=None, stream=None):
        return self.Normalize(self.fft(x, out, stream))

    # Origin shift (fftw::Shift) of the real side: None for classes that
    # ignore it, else ("in" | "out", shape of the real array).
    shift = None

    def _shift(self, t, stream):
        import torch
        s = (stream if stream is not None else
             torch.cuda.current_stream()).cuda_stream
        dims = list(t.shape) + [1] * (3 - t.dim())
        rc = self.lib.fgb_fft_origin_shift_device(
            ctypes.c_void_p(t.data_ptr()), dims[0], dims[1], dims[2],
            self.prec, ctypes.c_void_p(s))
        if rc != 0:
            raise ValueError(_native.last_error())

    def fft0(self, x, out=None, stream=None):
        """The transform with the Fourier origin shifted to (nx/2, 0) (2D) or
        (nx/2, ny/2, 0) (3D); the forward real-to-complex classes negate
        their input's entries with i (+ j) odd in place first, as fftw++
        does."""
        if self.shift == "in":
            self._check(x, self.in_shape, self.in_dtype, "input")
            self._shift(x, stream)
        out = self.fft(x, out, stream)
        if self.shift == "out":
            self._shift(out, stream)
        return out

    def fft0Normalized(self, x, out=None, stream=None):
        return self.Normalize(self.fft0(x, out, stream))


def _mgeom(n, M, stride, dist):
    """(C, B, stride, batch) of M sequences at t*dist + s*stride."""
    if M == 1:
        return 1, 1, stride, n * stride
    if dist == 1:
        return M, 1, stride, 0
    return 1, M, stride, dist


class fft1d(_Plain):
    def __init__(self, nx, sign, precision="f64"):
        super().__init__((nx,), "c", (nx,), "c",
                         [(C2C, nx, sign, 1, 1, 1, nx, 1, nx)], nx, precision)


class mfft1d(_Plain):
    """M transforms of length nx, element s of transform t at
    t*dist + s*stride (dist defaults to nx for stride 1, else 1)."""

    def __init__(self, nx, sign, M=1, stride=1, dist=None, precision="f64"):
        if dist is None:
            dist = nx if stride == 1 else 1
        C, B, st, bd = _mgeom(nx, M, stride, dist)
        size = (nx - 1) * stride + (M - 1) * dist + 1
        super().__init__((size,), "c", (size,), "c",
                         [(C2C, nx, sign, C, B, st, bd, st, bd)], nx,
                         precision)


class rcfft1d(_Plain):
    def __init__(self, nx, precision="f64"):
        h = nx // 2 + 1
        super().__init__((nx,), "r", (h,), "c",
                         [(R2C, nx, -1, 1, 1, 1, nx, 1, h)], nx, precision)


class crfft1d(_Plain):
    def __init__(self, nx, precision="f64"):
        h = nx // 2 + 1
        super().__init__((h,), "c", (nx,), "r",
                         [(C2R, nx, 1, 1, 1, 1, h, 1, nx)], nx, precision)


class mrcfft1d(_Plain):
    """M real sequences of length nx, one per row (rows of nx reals in,
    rows of nx/2+1 complex out)."""

    def __init__(self, nx, M=1, precision="f64"):
        h = nx // 2 + 1
        super().__init__((M, nx), "r", (M, h), "c",
                         [(R2C, nx, -1, 1, M, 1, nx, 1, h)], nx, precision)


class mcrfft1d(_Plain):
    def __init__(self, nx, M=1, precision="f64"):
        h = nx // 2 + 1
        super().__init__((M, h), "c", (M, nx), "r",
                         [(C2R, nx, 1, 1, M, 1, h, 1, nx)], nx, precision)


class fft2d(_Plain):
    def __init__(self, nx, ny, sign, precision="f64"):
        super().__init__((nx, ny), "c", (nx, ny), "c",
                         [(C2C, ny, sign, 1, nx, 1, ny, 1, ny),
                          (C2C, nx, sign, ny, 1, ny, 0, ny, 0)],
                         nx * ny, precision)


class rcfft2d(_Plain):
    """nx x ny reals -> nx x (ny/2+1) complex (the ky >= 0 half plane)."""

    shift = "in"

    def __init__(self, nx, ny, precision="f64"):
        h = ny // 2 + 1
        super().__init__((nx, ny), "r", (nx, h), "c",
                         [(R2C, ny, -1, 1, nx, 1, ny, 1, h),
                          (C2C, nx, -1, h, 1, h, 0, h, 0)],
                         nx * ny, precision)


class crfft2d(_Plain):
    shift = "out"

    def __init__(self, nx, ny, precision="f64"):
        h = ny // 2 + 1
        super().__init__((nx, h), "c", (nx, ny), "r",
                         [(C2C, nx, 1, h, 1, h, 0, h, 0),
                          (C2R, ny, 1, 1, nx, 1, h, 1, ny)],
                         nx * ny, precision, scratch=True)


class fft3d(_Plain):
    def __init__(self, nx, ny, nz, sign, precision="f64"):
        super().__init__((nx, ny, nz), "c", (nx, ny, nz), "c",
                         [(C2C, nz, sign, 1, nx * ny, 1, nz, 1, nz),
                          (C2C, ny, sign, nz, nx, nz, ny * nz, nz, ny * nz),
                          (C2C, nx, sign, ny * nz, 1, ny * nz, 0, ny * nz, 0)],
                         nx * ny * nz, precision)


class rcfft3d(_Plain):
    shift = "in"

    def __init__(self, nx, ny, nz, precision="f64"):
        h = nz // 2 + 1
        super().__init__((nx, ny, nz), "r", (nx, ny, h), "c",
                         [(R2C, nz, -1, 1, nx * ny, 1, nz, 1, h),
                          (C2C, ny, -1, h, nx, h, ny * h, h, ny * h),
                          (C2C, nx, -1, ny * h, 1, ny * h, 0, ny * h, 0)],
                         nx * ny * nz, precision)


class crfft3d(_Plain):
    shift = "out"

    def __init__(self, nx, ny, nz, precision="f64"):
        h = nz // 2 + 1
        super().__init__((nx, ny, h), "c", (nx, ny, nz), "r",
                         [(C2C, nx, 1, ny * h, 1, ny * h, 0, ny * h, 0),
                          (C2C, ny, 1, h, nx, h, ny * h, h, ny * h),
                          (C2R, nz, 1, 1, nx * ny, 1, h, 1, nz)],
                         nx * ny * nz, precision, scratch=True)
