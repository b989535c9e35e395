"""Device-tensor interface to the GB300 hybrid dealiased convolution.

PyTorch supplies device memory and the current CUDA stream only; every
convolution runs in the hand-written kernels of lib_fftwpp.so through the C
ABI of include/fftwpp_gb300.h.  There is no CPU or library fallback: if the
native library is missing, construction raises.

The class mirrors the reference's composition of padded transforms and a
Convolution driver (convolve.h:471-1893): one padded-transform kind per axis
(PAD = fftPad, CENTERED = fftPadCentered, HERMITIAN = fftPadHermitian,
REAL = fftPadReal), a minimum padded length M per axis, A inputs, B outputs
and a multiplier.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

from . import _native
from ._native import (CENTERED, F32, F64, FF, HERMITIAN, MULT, PAD,
                      PRECISIONS, REAL)

__all__ = ["HybridConvolution", "BatchedConvolution", "PaddedTransform",
           "PAD", "CENTERED", "HERMITIAN", "REAL", "default_M",
           "set_autotune", "set_residue_search", "set_host_path",
           "set_ff_range_guard", "export_wisdom", "import_wisdom",
           "forget_wisdom", "save_wisdom", "load_wisdom"]


def set_autotune(on: bool = True) -> None:
    """Plan-time timing of schedules and of m, process-wide (fgb_set_autotune)."""
    _native.load().fgb_set_autotune(int(bool(on)))


def export_wisdom() -> str:
    """The plan records of this process as text (fgb_wisdom_export)."""
    lib = _native.load()
    n = lib.fgb_wisdom_export(None, 0)
    buf = ctypes.create_string_buffer(n + 1)
    lib.fgb_wisdom_export(buf, n + 1)
    return buf.value.decode()


def import_wisdom(text: str) -> int:
    """Merge plan records (fgb_wisdom_import); returns the lines taken."""
    n = _native.load().fgb_wisdom_import(text.encode())
    if n < 0:
        raise ValueError(_native.last_error())
    return n


def forget_wisdom() -> None:
    """Drop every plan record of this process (fgb_wisdom_forget)."""
    _native.load().fgb_wisdom_forget()


def save_wisdom(path: str) -> None:
    """Write the plan records to `path`, merged with those already there,
    through a temporary file and a rename (as FFTW++ saves wisdom3.txt,
    fftw++.cc:31-72)."""
    import os
    if os.path.exists(path):
        with open(path) as f:
            import_wisdom(f.read())
    tmp = f"{path}.{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        f.write(export_wisdom())
    os.replace(tmp, path)


def load_wisdom(path: str) -> int:
    """Merge the plan records of `path` (none if it does not exist)."""
    import os
    if not os.path.exists(path):
        return 0
    with open(path) as f:
        return import_wisdom(f.read())


def set_residue_search(on: bool = True) -> None:
    """Timed choice of the residue block length m per axis, process-wide
    (fgb_set_residue_search; the counterpart of FFTW++'s OptBase search)."""
    _native.load().fgb_set_residue_search(int(bool(on)))


def set_ff_range_guard(on: bool = True) -> None:
    """Exponent scaling of FP64 data in the float-float mode, process-wide
    (fgb_set_ff_range_guard, default on)."""
    _native.load().fgb_set_ff_range_guard(int(bool(on)))


def set_host_path(inputs: int = -1, outputs: int = -1) -> None:
    """How page-locked host arrays cross the host link (fgb_set_host_path):
    0 copies through device memory, 1 in place, 2 in place with 64-byte
    column tiles, -1 measured per plan."""
    for w in (inputs, outputs):
        if w not in (-1, 0, 1, 2):
            raise ValueError("host path ways are -1, 0, 1 or 2")
    _native.load().fgb_set_host_path(int(inputs), int(outputs))


def default_M(kind: int, L: int, A: int = 2) -> int:
    """Default minimum padded length of the reference's C wrappers
    (wrappers/HybridConvolution.h:19, 39)."""
    if kind in (CENTERED, HERMITIAN):
        return 3 * ((L + 1) // 2) - 2 * (L % 2)
    return A * L - A + 1


class HybridConvolution:
    """A planned convolution on the current CUDA device.

    kinds, L, M: per axis, outermost first.  m: optional forced residue
    block lengths (the reference's Application m).  precision: "f64" (the
    drop-in mode), "f32" (FP32 data with split hi+lo twiddles) or "ff"
    (FP64 data, float-float arithmetic on the FP32 pipe).
    batch: independent 1D problems stored back to back.
    """

    def __init__(self, kinds: Sequence[int], L: Sequence[int],
                 M: Sequence[int] | None = None, *, m: Sequence[int] | None = None,
                 A: int = 2, B: int = 1, mult: str = "binary",
                 precision: str = "f64", batch: int = 1):
        import torch
        self.lib = _native.load()
        self.kinds = list(kinds)
        self.L = list(L)
        self.dim = len(self.kinds)
        if M is None:
            M = [default_M(k, l, A) for k, l in zip(self.kinds, self.L)]
        self.M = list(M)
        self.A, self.B = A, B
        self.mult = mult
        self.precision = precision
        if precision not in PRECISIONS:
            raise ValueError(f"unknown precision {precision!r}")
        self.prec = PRECISIONS[precision]
        self.batch = batch
        self.real = self.kinds[0] == REAL
        sz = ctypes.c_size_t
        d = self.dim
        karr = (ctypes.c_int * d)(*self.kinds)
        Larr = (sz * d)(*self.L)
        Marr = (sz * d)(*self.M)
        marr = (sz * d)(*(m or [0] * d))
        torch.cuda.current_device()   # make sure a context exists
        self.handle = self.lib.fgb_create(d, karr, Larr, Marr, marr, A, B,
                                          MULT[mult], self.prec, batch)
        if not self.handle:
            raise ValueError(_native.last_error())
        info = (ctypes.c_long * 32)()
        self.lib.fgb_info(self.handle, info)
        self.axes = []
        for a in range(d):
            o = info[8 * a: 8 * a + 8]
            self.axes.append(dict(m=o[0], p=o[1], q=o[2], N=o[3], stored=o[4],
                                  cshift=o[5], tile=o[6], rows=o[7],
                                  tileB=info[27 + a]))
        self.launches = info[24]
        self.staging_bytes = info[25]
        self.long_path = bool(info[26])
        self.rows_per_cta = info[30]
        self.threads_per_cta = info[31]
        self.shape = tuple(ax["stored"] for ax in self.axes)
        if batch > 1:
            self.shape = (batch,) + self.shape

    def describe(self) -> str:
        """The plan in words: the counterpart of the reference's verbose
        dump (convolve.cc:451-469: m, p, q, C, S and the padding kind per
        axis), plus the GPU launch schedule (column tiles, rows per CTA,
        kernels, staging bytes)."""
        names = {PAD: "fftPad", CENTERED: "fftPadCentered",
                 HERMITIAN: "fftPadHermitian", REAL: "fftPadReal"}
        lines = [f"{self.dim}D convolution, A={self.A} B={self.B} "
                 f"multiplier={self.mult} precision={self.precision}"
                 + (f" batch={self.batch}" if self.batch > 1 else "")]
        for d, (k, ax) in enumerate(zip(self.kinds, self.axes)):
            padding = "explicit" if ax["q"] == 1 else "hybrid"
            inner = d == self.dim - 1 and not self.long_path
            sched = (f"rows/CTA={self.rows_per_cta} "
                     f"threads/CTA={self.threads_per_cta}" if inner else
                     f"tile={ax['tile']} tileB={ax['tileB']}")
            lines.append(f"  axis {d}: {names[k]} L={self.L[d]} M={self.M[d]} "
                         f"m={ax['m']} p={ax['p']} q={ax['q']} N={ax['N']} "
                         f"stored={ax['stored']} ({padding}) {sched}")
        lines.append(f"  kernels: {', '.join(self.launch_names())}"
                     f"{' (long 1D path)' if self.long_path else ''}")
        lines.append(f"  staging: {self.staging_bytes} bytes")
        return "\n".join(lines)

    # -- layout -------------------------------------------------------------
    @property
    def dtype(self):
        import torch
        if self.real:
            return torch.float32 if self.prec == F32 else torch.float64
        return torch.complex64 if self.prec == F32 else torch.complex128

    @property
    def normalization(self) -> int:
        n = 1
        for ax in self.axes:
            n *= ax["N"]
        return n

    def _check(self, t):
        import torch
        if not isinstance(t, torch.Tensor) or not t.is_cuda:
            raise TypeError("inputs must be CUDA tensors")
        if t.dtype != self.dtype:
            raise TypeError(f"expected {self.dtype}, got {t.dtype}")
        if tuple(t.shape) != self.shape or not t.is_contiguous():
            raise ValueError(f"expected a contiguous tensor of shape "
                             f"{self.shape}, got {tuple(t.shape)}")

    # -- execution ----------------------------------------------------------
    def convolve(self, *inputs, out=None, stream=None):
        """Convolve A device tensors; returns the B outputs (new tensors
        unless `out` is given; out may alias the inputs)."""
        import torch
        if len(inputs) != self.A:
            raise ValueError(f"expected {self.A} inputs")
        for t in inputs:
            self._check(t)
        if out is None:
            out = [torch.empty_like(inputs[0]) for _ in range(self.B)]
        for t in out:
            self._check(t)
        ins = (ctypes.c_void_p * self.A)(*[t.data_ptr() for t in inputs])
        outs = (ctypes.c_void_p * self.B)(*[t.data_ptr() for t in out])
        s = stream if stream is not None else torch.cuda.current_stream()
        rc = self.lib.fgb_convolve_device(self.handle, ins, outs,
                                          ctypes.c_void_p(s.cuda_stream))
        if rc != 0:
            raise RuntimeError(_native.last_error())
        return out

    def convolve_host(self, *arrays):
        """Convolve host numpy arrays through the host-pointer C entry
        (copies in and out inside the call); results overwrite arrays[0..B-1]."""
        import numpy as np
        if len(arrays) != self.A:
            raise ValueError(f"expected {self.A} inputs")
        want = {"torch.float64": np.float64, "torch.float32": np.float32,
                "torch.complex128": np.complex128,
                "torch.complex64": np.complex64}[str(self.dtype)]
        for a in arrays:
            if not (isinstance(a, np.ndarray) and a.flags["C_CONTIGUOUS"]):
                raise TypeError("host inputs must be C-contiguous numpy arrays")
            # The library copies exactly this many bytes in and out.
            if a.dtype != want or tuple(a.shape) != tuple(self.shape):
                raise TypeError(f"host inputs must be {np.dtype(want).name} "
                                f"arrays of shape {self.shape}")
        ptrs = (ctypes.c_void_p * self.A)(*[a.ctypes.data for a in arrays])
        rc = self.lib.fgb_convolve_host(self.handle, ptrs, ptrs)
        if rc != 0:
            raise RuntimeError(_native.last_error())
        return list(arrays[:self.B])

    def host_path(self) -> tuple[int, int]:
        """How page-locked inputs and outputs of convolve_host cross the
        host link: 0 whole-array copies, 1 in place with the device-tuned
        tiles, 2 in place with 64-byte tiles; -1 before the first call."""
        wi, wo = ctypes.c_int(), ctypes.c_int()
        self.lib.fgb_host_path(self.handle, ctypes.byref(wi), ctypes.byref(wo))
        return wi.value, wo.value

    # -- per-kernel timing ---------------------------------------------------
    def launch_names(self) -> list[str]:
        """Kernel launched at each position of one convolve call."""
        k = self.kinds
        inner = "herm_row" if k[-1] == HERMITIAN else "row_conv"
        x = "real" if k[0] == REAL else ""
        # Long inner rows: column kernels around the row kernel.
        rows = (["outer_fwd_cols", "row_conv", "outer_bwd_cols"]
                if self.long_path else [inner])
        if self.dim == 1:
            names = rows
        elif self.dim == 2:
            names = [f"outer{x}_fwd_x", *rows, f"outer{x}_bwd_x"]
        else:
            names = [f"outer{x}_fwd_x", "outer_fwd_y", *rows, "outer_bwd_y",
                     f"outer{x}_bwd_x"]
        return names

    def enable_timing(self, on: bool = True) -> None:
        if self.lib.fgb_timing(self.handle, int(on)) != 0:
            raise RuntimeError(_native.last_error())
        if on:
            self._ms = [0.0] * self.launches

    def collect_timing(self) -> None:
        """Accumulate the last call's per-kernel times (stream synchronised)."""
        buf = (ctypes.c_double * self.launches)(*([0.0] * self.launches))
        n = self.lib.fgb_timing_collect(self.handle, buf, self.launches)
        for i in range(max(n, 0)):
            self._ms[i] += buf[i]

    def kernel_ms(self) -> list[float]:
        return list(self._ms)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            try:
                self.lib.fgb_destroy(h)
            except Exception:
                pass
            self.handle = None


class BatchedConvolution:
    """Many independent 1D convolutions of uneven lengths in one persistent
    kernel launch, optionally replayed from a captured CUDA graph.

    lengths[i], M[i]: data length and minimum padded length of problem i
    (default M = 2L-1).  Each input/output is one packed device tensor
    holding all problems back to back.  tune=True times the candidate plans
    of every distinct length on the GPU and keeps the fastest.
    """

    def __init__(self, lengths, M=None, *, A: int = 2, B: int = 1,
                 mult: str = "binary", precision: str = "f64",
                 kind: int = PAD, tune: bool = False):
        import torch
        self.lib = _native.load()
        self.L = [int(x) for x in lengths]
        self.M = [int(x) for x in (M if M is not None else
                                   [2 * l - 1 for l in self.L])]
        self.n = len(self.L)
        self.A, self.B = A, B
        if precision not in ("f64", "f32"):
            raise ValueError(f"precision must be 'f64' or 'f32', not "
                             f"{precision!r}")
        self.prec = F64 if precision == "f64" else F32
        sz = ctypes.c_size_t
        torch.cuda.current_device()
        self.handle = self.lib.fgb_batch_create(
            self.n, (sz * self.n)(*self.L), (sz * self.n)(*self.M), A, B,
            MULT[mult], self.prec, kind, int(tune))
        if not self.handle:
            raise ValueError(_native.last_error())
        info = (ctypes.c_long * 6)()
        self.lib.fgb_batch_info(self.handle, info)
        self.tasks, self.grid, self.smem = info[0], info[1], info[2]
        self.short_problems, self.long_problems = info[3], info[4]
        self.total = info[5]
        self.offsets = []
        off = 0
        for l in self.L:
            self.offsets.append(off)
            off += l

    @property
    def dtype(self):
        import torch
        return torch.complex128 if self.prec == F64 else torch.complex64

    def choice(self, i: int) -> int:
        return self.lib.fgb_batch_choice(self.handle, i)

    def split(self, packed):
        """Views of the problems inside a packed tensor."""
        return [packed[o:o + l] for o, l in zip(self.offsets, self.L)]

    def convolve(self, *inputs, out=None, graph: bool = True, stream=None):
        import torch
        if len(inputs) != self.A:
            raise ValueError(f"expected {self.A} inputs")
        for t in inputs:
            if (t.dtype != self.dtype or not t.is_cuda or t.ndim != 1 or
                    t.numel() != self.total or not t.is_contiguous()):
                raise ValueError("inputs must be packed contiguous CUDA "
                                 f"tensors of {self.total} {self.dtype}")
        if out is None:
            out = [torch.empty_like(inputs[0]) for _ in range(self.B)]
        ins = (ctypes.c_void_p * self.A)(*[t.data_ptr() for t in inputs])
        outs = (ctypes.c_void_p * self.B)(*[t.data_ptr() for t in out])
        s = stream if stream is not None else torch.cuda.current_stream()
        rc = self.lib.fgb_batch_convolve_device(
            self.handle, ins, outs, ctypes.c_void_p(s.cuda_stream), int(graph))
        if rc != 0:
            raise RuntimeError(_native.last_error())
        return out

    def error(self) -> int:
        return self.lib.fgb_batch_error(self.handle)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            try:
                self.lib.fgb_batch_destroy(h)
            except Exception:
                pass
            self.handle = None


class PaddedTransform:
    """Standalone forward/backward padded transform along one axis of C
    interleaved columns (fftPad / fftPadCentered / fftPadHermitian /
    fftPadReal, convolve.h:515-536, 623-646, 737-757, 855-877), for work in
    padded space.

    Complex kinds: f has shape (L, C) (or (L,) for C = 1); forward returns
    F of shape (N, C) whose row r*m + j is the padded DFT (sign +1) at
    transformed index q*j + r (index(r, j)); backward is the unnormalised
    adjoint, so backward(forward(f)) = N f.  Real kind: f real (L, C), F
    complex (N/2 + 1, C) in natural frequency order.  Hermitian kind: f
    complex (ceil(L/2), C), the stored modes k >= 0; F real (N, C), the
    physical values at grid points 0..N-1 (explicit padding, N even).
    """

    def __init__(self, kind: int, L: int, M: int | None = None, *, C: int = 1,
                 m: int = 0, precision: str = "f64"):
        import torch
        self.lib = _native.load()
        self.kind, self.L, self.C = kind, int(L), int(C)
        self.M = int(M) if M is not None else default_M(kind, L)
        self.precision = precision
        if precision not in ("f64", "f32"):
            raise ValueError(f"precision must be 'f64' or 'f32', not "
                             f"{precision!r}")
        self.prec = F64 if precision == "f64" else F32
        torch.cuda.current_device()
        self.handle = self.lib.fgb_pad_create(kind, self.L, self.M, self.C,
                                              int(m), self.prec)
        if not self.handle:
            raise ValueError(_native.last_error())
        info = (ctypes.c_long * 10)()
        self.lib.fgb_pad_info(self.handle, info)
        (self.m, self.p, self.q, self.N, _, _, self.rows,
         self.cshift) = list(info)[:8]
        # Entries stored on the data side (ceil(L/2) Hermitian modes).
        self.stored = (self.L + 1) // 2 if kind == HERMITIAN else self.L

    @property
    def cdtype(self):
        """Element type of the transformed side F."""
        import torch
        if self.kind == HERMITIAN:
            return torch.float64 if self.prec == F64 else torch.float32
        return torch.complex128 if self.prec == F64 else torch.complex64

    @property
    def idtype(self):
        """Element type of the data side f."""
        import torch
        if self.kind == REAL:
            return torch.float64 if self.prec == F64 else torch.float32
        return torch.complex128 if self.prec == F64 else torch.complex64

    def index(self, r: int, j: int) -> int:
        return self.lib.fgb_pad_index(self.handle, r, j)

    def _check(self, t, rows, dtype, what):
        if (not t.is_cuda or t.dtype != dtype or not t.is_contiguous() or
                t.numel() != rows * self.C):
            raise ValueError(f"{what} must be a contiguous CUDA tensor of "
                             f"{rows} x {self.C} {dtype}")

    def forward(self, f, out=None, stream=None):
        import torch
        self._check(f, self.stored, self.idtype, "f")
        if out is None:
            out = torch.empty((self.rows, self.C), dtype=self.cdtype,
                              device=f.device)
        self._check(out, self.rows, self.cdtype, "out")
        s = stream if stream is not None else torch.cuda.current_stream()
        rc = self.lib.fgb_pad_forward_device(
            self.handle, ctypes.c_void_p(f.data_ptr()),
            ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(s.cuda_stream))
        if rc != 0:
            raise RuntimeError(_native.last_error())
        return out

    def backward(self, F, out=None, stream=None):
        import torch
        self._check(F, self.rows, self.cdtype, "F")
        if out is None:
            out = torch.empty((self.stored, self.C), dtype=self.idtype,
                              device=F.device)
        self._check(out, self.stored, self.idtype, "out")
        s = stream if stream is not None else torch.cuda.current_stream()
        rc = self.lib.fgb_pad_backward_device(
            self.handle, ctypes.c_void_p(F.data_ptr()),
            ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(s.cuda_stream))
        if rc != 0:
            raise RuntimeError(_native.last_error())
        return out

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            try:
                self.lib.fgb_pad_destroy(h)
            except Exception:
                pass
