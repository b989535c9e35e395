"""A 2D convolution spread over several GPUs by one transpose per array,
the counterpart of the reference's Convolution2MPI (mpi/mpiconvolve.h:
72-176) over its mpitranspose (mpi/mpitranspose.h).

Layout and steps (rank r of P, one GPU each; every array is the caller's
Lx x Hy stored modes, Hy = the stored y extent):

1. input: rank r holds the y-slab of columns [y0_r, y1_r) of every input,
   a dense Lx x ny_r array;
2. the padded x transform of the slab (all residues, N_x rows: the
   standalone transform of the fftPad / fftPadCentered kind, row r*m + j
   holding residue r, entry j), on the rank's GPU;
3. all-to-all: rank r sends the rows of x-slab s, [x0_s, x1_s), of its
   columns to rank s, which assembles its nx_s x Hy rows (the reference's
   localize1);
4. the y sub-convolutions of those rows: the innermost-axis row kernel with
   the multiplier, as a batch of 1D convolutions (normalised by 1/N_y);
5. all-to-all back (localize0): each rank gets its columns of all N_x rows
   of the B outputs;
6. the backward x transform accumulated over residues and the 1/N_x
   normalisation, into the caller's y-slab.

The exchanges carry only the transformed x rows; no rank touches another
GPU's memory (NCCL all-to-all through local buffers), no multicast.  The
per-rank stages are an object with x_forward / rows / x_backward / scale;
the GPU one (GPUStages) runs the library's kernels; the tests on CPU ranks
pass the oracle as a stand-in.  This path has not been measured on more
than one GPU.
"""
from __future__ import annotations

from typing import Sequence

from ._native import CENTERED, HERMITIAN, PAD

__all__ = ["split", "Convolution2Distributed", "GPUStages"]


def split(n: int, parts: int, rank: int) -> tuple[int, int]:
    """[start, stop) of block `rank` when n items are split into `parts`
    contiguous blocks whose sizes differ by at most one (the first n % parts
    blocks take one more)."""
    if parts < 1 or not 0 <= rank < parts:
        raise ValueError("need 0 <= rank < parts")
    q, r = divmod(n, parts)
    start = rank * q + min(rank, r)
    return start, start + q + (1 if rank < r else 0)


class GPUStages:
    """The per-rank stages on the rank's GPU: the standalone padded x
    transform of the y-slab columns (fgb_pad_*), the batched 1D row
    convolutions with the multiplier (fgb_create with batch = the rank's x
    rows) and the normalisation kernel (fgb_scale_columns_device)."""

    def __init__(self, kinds, L, M, A, B, mult, precision, ny, nx_rows):
        from .gpu import HybridConvolution, PaddedTransform
        from . import _native
        self.lib = _native.load()
        self.xt = PaddedTransform(kinds[0], L[0], M[0], C=ny,
                                  precision=precision)
        self.Nx = self.xt.N
        self.rowconv = HybridConvolution([kinds[1]], [L[1]], [M[1]], A=A,
                                         B=B, mult=mult, precision=precision,
                                         batch=max(nx_rows, 1))
        self.precision = precision

    def x_forward(self, f):
        return self.xt.forward(f)

    def rows(self, Fs):
        return list(self.rowconv.convolve(*Fs))

    def x_backward(self, F):
        return self.xt.backward(F)

    def scale(self, h, s):
        import ctypes
        import torch
        from . import _native
        rows, cols = h.shape
        prec = _native.F64 if self.precision == "f64" else _native.F32
        st = torch.cuda.current_stream()
        rc = self.lib.fgb_scale_columns_device(
            rows, cols, s, s, ctypes.c_void_p(h.data_ptr()), prec,
            ctypes.c_void_p(st.cuda_stream))
        if rc != 0:
            raise RuntimeError(_native.last_error())
        return h


class Convolution2Distributed:
    """2D dealiased convolution over the ranks of a torch.distributed
    group.  kinds: x (outer) fftPad or fftPadCentered, y (inner) fftPad,
    fftPadCentered or fftPadHermitian; L, M per axis; A inputs, B outputs,
    a built-in multiplier.  Each rank passes its y-slab (`y_range`) of every
    input and receives its y-slab of the B outputs.  stages: the per-rank
    stage object (default: GPUStages on the current CUDA device)."""

    def __init__(self, kinds: Sequence[int], L: Sequence[int],
                 M: Sequence[int], *, A: int = 2, B: int = 1,
                 mult: str = "binary", precision: str = "f64", group=None,
                 stages=None, Nx: int | None = None):
        import torch.distributed as dist
        if len(kinds) != 2 or kinds[0] not in (PAD, CENTERED) or \
                kinds[1] not in (PAD, CENTERED, HERMITIAN):
            raise ValueError("a distributed 2D convolution takes a complex "
                             "x axis and a complex or Hermitian y axis")
        self.group = group
        self.P = dist.get_world_size(group)
        self.rank = dist.get_rank(group)
        self.kinds, self.L, self.M = list(kinds), list(L), list(M)
        self.A, self.B = A, B
        self.Hy = (L[1] + 1) // 2 if kinds[1] == HERMITIAN else L[1]
        if self.Hy < self.P:
            raise ValueError("fewer y columns than ranks")
        self.y_range = split(self.Hy, self.P, self.rank)
        self.ny = self.y_range[1] - self.y_range[0]
        if stages is None:
            # The x rows (N_x) come from the x transform's plan, the same
            # on every rank (it depends on L and M only).
            from .gpu import PaddedTransform
            Nx = PaddedTransform(kinds[0], L[0], M[0], C=1,
                                 precision=precision).N
            nx = split(Nx, self.P, self.rank)
            stages = GPUStages(kinds, L, M, A, B, mult, precision, self.ny,
                               nx[1] - nx[0])
        self.stages = stages
        self.Nx = stages.Nx if Nx is None else Nx
        if self.Nx < self.P:
            raise ValueError("fewer x rows than ranks")
        self.x_ranges = [split(self.Nx, self.P, s) for s in range(self.P)]
        self.y_ranges = [split(self.Hy, self.P, s) for s in range(self.P)]

    # -- the transposes ----------------------------------------------------
    def to_rows(self, F):
        """localize1: this rank's N_x x ny columns -> its x-slab rows of all
        Hy columns (one all-to-all)."""
        import torch
        import torch.distributed as dist
        ins = [torch.view_as_real(F[x0:x1]).reshape(-1)
               for x0, x1 in self.x_ranges]
        send = torch.cat(ins)
        x0, x1 = self.x_ranges[self.rank]
        nx = x1 - x0
        recv_sizes = [nx * (y1 - y0) * 2 for y0, y1 in self.y_ranges]
        recv = torch.empty(sum(recv_sizes), dtype=send.dtype,
                           device=send.device)
        dist.all_to_all_single(recv, send, recv_sizes,
                               [t.numel() for t in ins], group=self.group)
        blocks = torch.split(recv, recv_sizes)
        cols = [torch.view_as_complex(b.reshape(nx, y1 - y0, 2))
                for b, (y0, y1) in zip(blocks, self.y_ranges)]
        return torch.cat(cols, dim=1).contiguous()

    def to_columns(self, Hr):
        """localize0: this rank's x-slab rows of all Hy columns -> its
        columns of all N_x rows."""
        import torch
        import torch.distributed as dist
        ins = [torch.view_as_real(Hr[:, y0:y1].contiguous()).reshape(-1)
               for y0, y1 in self.y_ranges]
        send = torch.cat(ins)
        recv_sizes = [(x1 - x0) * self.ny * 2 for x0, x1 in self.x_ranges]
        recv = torch.empty(sum(recv_sizes), dtype=send.dtype,
                           device=send.device)
        dist.all_to_all_single(recv, send, recv_sizes,
                               [t.numel() for t in ins], group=self.group)
        blocks = torch.split(recv, recv_sizes)
        rows = [torch.view_as_complex(b.reshape(x1 - x0, self.ny, 2))
                for b, (x0, x1) in zip(blocks, self.x_ranges)]
        return torch.cat(rows, dim=0).contiguous()

    def convolve(self, *slabs):
        """slabs: the A inputs' y-slabs (Lx x ny complex tensors on this
        rank's device); returns the B outputs' y-slabs, normalised as
        Convolution::convolve does."""
        if len(slabs) != self.A:
            raise ValueError(f"expected {self.A} inputs")
        st = self.stages
        rows = [self.to_rows(st.x_forward(f)) for f in slabs]
        outs = st.rows(rows)
        res = []
        for h in outs[:self.B]:
            cols = self.to_columns(h)
            res.append(st.scale(st.x_backward(cols), 1.0 / self.Nx))
        return res
