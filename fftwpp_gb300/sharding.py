"""Sharding of a batch of independent 1D convolutions across ranks.

One process drives one GPU.  The problems of a batch are independent, so the
ranks exchange no data on the convolution path: every rank derives the same
partition from the list of lengths, plans a persistent batched launch over
its own shard and convolves it.  A host-side gather reassembles the outputs
in one process only when the caller asks for it.

The reference has no batched 1D path (a program keeps one Convolution object
per problem, convolve.h:1018-1166) and its MPI layer distributes a single
large 2D/3D convolution by transposition (mpi/mpiconvolve.h:121-176); that
all-to-all path is not built here.
"""
from __future__ import annotations

import math

import numpy as np


def problem_cost(L: int, M: int | None = None) -> float:
    """Relative cost of one convolution: M log2 M for the padded length M
    (default 2L-1), the operation count of its padded transforms."""
    M = 2 * int(L) - 1 if M is None else int(M)
    M = max(M, 2)
    return M * math.log2(M)


def partition(lengths, world: int, M=None) -> list[list[int]]:
    """Split problem indices into `world` shards of nearly equal total cost.

    Longest-processing-time-first greedy: problems in decreasing cost (ties
    by index) go to the least-loaded rank (ties by rank), so every rank that
    calls it with the same lengths gets the same answer.  Each shard is
    returned in increasing index order; a shard may be empty when there are
    fewer problems than ranks.
    """
    if world < 1:
        raise ValueError("world must be >= 1")
    n = len(lengths)
    Ms = [None] * n if M is None else list(M)
    if len(Ms) != n:
        raise ValueError("lengths and M differ in size")
    costs = [problem_cost(lengths[i], Ms[i]) for i in range(n)]
    order = sorted(range(n), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    shards: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        shards[r].append(i)
        load[r] += costs[i]
    return [sorted(s) for s in shards]


def offsets(lengths) -> list[int]:
    """Start of every problem in a packed array holding them back to back."""
    out, off = [], 0
    for L in lengths:
        out.append(off)
        off += int(L)
    return out


def _cat(pieces, like):
    try:
        import torch
        if isinstance(like, torch.Tensor):
            if not pieces:
                return like.new_empty((0,))
            return torch.cat(pieces)
    except ImportError:
        pass
    if not pieces:
        return np.empty(0, dtype=np.asarray(like).dtype)
    return np.concatenate(pieces)


def take(packed, lengths, index):
    """Pack problems `index` of a packed array (numpy array or torch
    tensor) into a new packed array, in the order given."""
    off = offsets(lengths)
    return _cat([packed[off[i]:off[i] + lengths[i]] for i in index], packed)


def place(local, lengths, index, out):
    """Inverse of take(): write the packed problems `local` (problems
    `index`, in that order) into their slots of the global packed `out`."""
    off = offsets(lengths)
    pos = 0
    for i in index:
        L = int(lengths[i])
        out[off[i]:off[i] + L] = local[pos:pos + L]
        pos += L
    if pos != len(local):
        raise ValueError("local array does not match the shard's lengths")
    return out


class ShardedBatch:
    """This rank's share of a batch of independent 1D convolutions.

    lengths, M: the whole batch (identical on every rank).  The plan is built
    on first use (`conv`), so the host-side logic needs no GPU.  Further
    keyword arguments go to BatchedConvolution (A, B, mult, precision, kind,
    tune).
    """

    def __init__(self, lengths, rank: int, world: int, M=None, **plan_kw):
        if not 0 <= rank < world:
            raise ValueError("rank out of range")
        self.lengths = [int(x) for x in lengths]
        self.M = ([2 * l - 1 for l in self.lengths] if M is None
                  else [int(x) for x in M])
        self.rank, self.world = rank, world
        self.shards = partition(self.lengths, world, self.M)
        self.index = self.shards[rank]
        self.local_lengths = [self.lengths[i] for i in self.index]
        self.local_M = [self.M[i] for i in self.index]
        self.local_total = sum(self.local_lengths)
        self.total = sum(self.lengths)
        self._plan_kw = plan_kw
        self._conv = None

    @property
    def conv(self):
        """The BatchedConvolution of this shard (None for an empty shard)."""
        if self._conv is None and self.index:
            from .gpu import BatchedConvolution
            self._conv = BatchedConvolution(self.local_lengths, self.local_M,
                                            **self._plan_kw)
        return self._conv

    def local(self, packed):
        """This shard's problems out of a global packed array."""
        return take(packed, self.lengths, self.index)

    def place(self, local, out):
        """Write this shard's packed outputs into a global packed array."""
        return place(local, self.lengths, self.index, out)

    def convolve(self, *inputs, out=None, graph: bool = True, stream=None):
        """Convolve this shard (inputs are local packed CUDA tensors)."""
        if self.conv is None:
            return [] if out is None else out
        return self.conv.convolve(*inputs, out=out, graph=graph, stream=stream)

    def gather(self, local_out, dst: int = 0, group=None):
        """Reassemble every rank's packed output on rank `dst` (host copy,
        through torch.distributed object gather); returns the global packed
        numpy array on `dst` and None elsewhere."""
        import torch
        import torch.distributed as dist
        arr = (local_out.detach().cpu().numpy()
               if isinstance(local_out, torch.Tensor) else np.asarray(local_out))
        parts = [None] * self.world if dist.get_rank(group) == dst else None
        dist.gather_object(arr, parts, dst=dst, group=group)
        if parts is None:
            return None
        out = np.zeros(self.total, dtype=arr.dtype)
        for r, part in enumerate(parts):
            place(part, self.lengths, self.shards[r], out)
        return out
