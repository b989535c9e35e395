"""The multi-GPU 2D convolution (fftwpp_gb300.distributed, the counterpart
of the reference's Convolution2MPI, mpi/mpiconvolve.h:72-176) on gloo CPU
ranks: the transposes move every value bit for bit, and the whole
convolution, with the oracle standing in for each rank's GPU stages,
matches the oracle's single-process 2D convolution to 1e-13.  Unmeasured
on hardware (one GPU per run here)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from fftwpp_gb300 import distributed as D


def test_split_covers_and_balances():
    for n in (1, 7, 10, 1023, 1536):
        for parts in (1, 2, 3, 4, 8):
            if parts > n:
                continue
            blocks = [D.split(n, parts, r) for r in range(parts)]
            assert blocks[0][0] == 0 and blocks[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(blocks, blocks[1:]))
            sizes = [b - a for a, b in blocks]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        D.split(5, 2, 2)


class OracleStages:
    """The per-rank stages computed by the oracle on the CPU: explicit
    padded x transforms on an N_x grid and the hybrid 1D convolution of
    each transformed row (normalised by its 1/N_y)."""

    def __init__(self, kinds, L, M, mult, Nx):
        self.kinds, self.L, self.M, self.mult = kinds, L, M, mult
        self.Nx = Nx

    def x_forward(self, f):
        from oracle import explicit as E
        return torch.from_numpy(E._forward(f.numpy(), self.kinds[0],
                                           self.L[0], self.Nx, 0))

    def rows(self, Fs):
        from oracle import hybrid as H
        n = Fs[0].shape[0]
        out = np.empty(Fs[0].shape, dtype=np.complex128)
        for i in range(n):
            out[i] = H.convolve([F[i].numpy() for F in Fs], [self.kinds[1]],
                                [self.L[1]], [self.M[1]], mult=self.mult)[0]
        return [torch.from_numpy(out)]

    def x_backward(self, F):
        from oracle import explicit as E
        return torch.from_numpy(E._backward(F.numpy(), self.kinds[0],
                                            self.L[0], self.Nx, 0))

    def scale(self, h, s):
        return h * s


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _inputs(kinds, L, seed):
    from oracle import hybrid as H
    rng = np.random.default_rng(seed)
    Hy = (L[1] + 1) // 2 if kinds[1] == H.HERMITIAN else L[1]
    fs = []
    for _ in range(2):
        f = rng.uniform(-1, 1, (L[0], Hy)) + 1j * rng.uniform(-1, 1, (L[0], Hy))
        if kinds[1] == H.HERMITIAN:
            H.hermitian_symmetrize_x(f, (L[0] + 1) // 2, Hy, L[0] // 2)
        fs.append(f)
    return fs


def _rank_main(rank, world, port, case, q):
    import torch.distributed as dist
    from oracle import hybrid as H
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        kinds, L, M, mult = case
        fs = _inputs(kinds, L, seed=sum(L))          # same everywhere
        Nx = M[0] + 3
        st = OracleStages(kinds, L, M, mult, Nx)
        conv = D.Convolution2Distributed(kinds, L, M, mult=mult, stages=st)
        y0, y1 = conv.y_range
        slabs = [torch.from_numpy(np.ascontiguousarray(f[:, y0:y1]))
                 for f in fs]
        # Transposes: bit for bit against the full transform's rows, and
        # back again.
        Fl = st.x_forward(slabs[0])
        rows = conv.to_rows(Fl)
        full = st.x_forward(torch.from_numpy(fs[0]))
        x0, x1 = conv.x_ranges[rank]
        exact = bool(torch.equal(rows, full[x0:x1]))
        back = bool(torch.equal(conv.to_columns(rows), Fl))
        h = conv.convolve(*slabs)[0]
        parts = [None] * world
        dist.all_gather_object(parts, (y0, y1, h.numpy()))
        if rank == 0:
            got = np.concatenate([p[2] for p in sorted(parts,
                                                       key=lambda t: t[0])],
                                 axis=1)
            want = H.convolve(fs, kinds, L, M, mult=mult)[0]
            err = float(np.linalg.norm(got - want) / np.linalg.norm(want))
            q.put(("ok", exact, back, err))
        dist.barrier()
    except Exception as e:
        q.put(("fail", repr(e), None, None))
        raise
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
@pytest.mark.parametrize("case", [
    ([1, 2], [31, 31], [46, 46], "realbinary"),     # hconv2d
    ([0, 0], [12, 10], [23, 19], "binary")])        # conv2d
def test_distributed_convolution2_gloo(case, world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, case, q))
             for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    for p in procs:
        if p.is_alive():
            p.kill()
    status, exact, back, err = q.get(timeout=10)
    assert status == "ok", exact
    assert exact and back
    assert err <= 1e-13, err
    assert all(p.exitcode == 0 for p in procs)
