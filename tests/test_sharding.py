"""Host-side logic of the sharded batched convolution: the partition, the
pack/unpack of shards and the gather, on world_size-2 gloo ranks (CPU).

Each rank stands in for one GPU: it convolves its own shard with the oracle
(the checker) instead of the CUDA kernel, which the GPU tests cover."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from fftwpp_gb300 import sharding as S


def lengths(n=40, seed=5):
    rng = np.random.default_rng(seed)
    return [int(round(np.exp(u))) for u in rng.uniform(np.log(4), np.log(300), n)]


def test_partition_covers_and_balances():
    Ls = lengths(200)
    for world in (1, 2, 3, 4, 8):
        shards = S.partition(Ls, world)
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(len(Ls)))
        loads = [sum(S.problem_cost(Ls[i]) for i in s) for s in shards]
        # LPT bound: no shard exceeds the mean by more than the largest job.
        assert max(loads) <= sum(loads) / world + max(
            S.problem_cost(L) for L in Ls) + 1e-9
        assert shards == S.partition(Ls, world)     # deterministic


def test_partition_edges():
    assert S.partition([], 3) == [[], [], []]
    assert S.partition([10], 2) == [[0], []]
    with pytest.raises(ValueError):
        S.partition([1, 2], 0)
    with pytest.raises(ValueError):
        S.partition([1, 2], 2, M=[3])


def test_take_place_roundtrip():
    Ls = lengths(17)
    x = np.arange(sum(Ls), dtype=np.complex128)
    out = np.zeros_like(x)
    for idx in S.partition(Ls, 3):
        loc = S.take(x, Ls, idx)
        assert len(loc) == sum(Ls[i] for i in idx)
        S.place(loc, Ls, idx, out)
    assert np.array_equal(out, x)
    with pytest.raises(ValueError):
        S.place(np.zeros(3), Ls, [0], np.zeros_like(x))


def test_take_place_torch():
    import torch
    Ls = [3, 1, 4, 1, 5]
    x = torch.arange(sum(Ls), dtype=torch.float64)
    idx = [4, 0, 2]
    loc = S.take(x, Ls, idx)
    assert loc.tolist() == [9.0, 10.0, 11.0, 12.0, 13.0, 0.0, 1.0, 2.0,
                            4.0, 5.0, 6.0, 7.0]
    out = torch.zeros_like(x)
    S.place(loc, Ls, idx, out)
    assert out[9:14].tolist() == x[9:14].tolist()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, Ls, q):
    import torch.distributed as dist
    from oracle import hybrid as H
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(11)       # same global inputs everywhere
        tot = sum(Ls)
        f = rng.uniform(-1, 1, tot) + 1j * rng.uniform(-1, 1, tot)
        g = rng.uniform(-1, 1, tot) + 1j * rng.uniform(-1, 1, tot)
        sh = S.ShardedBatch(Ls, rank, world)
        lf, lg = sh.local(f), sh.local(g)
        assert len(lf) == sh.local_total
        # The per-shard convolution (on the GPU in production).
        loc_off = S.offsets(sh.local_lengths)
        lh = np.empty_like(lf)
        for o, L in zip(loc_off, sh.local_lengths):
            lh[o:o + L] = H.convolve([lf[o:o + L], lg[o:o + L]], [H.PAD], [L],
                                     [2 * L - 1])[0]
        got = sh.gather(lh, dst=0)
        if rank == 0:
            off = S.offsets(Ls)
            err = 0.0
            for o, L in zip(off, Ls):
                want = H.convolve([f[o:o + L], g[o:o + L]], [H.PAD], [L],
                                  [2 * L - 1])[0]
                err = max(err, float(np.abs(got[o:o + L] - want).max()))
            q.put(("ok", err, [len(s) for s in sh.shards]))
        else:
            assert got is None
        dist.barrier()
    except Exception as e:                    # report to the parent
        q.put(("fail", repr(e), None))
        raise
    finally:
        dist.destroy_process_group()


def test_sharded_gather_gloo_world2():
    Ls = lengths(23)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, Ls, q))
             for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    for p in procs:
        if p.is_alive():
            p.kill()
    status, err, sizes = q.get(timeout=10)
    assert status == "ok", err
    assert err == 0.0                # gather places results bit for bit
    assert sum(sizes) == len(Ls) and min(sizes) > 0
    assert all(p.exitcode == 0 for p in procs)
