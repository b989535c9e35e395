"""GPU: many uneven 1D convolutions in one persistent launch (short problems
in one CTA, long ones through the column/row/column phases with bounded
in-kernel waits), replayed from a CUDA graph, against the CPU oracle."""
import numpy as np
import pytest

from oracle import hybrid as H
from oracle.direct import rel_l2

pytestmark = pytest.mark.gpu


def _lengths(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    return [int(round(np.exp(u))) for u in
            rng.uniform(np.log(lo), np.log(hi), n)]


@pytest.mark.parametrize("precision,tol", [("f64", 1e-13), ("f32", 2e-6)])
@pytest.mark.parametrize("tune", [False, True])
def test_batched_uneven(precision, tol, tune, native_lib):
    import torch
    from fftwpp_gb300.gpu import BatchedConvolution
    Ls = _lengths(24, 8, 9000, seed=5) + [1, 2, 3, 6000]
    conv = BatchedConvolution(Ls, precision=precision, tune=tune)
    assert conv.long_problems > 0 and conv.short_problems > 0
    rng = np.random.default_rng(1)
    f = rng.uniform(-1, 1, conv.total) + 1j * rng.uniform(-1, 1, conv.total)
    g = rng.uniform(-1, 1, conv.total) + 1j * rng.uniform(-1, 1, conv.total)
    tf = torch.from_numpy(f).to(conv.dtype).cuda()
    tg = torch.from_numpy(g).to(conv.dtype).cuda()
    for graph in (False, True, True):   # direct, capture, replay
        out = conv.convolve(tf, tg, graph=graph)[0]
        torch.cuda.synchronize()
        assert conv.error() == 0
        h = out.cpu().numpy()
        for o, L, M in zip(conv.offsets, conv.L, conv.M):
            want = H.convolve([f[o:o + L], g[o:o + L]], [H.PAD], [L], [M])[0]
            assert rel_l2(h[o:o + L], want) <= tol, (L, conv.choice(
                conv.L.index(L)))


def test_batched_matches_single_plans(native_lib):
    """Each problem of the batch equals the same problem run alone."""
    import torch
    from fftwpp_gb300.gpu import BatchedConvolution, HybridConvolution
    Ls = [100, 3000, 17]
    conv = BatchedConvolution(Ls)
    rng = np.random.default_rng(2)
    f = rng.uniform(-1, 1, conv.total) + 1j * rng.uniform(-1, 1, conv.total)
    g = rng.uniform(-1, 1, conv.total) + 1j * rng.uniform(-1, 1, conv.total)
    out = conv.convolve(torch.from_numpy(f).cuda(),
                        torch.from_numpy(g).cuda())[0].cpu().numpy()
    for o, L in zip(conv.offsets, Ls):
        single = HybridConvolution([H.PAD], [L], [2 * L - 1])
        s = single.convolve(torch.from_numpy(f[o:o + L].copy()).cuda(),
                            torch.from_numpy(g[o:o + L].copy()).cuda())[0]
        assert rel_l2(out[o:o + L], s.cpu().numpy()) <= 1e-13


@pytest.mark.parametrize("graph", [False, True])
def test_bounded_wait_runs_out(native_lib, graph):
    """Failure detection without a GPU fault: one long problem's dependency
    counter is made unreachable, so its row and column tasks poll a count
    that never completes until the (short) poll limit runs out; they give
    up, the error flag is raised, the launch finishes, every other problem
    is still exact, and the context stays usable."""
    import torch
    from fftwpp_gb300.gpu import BatchedConvolution
    lib = native_lib
    Ls = [40, 700, 20000, 3000, 25000, 90]
    conv = BatchedConvolution(Ls, precision="f64")
    long_ids = [i for i in range(len(Ls)) if conv.choice(i) < 0]
    short_ids = [i for i in range(len(Ls)) if conv.choice(i) > 0]
    assert long_ids and short_ids
    assert lib.fgb_batch_block_problem(conv.handle, short_ids[0], 1) == -1
    bad = long_ids[0]
    rng = np.random.default_rng(3)
    f = rng.uniform(-1, 1, conv.total) + 1j * rng.uniform(-1, 1, conv.total)
    g = rng.uniform(-1, 1, conv.total) + 1j * rng.uniform(-1, 1, conv.total)
    tf, tg = torch.from_numpy(f).cuda(), torch.from_numpy(g).cuda()
    want = [H.convolve([f[o:o + L], g[o:o + L]], [H.PAD], [L], [2 * L - 1])[0]
            for o, L in zip(conv.offsets, Ls)]

    assert lib.fgb_batch_set_spin_limit(conv.handle, 2000) == 0
    assert lib.fgb_batch_block_problem(conv.handle, bad, 1) == 0
    out = conv.convolve(tf, tg, graph=graph)[0]
    torch.cuda.synchronize()
    assert conv.error() == 1
    assert conv.error() == 0                      # reading clears the flag
    h = out.cpu().numpy()
    for i, (o, L) in enumerate(zip(conv.offsets, Ls)):
        if i != bad:
            assert rel_l2(h[o:o + L], want[i]) <= 1e-13

    assert lib.fgb_batch_block_problem(conv.handle, bad, 0) == 0
    assert lib.fgb_batch_set_spin_limit(conv.handle, 20000000) == 0
    out = conv.convolve(tf, tg, graph=graph)[0]
    torch.cuda.synchronize()
    assert conv.error() == 0
    h = out.cpu().numpy()
    for i, (o, L) in enumerate(zip(conv.offsets, Ls)):
        assert rel_l2(h[o:o + L], want[i]) <= 1e-13
