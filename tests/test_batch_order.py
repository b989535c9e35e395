"""Queue order of the batched launch (host logic, no GPU).

The persistent kernel dequeues tasks in this order and a consumer waits
(bounded) on its producers, so every problem's forward column tiles must
precede its row tasks and those its backward column tiles; the long
problems go in staging groups, software-pipelined, so that a problem's
staging is written and read back while few others are open.
"""
import ctypes

import numpy as np
import pytest

SMALL, COLFWD, ROW, COLBWD = 0, 1, 2, 3


def _order(lib, staging, fwd, rows, bwd, nsmall, A, B, group):
    n = len(staging)
    sz = ctypes.c_size_t
    ci = ctypes.c_int
    st = (sz * max(n, 1))(*staging)
    f = (ci * max(n, 1))(*fwd)
    r = (ci * max(n, 1))(*rows)
    b = (ci * max(n, 1))(*bwd)
    total = sum(fwd) * A + sum(rows) + sum(bwd) * B + nsmall
    typ = (ci * max(total, 1))()
    prob = (ci * max(total, 1))()
    k = lib.fgb_batch_task_order(n, st, f, r, b, nsmall, A, B, group, typ,
                                 prob, total)
    assert k == total
    return list(typ[:k]), list(prob[:k])


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("group", [1 << 20, 8 << 20, 24 << 20, 1 << 40])
def test_batch_task_order(native_lib, seed, group):
    rng = np.random.default_rng(seed)
    nlong = int(rng.integers(0, 40))
    nsmall = int(rng.integers(0, 300))
    A = int(rng.integers(1, 5))
    B = int(rng.integers(1, A + 1))
    staging = [int(x) for x in rng.integers(1 << 16, 4 << 20, nlong)]
    fwd = [int(x) for x in rng.integers(1, 9, nlong)]
    rows = [int(x) for x in rng.integers(1, 65, nlong)]
    bwd = [int(x) for x in rng.integers(1, 9, nlong)]
    typ, prob = _order(native_lib, staging, fwd, rows, bwd, nsmall, A, B,
                       group)
    # Every task exactly once.
    count = {}
    for t, p in zip(typ, prob):
        count[(t, p)] = count.get((t, p), 0) + 1
    for i in range(nlong):
        assert count.get((COLFWD, i), 0) == fwd[i] * A
        assert count.get((ROW, i), 0) == rows[i]
        assert count.get((COLBWD, i), 0) == bwd[i] * B
        assert count.get((SMALL, i), 0) == 0
    for j in range(nsmall):
        assert count.get((SMALL, nlong + j), 0) == 1
    assert len(typ) == sum(count.values())
    # Producers before consumers, per long problem.
    pos = {}
    for k, (t, p) in enumerate(zip(typ, prob)):
        lo, hi = pos.get((t, p), (k, k))
        pos[(t, p)] = (min(lo, k), max(hi, k))
    for i in range(nlong):
        assert pos[(COLFWD, i)][1] < pos[(ROW, i)][0]
        assert pos[(ROW, i)][1] < pos[(COLBWD, i)][0]
    # Staging open at any point of the queue: at most three groups (plus
    # the problem that overflows a group).
    first = {i: pos[(COLFWD, i)][0] for i in range(nlong)}
    last = {i: pos[(COLBWD, i)][1] for i in range(nlong)}
    events = sorted([(first[i], staging[i]) for i in range(nlong)] +
                    [(last[i] + 0.5, -staging[i]) for i in range(nlong)])
    open_bytes, peak = 0, 0
    for _, d in events:
        open_bytes += d
        peak = max(peak, open_bytes)
    bound = 3 * (group + max(staging, default=0))
    assert peak <= max(bound, 0) or group >= sum(staging)
