"""GPU: the per-rank stages of the distributed 2D convolution
(fftwpp_gb300.distributed.GPUStages: the standalone padded x transform of
a y-slab, the batched row convolutions, the normalisation kernel) on one
GPU as a one-rank NCCL group, against the oracle.  The exchange between
several GPUs is covered on CPU ranks (tests/test_distributed.py); runs on
more than one GPU are not made here."""
import os
import socket

import numpy as np
import pytest

from oracle import hybrid as H
from oracle.direct import rel_l2

pytestmark = pytest.mark.gpu


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("case", [
    ([H.CENTERED, H.HERMITIAN], [63, 63], [94, 94], "realbinary", "f64"),
    ([H.PAD, H.PAD], [24, 20], [47, 39], "binary", "f64"),
    ([H.CENTERED, H.HERMITIAN], [63, 63], [94, 94], "realbinary", "f32")])
def test_gpu_stages_one_rank(native_lib, case):
    import torch
    import torch.distributed as dist
    from fftwpp_gb300.distributed import Convolution2Distributed
    kinds, L, M, mult, prec = case
    rng = np.random.default_rng(3)
    Hy = (L[1] + 1) // 2 if kinds[1] == H.HERMITIAN else L[1]
    fs = []
    for _ in range(2):
        f = rng.uniform(-1, 1, (L[0], Hy)) + 1j * rng.uniform(-1, 1, (L[0], Hy))
        if kinds[1] == H.HERMITIAN:
            H.hermitian_symmetrize_x(f, (L[0] + 1) // 2, Hy, L[0] // 2)
        fs.append(f)
    want = H.convolve(fs, kinds, L, M, mult=mult)[0]
    store = dist.TCPStore("127.0.0.1", _free_port(), 1, True)
    dist.init_process_group("nccl", store=store, rank=0, world_size=1)
    try:
        conv = Convolution2Distributed(kinds, L, M, mult=mult, precision=prec)
        dt = torch.complex128 if prec == "f64" else torch.complex64
        out = conv.convolve(*[torch.from_numpy(f).to(dt).cuda() for f in fs])
        torch.cuda.synchronize()
        got = out[0].cpu().numpy().astype(np.complex128)
    finally:
        dist.destroy_process_group()
    assert rel_l2(got, want) <= (1e-13 if prec == "f64" else 2e-6)
