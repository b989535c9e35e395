"""GPU: standalone padded transforms (fgb_pad_*, PaddedTransform) against
the forward residue layouts the reference itself produced
(tests/golden/layouts.npz, made by FFTW++'s fftPad/fftPadCentered forward)
and against explicit padded DFTs; backward(forward(f)) = N f at large
sizes."""
import os

import numpy as np
import pytest

from oracle import hybrid as H
from oracle.direct import rel_l2

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _smooth(n):
    for f in (2, 3, 5, 7):
        while n % f == 0:
            n //= f
    return n == 1


def _layouts():
    data = np.load(os.path.join(GOLD, "layouts.npz"))
    for line in open(os.path.join(GOLD, "layouts.txt")):
        if line.startswith("#"):
            continue
        key, kind, L, M, m, D, I = line.split()
        yield (key, int(kind), int(L), int(M), data[key + "_F"],
               data[key + "_idx"], data[key + "_info"])


def test_forward_matches_reference_layouts(native_lib):
    """Every value the reference's forward transform emitted, looked up by
    its transformed index in the GPU's residue-major output."""
    import torch
    from fftwpp_gb300.gpu import PaddedTransform
    checked = 0
    seen = set()
    for key, kind, L, M, F, idx, info in _layouts():
        m, N = int(info[0]), int(info[7])
        if not _smooth(m) or (kind, L, M, m) in seen:
            continue
        seen.add((kind, L, M, m))
        t = PaddedTransform(kind, L, M, m=m)
        assert t.N == N and t.m == m, key
        f = (np.arange(L) + 1) + 1j * (np.arange(L) + 2)
        got = t.forward(torch.from_numpy(f).cuda()).cpu().numpy()[:, 0]
        r, j = idx % t.q, idx // t.q
        assert rel_l2(got[r * t.m + j], F) <= 1e-13, key
        assert all(t.index(int(a), int(b)) == int(k)
                   for a, b, k in zip(r[:5], j[:5], idx[:5]))
        checked += 1
    assert checked >= 40


def _explicit(kind, f, N, c):
    """Explicit padded DFT (sign +1) of the columns of f."""
    L = f.shape[0]
    s = np.arange(L)
    k = np.arange(N if kind != H.REAL else N // 2 + 1)
    E = np.exp(2j * np.pi * (np.outer(k, s - c) % N) / N)
    return E @ f


CASES = [(H.PAD, 100, 199, 7, 0), (H.PAD, 1000, 1999, 3, 0),
         (H.PAD, 96, 191, 5, 32), (H.CENTERED, 63, 94, 4, 0),
         (H.CENTERED, 127, 190, 9, 0), (H.CENTERED, 64, 96, 2, 16),
         (H.REAL, 100, 199, 6, 0), (H.REAL, 255, 510, 3, 0)]


@pytest.mark.parametrize("precision,tol", [("f64", 1e-13), ("f32", 2e-6)])
@pytest.mark.parametrize("kind,L,M,C,m", CASES)
def test_forward_backward_explicit(native_lib, kind, L, M, C, m, precision,
                                   tol):
    import torch
    from fftwpp_gb300.gpu import PaddedTransform
    t = PaddedTransform(kind, L, M, C=C, m=m, precision=precision)
    rng = np.random.default_rng(L + C)
    if kind == H.REAL:
        f = rng.normal(size=(L, C))
    else:
        f = rng.uniform(-1, 1, (L, C)) + 1j * rng.uniform(-1, 1, (L, C))
    F = t.forward(torch.from_numpy(f).to(t.idtype).cuda())
    want = _explicit(kind, f, t.N, t.cshift)
    got = F.cpu().numpy().astype(np.complex128)
    if kind == H.REAL:
        assert rel_l2(got, want) <= tol
    else:
        rows = np.array([t.index(r, j) for r in range(t.q)
                         for j in range(t.m)])
        assert rel_l2(got, want[rows]) <= tol
    # Backward: the unnormalised adjoint of a random spectrum.
    G = rng.uniform(-1, 1, got.shape) + 1j * rng.uniform(-1, 1, got.shape)
    if kind == H.REAL:
        G[0] = G[0].real
        if t.N % 2 == 0:
            G[-1] = G[-1].real
    g = t.backward(torch.from_numpy(G).to(t.cdtype).cuda()).cpu().numpy()
    s = np.arange(L) - t.cshift
    if kind == H.REAL:
        k = np.arange(t.N // 2 + 1)
        w = np.where((k == 0) | (2 * k == t.N), 1.0, 2.0)
        E = np.exp(-2j * np.pi * (np.outer(s, k) % t.N) / t.N)
        wantb = (E @ (w[:, None] * G)).real
    else:
        kk = rows
        E = np.exp(-2j * np.pi * (np.outer(s, kk) % t.N) / t.N)
        wantb = E @ G
    assert rel_l2(g.astype(wantb.dtype), wantb) <= tol


@pytest.mark.parametrize("kind,L,C", [(H.PAD, 8192, 64), (H.CENTERED, 4095, 48),
                                      (H.REAL, 4096, 64)])
def test_roundtrip_large(native_lib, kind, L, C):
    """backward(forward(f)) = N f, a size-independent property."""
    import torch
    from fftwpp_gb300.gpu import PaddedTransform
    t = PaddedTransform(kind, L, C=C)
    rng = np.random.default_rng(1)
    if kind == H.REAL:
        f = torch.from_numpy(rng.normal(size=(L, C))).cuda()
    else:
        f = torch.from_numpy(rng.uniform(-1, 1, (L, C)) +
                             1j * rng.uniform(-1, 1, (L, C))).cuda()
    g = t.backward(t.forward(f))
    err = float(torch.linalg.norm(g / t.N - f) / torch.linalg.norm(f))
    assert err <= 1e-13


def test_rejects_bad_tensors(native_lib):
    import torch
    from fftwpp_gb300.gpu import PaddedTransform
    t = PaddedTransform(H.PAD, 16, C=2)
    with pytest.raises(ValueError):
        t.forward(torch.zeros(16, 3, dtype=torch.complex128, device="cuda"))
    with pytest.raises(ValueError):
        t.forward(torch.zeros(16, 2, dtype=torch.complex64, device="cuda"))


def _hermitian_layouts():
    data = np.load(os.path.join(GOLD, "hlayouts.npz"))
    for line in open(os.path.join(GOLD, "hlayouts.txt")):
        if line.startswith("#"):
            continue
        key, L, M, m, D = line.split()
        yield (key, int(L), int(M), int(m), data[key + "_F"],
               data[key + "_idx"], data[key + "_info"])


def test_hermitian_forward_matches_reference_layouts(native_lib):
    """The standalone Hermitian transform against every real value the
    reference's fftPadHermitian forward produced (tests/hybridh.cc:74-99,
    explicit and hybrid plans), looked up by transformed index, wherever the
    reference's padded length N is even with N/2 a product of 2, 3, 5, 7
    (the GPU's explicit grid is then the same)."""
    import torch
    from fftwpp_gb300.gpu import PaddedTransform
    checked = 0
    for key, L, M, m, F, idx, info in _hermitian_layouts():
        N = int(info[7])
        if N % 2 or not _smooth(N // 2):
            continue
        t = PaddedTransform(H.HERMITIAN, L, N)
        assert t.N == N, key
        Hm = (L + 1) // 2
        f = (np.arange(Hm) + 1) + 1j * (np.arange(Hm) + 2)
        f[0] = 1
        got = t.forward(torch.from_numpy(f).cuda()).cpu().numpy()[:, 0]
        assert rel_l2(got[idx], F) <= 1e-13, key
        assert t.index(0, int(idx[3])) == int(idx[3])
        checked += 1
    assert checked >= 60


@pytest.mark.parametrize("precision,tol", [("f64", 1e-13), ("f32", 2e-6)])
@pytest.mark.parametrize("L,M,C,m", [(15, 22, 1, 0), (63, 94, 5, 0),
                                     (1023, 1534, 3, 0), (31, 46, 2, 8)])
def test_hermitian_forward_backward(native_lib, L, M, C, m, precision, tol):
    """Forward against the explicit oracle on C interleaved columns;
    backward(forward(f)) = N f."""
    import torch
    from fftwpp_gb300.gpu import PaddedTransform
    from oracle import explicit as E
    t = PaddedTransform(H.HERMITIAN, L, M, C=C, m=m, precision=precision)
    assert t.N % 2 == 0 and t.N >= M
    Hm = (L + 1) // 2
    rng = np.random.default_rng(L + C)
    f = rng.uniform(-1, 1, (Hm, C)) + 1j * rng.uniform(-1, 1, (Hm, C))
    f[0] = f[0].real
    tf = torch.from_numpy(f).to(t.idtype).cuda()
    F = t.forward(tf)
    want = E._forward(f.T, E.HERMITIAN, L, t.N, 1).T
    assert rel_l2(F.cpu().numpy().astype(np.float64), want) <= tol
    back = t.backward(F).cpu().numpy().astype(np.complex128)
    assert rel_l2(back, t.N * f) <= tol
