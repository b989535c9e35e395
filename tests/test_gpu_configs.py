"""GPU parity at the sizes of the five benchmark configurations, through
the C ABI of lib_fftwpp.so, against the CPU oracle (the numpy restatement
pinned to the compiled reference) or, where a full oracle run is out of
reach, against FP64 direct sums (tests/direct.h:10-156).

Tolerances (relative L2): 1e-13 in FP64 and float-float, 2e-6 in
FP32-compensated mode; 1e-6 relative for the adjoint against central
differences."""
import os

import numpy as np
import pytest

import bench
from oracle import hybrid as H
from oracle.direct import directconv3_at, rel_l2

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-13, "ff": 1e-13, "f32": 2e-6}
WORKERS = os.cpu_count() or 1


def _gpu(w, fs, precision):
    import torch
    from fftwpp_gb300.gpu import HybridConvolution
    conv = HybridConvolution(w["kinds"], w["L"], w["M"], A=w["A"], B=w["B"],
                             mult=w["mult"], precision=precision)
    ts = [torch.from_numpy(np.ascontiguousarray(f)).to(conv.dtype).cuda()
          for f in fs]
    out = conv.convolve(*ts)[0]
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("precision", ["f64", "ff", "f32"])
def test_hconv2d_full_size_vs_oracle(native_lib, precision):
    """2D centred-Hermitian binary convolution, 1023 x 512 complex128
    modes, Mx = My = 1534, seeded U[-1,1] and Hermitian-symmetrised: the
    benchmark's own inputs against the oracle at full size."""
    w = bench.WORKLOADS["hconv2d"]
    fs = bench.synth_inputs(w, seed=1)
    want = H.convolve(fs, w["kinds"], w["L"], w["M"], mult=w["mult"],
                      workers=WORKERS)[0]
    got = _gpu(w, fs, precision)
    assert rel_l2(got.astype(np.complex128), want) <= TOL[precision]


@pytest.mark.parametrize("precision", ["f64", "ff", "f32"])
def test_real3d_full_size_vs_direct_sums(native_lib, precision):
    """3D real convolution of two 256^3 float64 N(0,1) fields, M = 511 per
    axis: 64 outputs sampled across the whole cube (corners included)
    against FP64 direct sums."""
    w = bench.WORKLOADS["real3d"]
    fs = bench.synth_inputs(w, seed=1)
    got = _gpu(w, fs, precision).astype(np.float64)
    rng = np.random.default_rng(31)
    pts = [tuple(int(x) for x in rng.integers(0, 256, 3)) for _ in range(60)]
    pts += [(0, 0, 0), (255, 255, 255), (255, 0, 128), (17, 255, 3)]
    want = directconv3_at(fs[0], fs[1], pts)
    err = rel_l2(np.array([got[p] for p in pts]), want)
    assert err <= TOL[precision], err


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_batched_512_seeded_lengths(native_lib, precision):
    """The batched workload exactly: 512 lengths drawn log-uniformly in
    [64, 65536] from the benchmark's seed, M = 2L - 1, in one persistent
    launch (direct, then captured and replayed from a CUDA graph), every
    problem against the oracle."""
    import torch
    from fftwpp_gb300.gpu import BatchedConvolution
    Ls = bench.batched_lengths()
    assert len(Ls) == 512 and min(Ls) >= 64 and max(Ls) <= 65536
    conv = BatchedConvolution(Ls, precision=precision, tune=True)
    rng = np.random.default_rng(5)
    f = rng.uniform(-1, 1, conv.total) + 1j * rng.uniform(-1, 1, conv.total)
    g = rng.uniform(-1, 1, conv.total) + 1j * rng.uniform(-1, 1, conv.total)
    tf = torch.from_numpy(f).to(conv.dtype).cuda()
    tg = torch.from_numpy(g).to(conv.dtype).cuda()
    want = [H.convolve([f[o:o + L], g[o:o + L]], [H.PAD], [L], [2 * L - 1])[0]
            for o, L in zip(conv.offsets, conv.L)]
    for graph in (False, True, True):
        out = conv.convolve(tf, tg, graph=graph)[0]
        torch.cuda.synchronize()
        assert conv.error() == 0
        h = out.cpu().numpy().astype(np.complex128)
        worst = max(rel_l2(h[o:o + L], wv)
                    for o, L, wv in zip(conv.offsets, conv.L, want))
        assert worst <= TOL[precision], worst


def _jacobian_inputs(Lx, Ly, seed):
    psi, omega = bench.grad_spectra(Lx, Ly, seed)
    kx = (np.arange(Lx) - Lx // 2)[:, None]
    ky = np.arange((Ly + 1) // 2)[None, :]
    return [1j * kx * psi, 1j * ky * psi, 1j * kx * omega, 1j * ky * omega]


@pytest.mark.parametrize("precision", ["f64", "ff", "f32"])
def test_jacobian_full_size_vs_oracle(native_lib, precision):
    """The advection Jacobian at its benchmark size: four centred-Hermitian
    inputs (i kx psi, i ky psi, i kx omega, i ky omega) on 1023 x 512 modes
    with |k|^-2 spectra and random phases, 2/3-rule padding M = 1534."""
    w = bench.WORKLOADS["jacobian2d"]
    fs = _jacobian_inputs(1023, 1023, seed=11)
    want = H.convolve(fs, w["kinds"], w["L"], w["M"], mult=w["mult"],
                      workers=WORKERS)[0]
    got = _gpu(w, fs, precision)
    assert rel_l2(got.astype(np.complex128), want) <= TOL[precision]


def test_adjoint_full_size_central_differences(native_lib):
    """The hand-written adjoint at the benchmark size (1023 x 512 modes,
    FP64): autograd's directional derivatives of loss = sum |J|^2 against
    central differences (h = 1e-6) along 8 directions shaped like the
    |k|^-2 spectra, and the gradient against the oracle's FP64 gradient
    (forward and adjoint convolutions of the restatement)."""
    import torch
    from fftwpp_gb300.autograd import AdvectionJacobian
    Lx = Ly = 1023
    op = AdvectionJacobian(Lx, Ly, precision="f64")
    p0, o0 = bench.grad_spectra(Lx, Ly, seed=11)
    psi = torch.from_numpy(p0).cuda().requires_grad_(True)
    omega = torch.from_numpy(o0).cuda().requires_grad_(True)

    def loss_of(p, o):
        J = op(p, o)
        return (J.real ** 2 + J.imag ** 2).sum()
    gp, go = torch.autograd.grad(loss_of(psi, omega), (psi, omega))
    _, wp, wo = bench.oracle_grad_step(p0, o0, Lx, Ly, WORKERS)
    num = (np.linalg.norm(gp.cpu().numpy() - wp) ** 2 +
           np.linalg.norm(go.cpu().numpy() - wo) ** 2)
    den = np.linalg.norm(wp) ** 2 + np.linalg.norm(wo) ** 2
    assert (num / den) ** 0.5 <= 1e-12
    rng = np.random.default_rng(17)
    kx = (np.arange(Lx) - Lx // 2)[:, None]
    ky = np.arange((Ly + 1) // 2)[None, :]
    k2 = (kx ** 2 + ky ** 2).astype(float)
    amp = np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0)
    h, worst = 1e-6, 0.0
    with torch.no_grad():
        for _ in range(8):
            vp = torch.from_numpy(amp * (rng.normal(size=p0.shape) + 1j *
                                         rng.normal(size=p0.shape))).cuda()
            vo = torch.from_numpy(amp * (rng.normal(size=p0.shape) + 1j *
                                         rng.normal(size=p0.shape))).cuda()
            fd = float((loss_of(psi + h * vp, omega + h * vo) -
                        loss_of(psi - h * vp, omega - h * vo)) / (2 * h))
            an = float((torch.conj(gp) * vp).real.sum() +
                       (torch.conj(go) * vo).real.sum())
            worst = max(worst, abs(fd - an) / abs(an))
    assert worst <= 1e-6, worst
