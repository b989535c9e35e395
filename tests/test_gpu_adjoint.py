"""GPU: the differentiable 2D advection Jacobian (torch.autograd.Function
over the hand-written adjoint convolution) against central finite
differences and against a reference gradient assembled from FP64 forward
convolutions of the CPU oracle."""
import numpy as np
import pytest

from oracle import hybrid as H
from oracle.direct import rel_l2

pytestmark = pytest.mark.gpu


def spectra(Lx, Ly, seed, dtype):
    """psi, omega with amplitude |k|^-2 (0 at k=0) and uniform random
    phases, Hermitian-symmetrised on the k_y = 0 column."""
    import torch
    Hy = (Ly + 1) // 2
    rng = np.random.default_rng(seed)
    kx = (np.arange(Lx) - Lx // 2)[:, None]
    ky = np.arange(Hy)[None, :]
    k2 = (kx ** 2 + ky ** 2).astype(float)
    amp = np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0)
    out = []
    for _ in range(2):
        f = amp * np.exp(2j * np.pi * rng.uniform(size=(Lx, Hy)))
        H.hermitian_symmetrize_x(f, (Lx + 1) // 2, Hy, Lx // 2)
        out.append(torch.from_numpy(f).to(dtype).cuda())
    return out


def test_adjoint_convolution_parity(native_lib):
    """The A=5, B=4 adjoint convolution matches the oracle."""
    import torch
    from fftwpp_gb300.gpu import HybridConvolution
    kinds, L = [H.CENTERED, H.HERMITIAN], [15, 15]
    M = [H.default_M(k, l) for k, l in zip(kinds, L)]
    rng = np.random.default_rng(8)
    fs = [rng.uniform(-1, 1, (15, 8)) + 1j * rng.uniform(-1, 1, (15, 8))
          for _ in range(5)]
    want = H.convolve(fs, kinds, L, M, mult="realjacadj", B=4)
    conv = HybridConvolution(kinds, L, M, A=5, B=4, mult="realjacadj")
    got = conv.convolve(*[torch.from_numpy(f).cuda() for f in fs])
    for g, w in zip(got, want):
        assert rel_l2(g.cpu().numpy(), w) <= 1e-13


def _loss(op, psi, omega):
    J = op(psi, omega)
    return (J.real ** 2 + J.imag ** 2).sum()


def test_finite_differences(native_lib):
    """Directional derivatives of loss = sum |J|^2 along 64 random
    directions: autograd vs central differences (h = 1e-6, FP64)."""
    import torch
    from fftwpp_gb300.autograd import AdvectionJacobian
    Lx = Ly = 31
    op = AdvectionJacobian(Lx, Ly, "f64")
    psi, omega = spectra(Lx, Ly, 3, torch.complex128)
    psi.requires_grad_(True)
    omega.requires_grad_(True)
    loss = _loss(op, psi, omega)
    gp, go = torch.autograd.grad(loss, (psi, omega))
    rng = np.random.default_rng(17)
    h = 1e-6
    worst = 0.0
    with torch.no_grad():
        for _ in range(64):
            vp = torch.from_numpy(rng.normal(size=psi.shape) +
                                  1j * rng.normal(size=psi.shape)).cuda()
            vo = torch.from_numpy(rng.normal(size=psi.shape) +
                                  1j * rng.normal(size=psi.shape)).cuda()
            vp *= psi.abs().max()
            vo *= omega.abs().max()
            lp = _loss(op, psi + h * vp, omega + h * vo)
            lm = _loss(op, psi - h * vp, omega - h * vo)
            fd = float((lp - lm) / (2 * h))
            an = float((torch.conj(gp) * vp).real.sum() +
                       (torch.conj(go) * vo).real.sum())
            worst = max(worst, abs(fd - an) / max(abs(an), 1e-300))
    assert worst <= 1e-6, worst


def test_reference_gradient(native_lib):
    """The adjoint equals the gradient assembled from FP64 forward
    convolutions of the CPU oracle:
    dL/da0 = w . P(T(a3) T(G/w)) etc., then the chain through i k."""
    import torch
    from fftwpp_gb300.autograd import AdvectionJacobian
    Lx = Ly = 63
    op = AdvectionJacobian(Lx, Ly, "f64")
    psi, omega = spectra(Lx, Ly, 4, torch.complex128)
    psi.requires_grad_(True)
    omega.requires_grad_(True)
    J = op(psi, omega)
    loss = (J.real ** 2 + J.imag ** 2).sum()
    gp, go = torch.autograd.grad(loss, (psi, omega))

    kinds, L = [H.CENTERED, H.HERMITIAN], [Lx, Ly]
    M = [H.default_M(k, l) for k, l in zip(kinds, L)]
    Hy = (Ly + 1) // 2
    kx = (np.arange(Lx) - Lx // 2)[:, None] * np.ones((1, Hy))
    ky = np.ones((Lx, 1)) * np.arange(Hy)[None, :]
    p, o = psi.detach().cpu().numpy(), omega.detach().cpu().numpy()
    a = [1j * kx * p, 1j * ky * p, 1j * kx * o, 1j * ky * o]
    Jr = H.convolve(a, kinds, L, M, mult="realjacobian")[0]
    assert rel_l2(J.detach().cpu().numpy(), Jr) <= 1e-13
    G = 2 * Jr
    w = np.ones((Lx, Hy))
    w[:, 1:] = 2.0
    Gw = G / w

    def conv(u):
        return w * H.convolve([u, Gw], kinds, L, M, mult="realbinary")[0]

    g0, g1, g2, g3 = conv(a[3]), -conv(a[2]), -conv(a[1]), conv(a[0])
    ref_p = -1j * kx * g0 - 1j * ky * g1
    ref_o = -1j * kx * g2 - 1j * ky * g3
    assert rel_l2(gp.cpu().numpy(), ref_p) <= 1e-12
    assert rel_l2(go.cpu().numpy(), ref_o) <= 1e-12


def test_fp32_gradient_close_to_fp64(native_lib):
    import torch
    from fftwpp_gb300.autograd import AdvectionJacobian
    Lx = Ly = 63
    grads = {}
    for prec, dt in (("f64", torch.complex128), ("f32", torch.complex64)):
        op = AdvectionJacobian(Lx, Ly, prec)
        psi, omega = spectra(Lx, Ly, 5, dt)
        psi.requires_grad_(True)
        omega.requires_grad_(True)
        loss = _loss(op, psi, omega)
        grads[prec] = [g.detach().cpu().numpy().astype(np.complex128)
                       for g in torch.autograd.grad(loss, (psi, omega))]
    for g32, g64 in zip(grads["f32"], grads["f64"]):
        assert rel_l2(g32, g64) <= 1e-5


def test_float_float_gradient_matches_fp64(native_lib):
    """The float-float mode (FP64 tensors, hi+lo float arithmetic) gives the
    FP64 gradient to FP64-grade accuracy."""
    import torch
    from fftwpp_gb300.autograd import AdvectionJacobian
    Lx = Ly = 63
    grads = {}
    for prec in ("f64", "ff"):
        op = AdvectionJacobian(Lx, Ly, prec)
        assert op.dtype == torch.complex128
        psi, omega = spectra(Lx, Ly, 6, torch.complex128)
        psi.requires_grad_(True)
        omega.requires_grad_(True)
        loss = _loss(op, psi, omega)
        grads[prec] = [g.detach().cpu().numpy()
                       for g in torch.autograd.grad(loss, (psi, omega))]
    for gff, g64 in zip(grads["ff"], grads["f64"]):
        assert rel_l2(gff, g64) <= 1e-12


@pytest.mark.parametrize("precision", ["f64", "ff", "f32"])
def test_graphed_loss_step(native_lib, precision):
    """The CUDA-graph training step (forward, loss, adjoint backward in one
    replay) gives the eager autograd loss and gradients, and recomputes
    from new values written into its static inputs."""
    import torch
    from fftwpp_gb300.autograd import AdvectionJacobian, GraphedLossStep
    Lx = Ly = 63
    op = AdvectionJacobian(Lx, Ly, precision)
    dt = op.dtype
    psi, omega = spectra(Lx, Ly, 5, dt)
    p2, o2 = spectra(Lx, Ly, 6, dt)

    def eager(p, o):
        p = p.detach().requires_grad_(True)
        o = o.detach().requires_grad_(True)
        loss = _loss(op, p, o)
        gp, go = torch.autograd.grad(loss, (p, o))
        return loss.detach(), gp, go

    step = GraphedLossStep(op, psi.clone(), omega.clone())
    for p, o in ((psi, omega), (p2, o2)):
        step.set_inputs(p, o)
        got = [t.clone() for t in step()]
        want = eager(p, o)
        torch.cuda.synchronize()
        for g, w in zip(got, want):
            assert torch.equal(g, w)
