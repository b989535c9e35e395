"""CPU: the gradient step the benchmark's CPU arms time for the
differentiable Jacobian (bench.oracle_grad_step: forward Jacobian and
adjoint convolutions of the oracle, chain rule in numpy) gives the
directional derivatives of loss = sum |J|^2 by central differences."""
import numpy as np

import bench
from oracle import hybrid as H


def _loss(psi, omega, L):
    kinds = [H.CENTERED, H.HERMITIAN]
    M = [H.default_M(k, l) for k, l in zip(kinds, [L, L])]
    Hy = (L + 1) // 2
    kx = (np.arange(L) - L // 2)[:, None]
    ky = np.arange(Hy)[None, :]
    a = [1j * kx * psi, 1j * ky * psi, 1j * kx * omega, 1j * ky * omega]
    J = H.convolve(a, kinds, [L, L], M, mult="realjacobian")[0]
    return float(np.sum(np.abs(J) ** 2))


def test_oracle_grad_step_matches_central_differences():
    L = 9
    psi, omega = bench.grad_spectra(L, L, seed=3)
    loss, gp, go = bench.oracle_grad_step(psi, omega, L, L, 1)
    assert abs(loss - _loss(psi, omega, L)) <= 1e-12 * loss
    rng = np.random.default_rng(4)
    h = 1e-6
    for _ in range(8):
        vp = rng.normal(size=psi.shape) + 1j * rng.normal(size=psi.shape)
        vo = rng.normal(size=psi.shape) + 1j * rng.normal(size=psi.shape)
        fd = (_loss(psi + h * vp, omega + h * vo, L) -
              _loss(psi - h * vp, omega - h * vo, L)) / (2 * h)
        an = float(np.sum((np.conj(gp) * vp).real) +
                   np.sum((np.conj(go) * vo).real))
        assert abs(fd - an) <= 1e-6 * abs(an)
