"""Differentiable 2D pseudo-spectral advection term on the GB300 engine.

J(psi, omega) = psi_x omega_y - psi_y omega_x, computed as a dealiased
centred-Hermitian convolution with four inputs (i kx psi, i ky psi,
i kx omega, i ky omega) and the physical-space Jacobian multiplier
(FFTW++ Convolution2 over fftPadCentered x fftPadHermitian with a custom
multiplier, convolve.h:1269-1548; multiplier hook convolve.h:78-79).

Backward (hand-written adjoint, recomputing the padded transforms instead of
storing them).  With the forward complex-to-real transform
T(a)(x) = Re sum_k w_k a_k e^{ik.x}  (w = 1 on the k_y = 0 column, 2 elsewhere)
and the normalised real-to-complex transform P of the convolution, the
adjoints for the real inner product Re <a, b> on the stored modes are
P* = T(. / w) / N and T* = N w . P, so for J = P(T(a0)T(a3) - T(a1)T(a2))
and an output cotangent G (PyTorch's convention dL/dRe + i dL/dIm):

    dL/da0 =  w . P(T(a3) T(G/w)),   dL/da3 =  w . P(T(a0) T(G/w)),
    dL/da1 = -w . P(T(a2) T(G/w)),   dL/da2 = -w . P(T(a1) T(G/w)).

That is one more dealiased convolution: five inputs (a0..a3, G/w), four
outputs and the Jacobian-adjoint multiplier -- the gradient of a bilinear
dealiased convolution is itself a dealiased convolution (a correlation in
spectral space).
"""
from __future__ import annotations

import ctypes

import torch

from . import _native
from .gpu import CENTERED, HERMITIAN, HybridConvolution

__all__ = ["AdvectionJacobian", "GraphedLossStep", "wavenumbers"]


def wavenumbers(Lx: int, Ly: int, device=None, dtype=torch.float64):
    """kx (centred, index i <-> i - floor(Lx/2)) and ky (0..ceil(Ly/2)-1)
    grids of the stored Lx x ceil(Ly/2) modes."""
    Hy = (Ly + 1) // 2
    kx = (torch.arange(Lx, device=device, dtype=dtype) - Lx // 2)[:, None]
    ky = torch.arange(Hy, device=device, dtype=dtype)[None, :]
    return kx.expand(Lx, Hy), ky.expand(Lx, Hy)


class _Jacobian(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a0, a1, a2, a3, op):
        ctx.op = op
        ctx.save_for_backward(a0, a1, a2, a3)
        return op.fwd.convolve(a0, a1, a2, a3)[0]

    @staticmethod
    def backward(ctx, G):
        op = ctx.op
        a0, a1, a2, a3 = ctx.saved_tensors
        g = G.contiguous().clone()
        op.scale_columns(g, 1.0, 0.5)          # G / w
        outs = op.adj.convolve(a0, a1, a2, a3, g)
        for o in outs:
            op.scale_columns(o, 1.0, 2.0)      # w . P(...)
        return outs[0], outs[1], outs[2], outs[3], None


class AdvectionJacobian:
    """J(psi, omega) on Lx x ceil(Ly/2) centred-Hermitian modes with the
    2/3-rule padding M = 3 ceil(L/2) - 2 (L mod 2) on both axes.
    precision: "f64", "ff" (FP64 tensors, float-float arithmetic) or
    "f32"."""

    def __init__(self, Lx: int, Ly: int, precision: str = "f64"):
        self.Lx, self.Ly = Lx, Ly
        self.precision = precision
        kinds = [CENTERED, HERMITIAN]
        self.fwd = HybridConvolution(kinds, [Lx, Ly], A=4, B=1,
                                     mult="realjacobian", precision=precision)
        self.adj = HybridConvolution(kinds, [Lx, Ly], A=5, B=4,
                                     mult="realjacadj", precision=precision)
        self.lib = _native.load()
        self.shape = self.fwd.shape
        self.dtype = self.fwd.dtype

    def scale_columns(self, t, s0, s1):
        rows, cols = t.shape
        s = torch.cuda.current_stream()
        # The float-float mode keeps FP64 data: scale it as FP64.
        data = _native.F32 if self.fwd.prec == _native.F32 else _native.F64
        rc = self.lib.fgb_scale_columns_device(
            rows, cols, s0, s1, ctypes.c_void_p(t.data_ptr()),
            data, ctypes.c_void_p(s.cuda_stream))
        if rc != 0:
            raise RuntimeError(_native.last_error())

    def jacobian(self, a0, a1, a2, a3):
        """Differentiable J from the four derivative fields."""
        return _Jacobian.apply(a0.contiguous(), a1.contiguous(),
                               a2.contiguous(), a3.contiguous(), self)

    def __call__(self, psi, omega):
        """J(psi, omega) from the two spectra (derivatives formed here)."""
        kx, ky = wavenumbers(self.Lx, self.Ly, psi.device,
                             psi.real.dtype)
        ikx = 1j * kx
        iky = 1j * ky
        return self.jacobian(ikx * psi, iky * psi, ikx * omega, iky * omega)


def _sum_sq(J):
    return (J.real ** 2 + J.imag ** 2).sum()


class GraphedLossStep:
    """A training step (J from psi and omega, loss, gradients) captured
    once in a CUDA graph and replayed: the forward Jacobian convolution,
    the loss, the adjoint convolution and the chain rule run as one graph
    launch, without the per-operation launch cost of eager autograd.

    psi and omega are the static input tensors (CUDA, the operator's dtype):
    give new values with set_inputs() between calls (they are leaves that
    require grad, so a plain copy_ into step.psi outside torch.no_grad()
    raises).  Each call returns the static (loss, dL/dpsi, dL/domega)
    tensors, overwritten by the next call.  loss_fn maps J to a scalar
    (default: sum |J|^2)."""

    def __init__(self, op: AdvectionJacobian, psi, omega, loss_fn=None):
        if psi.dtype != op.dtype or omega.dtype != op.dtype:
            raise ValueError(f"psi and omega must be {op.dtype} tensors")
        loss_fn = loss_fn or _sum_sq
        self.psi = psi.detach().requires_grad_(True)
        self.omega = omega.detach().requires_grad_(True)

        def body():
            loss = loss_fn(op(self.psi, self.omega))
            gp, go = torch.autograd.grad(loss, (self.psi, self.omega))
            return loss.detach(), gp, go

        # Warm-up on a side stream (allocator pools, plan caches), then
        # capture on it.
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(3):
                body()
        torch.cuda.current_stream().wait_stream(side)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.out = body()

    def set_inputs(self, psi=None, omega=None):
        """Copy new spectra into the captured input tensors (either may be
        None to keep its current values)."""
        with torch.no_grad():
            if psi is not None:
                self.psi.copy_(psi)
            if omega is not None:
                self.omega.copy_(omega)

    def __call__(self):
        self.graph.replay()
        return self.out

