"""CPU oracle: explicitly zero-padded convolutions on a given padded grid,
with a multiplier that may depend on the grid position.

TEST INFRASTRUCTURE ONLY (imported by tests/ as the checker).

The reference calls its multiplier on blocks of the padded transforms and
tells it, through Indices and fftBase::index (convolve.h:48-82, 297-326),
where on the padded grid each value lies.  A multiplier that depends on
that position gives a result that depends on the padded lengths N (not on
the residue decomposition m, q), so the checker for such multipliers is
the explicit transform on the same N grid: every axis zero-padded to N and
transformed with the FFTW++ sign conventions of its kind --

* fftPad:         F[k] = sum_{s<L} f[s] w^{s k},       w = exp(2 pi i/N)
* fftPadCentered: F[k] = sum_{s<L} f[s] w^{(s-c) k},   c = floor(L/2)
* fftPadHermitian (innermost axis): the ceil(L/2) stored modes, Hermitian
  extended, to N real values u[t] = sum_k f_k w^{k t} (the multiplier sees
  real values, as realMultBinary does, convolve.cc:60-83)
* fftPadReal (outermost axis): real data to the N/2+1 modes
  F[k] = sum_s f[s] w^{s k}, k = 0..N/2

-- and back with the conjugate transforms, keeping the stored entries and
normalising by 1/prod(N) (Convolution::convolve, convolve.h:1157-1160).
For a position-independent multiplier it equals the hybrid result for any
N >= M (tests pin this against oracle.hybrid).
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np

PAD, CENTERED, HERMITIAN, REAL = 0, 1, 2, 3


def _stored(kind: int, L: int) -> int:
    return (L + 1) // 2 if kind == HERMITIAN else L


def _forward(f: np.ndarray, kind: int, L: int, N: int, axis: int):
    if kind == HERMITIAN:
        g = np.zeros(f.shape[:-1] + (N // 2 + 1,), dtype=np.complex128)
        g[..., :f.shape[-1]] = f
        return np.fft.irfft(g, n=N, axis=-1) * N
    if kind == REAL:
        return np.conj(np.fft.rfft(f.real, n=N, axis=axis))
    shape = list(f.shape)
    shape[axis] = N
    g = np.zeros(shape, dtype=np.complex128)
    idx = [slice(None)] * f.ndim
    idx[axis] = slice(0, L)
    g[tuple(idx)] = f
    if kind == CENTERED:
        g = np.roll(g, -(L // 2), axis=axis)
    return np.fft.ifft(g, axis=axis) * N


def _backward(F: np.ndarray, kind: int, L: int, N: int, axis: int):
    if kind == HERMITIAN:
        return np.fft.rfft(F.real, axis=-1)[..., :_stored(kind, L)]
    if kind == REAL:
        h = np.fft.irfft(np.conj(F), n=N, axis=axis) * N
        return np.take(h, np.arange(L), axis=axis)
    h = np.fft.fft(F, axis=axis)
    s = np.arange(L)
    if kind == CENTERED:
        s = (s - L // 2) % N
    return np.take(h, s, axis=axis)


def convolve(inputs: Sequence[np.ndarray], kinds: Sequence[int],
             Ls: Sequence[int], Ns: Sequence[int],
             mult: Callable[[list, tuple], list], *,
             normalize: bool = True) -> list[np.ndarray]:
    """mult(values, index) receives the A transformed inputs on the padded
    grid (complex arrays, real ones when the innermost axis is Hermitian)
    and index, one integer grid per axis (the transformed index of every
    point, outermost first); it returns the B products."""
    dim = len(kinds)
    fs = [np.asarray(f).astype(np.complex128) for f in inputs]
    for d in range(dim):
        fs = [_forward(f, kinds[d], Ls[d], Ns[d], d) for f in fs]
    index = np.meshgrid(*[np.arange(n) for n in fs[0].shape],
                        indexing="ij")
    hs = mult(fs, tuple(index))
    for d in reversed(range(dim)):
        hs = [_backward(h, kinds[d], Ls[d], Ns[d], d) for h in hs]
    scale = 1.0 / np.prod([float(n) for n in Ns]) if normalize else 1.0
    out = []
    for h in hs:
        h = h * scale
        out.append(h.real.copy() if kinds[0] == REAL else h)
    return out
