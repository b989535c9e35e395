"""CPU oracle: a numpy restatement of FFTW++'s hybrid dealiased convolution.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by ``__graft_entry__.smoke()``
and by the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py``, and
only as the checker or the timed CPU baseline -- never by the GPU product
(``fftwpp_gb300``), which must fail loudly when its CUDA library is missing.

What it restates (reference = FFTW++ ``convolve.h`` / ``convolve.cc``):

* the parameter rules ``fftBase::parameters`` (convolve.cc:403-410),
  ``nextfftsize`` (convolve.cc:114-124), ``nextpuresize``/``ispure``
  (convolve.cc:144-175) and the four ``valid()`` predicates
  (convolve.h:482-485, 605-607, 721-723, 833-836);
* the transformed-index maps ``fftBase::index`` (convolve.h:297-326) and
  ``fftPadReal::index`` (convolve.h:956-979);
* the residue-decomposed padded transforms.  For a padded length N = m*q and
  residue r the forward block is
      F_r[j] = sum_{s<L} f[s] w_N^{s(qj+r)},     w_N = exp(+2 pi i/N),
  evaluated as the reference does it (fftPad::forwardInner,
  convolve.cc:1227-1327): fold the p length-m blocks with w_q^{ur}, apply the
  pre-twiddle w_N^{sr} (Zetaqm, convolve.cc:126-140), then an m-point DFT with
  FFTW sign +1.  The backward block inverts each step with conjugate twiddles
  and accumulates over residues (fftPad::backwardInner, convolve.cc:1765-1850);
* the centred variant (fftPadCentered, convolve.cc:1967-2110): data index s
  carries wavenumber s - floor(L/2), i.e. an extra phase w_N^{-floor(L/2) k};
* the Hermitian variant (fftPadHermitian, convolve.cc:4309-5448): the
  ceil(L/2) stored modes k >= 0 are Hermitian-extended to 2H-1 centred modes,
  transformed to real physical space (complex-to-real), and the multiplier
  acts on doubles (realMultBinary, convolve.cc:60-83);
* the real variant (fftPadReal, convolve.cc:5449-7484): real data in, real
  data out;
* the drivers ``Convolution::convolveRaw`` (convolve.cc:7513-7575),
  ``Convolution2::convolveRaw`` (convolve.h:1475-1535) and
  ``Convolution3::convolveRaw`` (convolve.h:1812-1879): loop over the outer
  residues, forward all A inputs, run the inner sub-convolution on every
  transformed row, backward the B outputs with accumulation, and normalise
  by 1/prod(m*q);
* the multipliers multBinary / realMultBinary / multcorrelation
  (convolve.cc:33-110) plus the physical-space Jacobian used by the 2D
  advection workload.

The result of a dealiased convolution does not depend on (m, p, q) once
m*q >= M >= the dealiasing bound, so the oracle accepts any m; by default it
uses the reference's explicit choice m = M (q = 1) unless one is given.
"""
from __future__ import annotations

import math
from typing import Callable, Sequence

import numpy as np

try:  # scipy.fft is multi-threaded through ``workers``; numpy is the fallback
    import scipy.fft as _sfft

    def _fft(x, axis, workers):
        return _sfft.fft(x, axis=axis, workers=workers)

    def _ifft_unscaled(x, axis, workers):
        return _sfft.ifft(x, axis=axis, norm="forward", workers=workers)
except ImportError:  # pragma: no cover
    def _fft(x, axis, workers):
        return np.fft.fft(x, axis=axis)

    def _ifft_unscaled(x, axis, workers):
        return np.fft.ifft(x, axis=axis, norm="forward")

PAD, CENTERED, HERMITIAN, REAL = 0, 1, 2, 3
KIND_NAMES = {PAD: "pad", CENTERED: "centered", HERMITIAN: "hermitian",
              REAL: "real"}

WORKERS = 1


# ---------------------------------------------------------------------------
# Integer helpers (convolve.cc:114-175, utils.h).

def ceilquotient(a: int, b: int) -> int:
    return (a + b - 1) // b


def ceilpow2(n: int) -> int:
    p = 1
    while p < n:
        p <<= 1
    return p


def ceilpow(base: int, n: int) -> int:
    p = 1
    while p < n:
        p *= base
    return p


def nextfftsize(m: int) -> int:
    """Smallest 2^a 3^b 5^c 7^d >= m (convolve.cc:114-124)."""
    N = ceilpow2(m)
    if m == N:
        return m
    ni = 1
    while ni < N:
        nj = ni
        while nj < N:
            nk = nj
            while nk < N:
                N = min(N, nk * ceilpow2(ceilquotient(m, nk)))
                nk *= 3
            nj *= 5
        ni *= 7
    return N


def nextpuresize(m: int) -> int:
    """Smallest power of 2, 3, 5 or 7 >= m (convolve.cc:144-157)."""
    M = ceilpow2(m)
    if m == M:
        return m
    M = min(M, ceilpow(3, m))
    if m == M:
        return m
    M = min(M, ceilpow(5, m))
    if m == M:
        return m
    return min(M, ceilpow(7, m))


def ispure(m: int) -> bool:
    """m is a power of 2, 3, 5 or 7 (convolve.cc:159-175)."""
    return any(m == ceilpow(b, m) for b in (2, 3, 5, 7))


def parameters(L: int, M: int, m: int, centered: bool):
    """(p, n, q) for padding L values to >= M with block size m
    (fftBase::parameters, convolve.cc:403-410)."""
    p = ceilquotient(L, m)
    P = p // 2 if ((centered and p % 2 == 0) or p == 2) else p
    n = ceilquotient(M, P * m)
    return p, n, P * n


def valid_pad(m, p, q, n, D, S):
    """fftPad::valid (convolve.h:482-485)."""
    if q == 1:
        return D == 1
    return D == 1 or (S == 1 and ((D < n and D % 2 == 0) or D == n))


def valid_centered(m, p, q, n, D, S):
    """fftPadCentered::Opt::valid (convolve.h:605-607)."""
    return (q == 1 or p % 2 == 0) and valid_pad(m, p, q, n, D, S)


def valid_hermitian(m, p, q, n, D, C):
    """fftPadHermitian::Opt::valid (convolve.h:721-723)."""
    return (D == 1 and q == 1) or (D == 2 and p % 2 == 0 and (p == 2 or C == 1))


def valid_real(m, p, q, n, D, S):
    """fftPadReal::Opt::valid (convolve.h:833-836)."""
    return ((n % 2 == 1 or (p % 2 == 0 or p <= 2)) and (q % 2 == 1 or m % 2 == 0)
            and (D == 1 or (S == 1 and ((D < (n - 1) // 2 and D % 2 == 0)
                                        or D == (n - 1) // 2))))


# ---------------------------------------------------------------------------
# Transformed-index maps (layout of every residue block).

def index_base(r: int, i: int, *, m, p, q, n, D, D0, centered, overwrite=False):
    """fftBase::index (convolve.h:297-326)."""
    if q == 1:
        return i
    P = ceilquotient(p, 2)
    if overwrite and centered and r == 2:
        if i < m:
            i = (i - 1) % m
        if p > 2:
            i = (i + m) % (P * m)
    s = i % m
    if D > 1 and ((centered and p % 2 == 0) or p <= 2):
        u = (i // m) % P
        offset = 1 if (r == 0 and i >= P * m and D0 % 2 == 1) else 0
        incr = (i + P * m * offset) // (2 * P * m)
        r += incr
        if i // (P * m) - 2 * incr + offset == 1:
            if (not centered and p == 2) or (r > 0 and u == 0):
                s = s - 1 if s > 0 else m - 1
            if r == 0:
                r = n // 2
            else:
                r = n - r
                u = u - 1 if u > 0 else P - 1
    else:
        u = (i // m) % p
        r += i // (p * m)
    return q * s + n * u + r


def index_real(r: int, i: int, *, m, p, q, n):
    """fftPadReal::index (convolve.h:956-979)."""
    if q == 1:
        return i
    s = i % m
    P = 1 if p == 2 else p
    r += i // (P * m)
    if p <= 2:
        if r == 0:
            return q * i
        if 2 * r == q:
            return q * m - (q * 2 * i + r)
    else:
        u = (i // m) % p
        if r == 0:
            if 2 * u == p:
                return q * m - (q * 2 * s + u * n)
            return u * n if s == 0 else q * m - (q * s - u * n)
        if 2 * r == n:
            return q * m - (q * s + 2 * u * n + r)
        return q * (m - s) - (u * n + r)
    return q * (m - s) - r


# ---------------------------------------------------------------------------
# Residue-decomposed padded transforms along one axis.

def _roots(N: int, e: np.ndarray) -> np.ndarray:
    """exp(2 pi i e/N) with the exponent reduced mod N first."""
    return np.exp(2j * np.pi * (np.asarray(e) % N) / N)


class PaddedAxis:
    """One dimension of the hybrid padding: L data values padded to N = m*q."""

    def __init__(self, kind: int, L: int, M: int, m: int | None = None):
        self.kind = kind
        self.L = L
        self.M = M
        centered = kind in (CENTERED, HERMITIAN)
        if kind == HERMITIAN:
            self.H = ceilquotient(L, 2)
            self.Lc = 2 * self.H - 1          # extended centred length
            self.c = self.H - 1
        else:
            self.Lc = L
            self.c = L // 2 if kind == CENTERED else 0
        self.m = M if not m else m
        if kind == HERMITIAN:
            # The Hermitian axis pads the extended sequence; the fold works on
            # its 2H-1 values.
            self.p, self.n, self.q = parameters(self.Lc, M, self.m, True)
        else:
            self.p, self.n, self.q = parameters(L, M, self.m, centered)
        self.N = self.m * self.q
        if self.N < M:
            raise ValueError("m*q < M")

    # Stored length along this axis.
    @property
    def stored(self) -> int:
        return self.H if self.kind == HERMITIAN else self.L

    def residues(self):
        return range(self.q)

    def extend(self, x: np.ndarray) -> np.ndarray:
        """Hermitian axis: stored modes k = 0..H-1 -> centred 2H-1 modes."""
        if self.kind != HERMITIAN:
            return x
        neg = np.conj(x[1:][::-1])
        return np.concatenate([neg, x], axis=0)

    def forward(self, x: np.ndarray, r: int, workers: int = WORKERS) -> np.ndarray:
        """Residue block r of the padded forward transform along axis 0."""
        m, p, q, N = self.m, self.p, self.q, self.N
        x = self.extend(x).astype(np.complex128, copy=False)
        Lc = x.shape[0]
        rest = x.shape[1:]
        pp = ceilquotient(Lc, m)
        xe = np.zeros((pp * m,) + rest, dtype=np.complex128)
        xe[:Lc] = x
        xe = xe.reshape((pp, m) + rest)
        u = np.arange(pp).reshape((pp, 1) + (1,) * len(rest))
        g = np.sum(xe * _roots(q, u * r), axis=0)           # fold, w_q^{ur}
        s = np.arange(m).reshape((m,) + (1,) * len(rest))
        g = g * _roots(N, s * r)                             # Zetaqm, w_N^{sr}
        F = _ifft_unscaled(g, 0, workers)                    # sign +1 DFT
        if self.c:
            j = np.arange(m).reshape((m,) + (1,) * len(rest))
            F = F * _roots(N, -self.c * (q * j + r))
        if self.kind == HERMITIAN:
            F = F.real.astype(np.complex128)
        return F

    def backward(self, F: np.ndarray, r: int, acc: np.ndarray,
                 workers: int = WORKERS) -> None:
        """Accumulate residue block r of the backward transform into acc
        (axis 0 of acc has the extended/stored length of this axis)."""
        m, q, N = self.m, self.q, self.N
        rest = F.shape[1:]
        F = F.astype(np.complex128, copy=False)
        if self.c:
            j = np.arange(m).reshape((m,) + (1,) * len(rest))
            F = F * _roots(N, self.c * (q * j + r))
        G = _fft(F, 0, workers)                              # sign -1 DFT
        s = np.arange(m).reshape((m,) + (1,) * len(rest))
        G = G * _roots(N, -s * r)
        Lc = acc.shape[0]
        pp = ceilquotient(Lc, m)
        for u in range(pp):
            lo = u * m
            hi = min(Lc, lo + m)
            acc[lo:hi] += G[: hi - lo] * _roots(q, -u * r)

    def finish(self, acc: np.ndarray) -> np.ndarray:
        """Map the accumulated extended data back to the stored layout."""
        if self.kind == HERMITIAN:
            return acc[self.c:]
        return acc


# ---------------------------------------------------------------------------
# Multipliers (convolve.cc:26-110) in physical space.

def mult_binary(F):
    return [F[0] * F[1]]


def mult_realbinary(F):
    return [(F[0].real * F[1].real).astype(np.complex128)]


def mult_correlation(F):
    return [F[0] * np.conj(F[1])]


def mult_jacobian(F):
    """Physical-space Jacobian F0*F3 - F1*F2 (ux*wy - uy*wx)."""
    return [F[0] * F[3] - F[1] * F[2]]


def mult_realjacobian(F):
    R = [f.real for f in F]
    return [(R[0] * R[3] - R[1] * R[2]).astype(np.complex128)]


def mult_realjacadj(F):
    """Adjoint products of the real Jacobian: inputs u0..u3 and the
    back-propagated field g, outputs g u3, -g u2, -g u1, g u0."""
    R = [f.real for f in F]
    g = R[4]
    return [(g * R[3]).astype(np.complex128), (-g * R[2]).astype(np.complex128),
            (-g * R[1]).astype(np.complex128), (g * R[0]).astype(np.complex128)]


def mult_dot(F):
    """Sum of A/2 binary products F_k F_{A/2+k}: the convolution of a dot
    product, declared (not defined) by the old C interface's *_dot entry
    points (wrappers/cfftw++.h:30-47)."""
    K = len(F) // 2
    return [sum(F[k] * F[K + k] for k in range(K))]


def mult_realdot(F):
    """mult_dot on real data (realMultBinary per pair, convolve.cc:60-83)."""
    K = len(F) // 2
    return [sum(F[k].real * F[K + k].real for k in range(K))
            .astype(np.complex128)]


MULTIPLIERS: dict[str, Callable] = {
    "dot": mult_dot,
    "realdot": mult_realdot,
    "realjacadj": mult_realjacadj,
    "binary": mult_binary,
    "realbinary": mult_realbinary,
    "correlation": mult_correlation,
    "jacobian": mult_jacobian,
    "realjacobian": mult_realjacobian,
}


# ---------------------------------------------------------------------------
# Drivers: Convolution / Convolution2 / Convolution3 restated recursively.

def _convolve_axes(fs: Sequence[np.ndarray], axes: Sequence[PaddedAxis],
                   mult: Callable, B: int, workers: int) -> list[np.ndarray]:
    """Raw (unnormalised) convolution of the A arrays fs over the leading
    len(axes) axes; returns B arrays in the extended layout of axes[0]."""
    ax = axes[0]
    shape = (ax.Lc,) + fs[0].shape[1:]
    acc = [np.zeros(shape, dtype=np.complex128) for _ in range(B)]
    for r in ax.residues():
        F = [ax.forward(f, r, workers) for f in fs]
        if len(axes) == 1:
            H = mult(F)
        else:
            # Inner sub-convolution of every transformed row
            # (Convolution2::subconvolution, convolve.h:1434-1445).
            Fi = [np.moveaxis(Fa, 0, -1) for Fa in F]
            Hi = _convolve_axes_inner(Fi, axes[1:], mult, B, workers)
            H = [np.moveaxis(h, -1, 0) for h in Hi]
        for b in range(B):
            ax.backward(H[b], r, acc[b], workers)
    return [ax.finish(a) for a in acc]


def _convolve_axes_inner(fs, axes, mult, B, workers):
    # fs: arrays whose leading axes are the remaining data axes and whose
    # last axis indexes the outer transformed rows.
    return _convolve_axes(fs, axes, mult, B, workers)


def convolve(inputs: Sequence[np.ndarray], kinds: Sequence[int],
             Ls: Sequence[int], Ms: Sequence[int], *,
             ms: Sequence[int] | None = None, mult: str = "binary",
             B: int = 1, normalize: bool = True,
             workers: int = WORKERS) -> list[np.ndarray]:
    """Hybrid dealiased convolution of A dense arrays (row-major, stored
    layout: Hermitian last axis holds ceil(L/2) modes; a real first axis
    means real data throughout).  Returns the B outputs."""
    dim = len(kinds)
    axes = [PaddedAxis(kinds[d], Ls[d], Ms[d], ms[d] if ms else None)
            for d in range(dim)]
    real = kinds[0] == REAL
    fs = [np.asarray(f).astype(np.complex128) for f in inputs]
    for f in fs:
        expect = tuple(ax.stored for ax in axes)
        if f.shape != expect:
            raise ValueError(f"input shape {f.shape} != {expect}")
    out = _convolve_axes(fs, axes, MULTIPLIERS[mult], B, workers)
    scale = 1.0
    if normalize:
        for ax in axes:
            scale /= ax.N
    res = []
    for h in out:
        h = h * scale
        res.append(h.real.copy() if real else h)
    return res


def default_M(kind: int, L: int, A: int = 2) -> int:
    """Default minimum padded length of the reference's C wrappers
    (wrappers/HybridConvolution.h:19, 39): A*L-A+1 for complex/real data,
    3*ceil(L/2)-2*(L%2) for centred/Hermitian data."""
    if kind in (CENTERED, HERMITIAN):
        return 3 * ceilquotient(L, 2) - 2 * (L % 2)
    return A * L - A + 1


# ---------------------------------------------------------------------------
# Input preparation shared with the reference's tests.

def hermitian_symmetrize_x(f: np.ndarray, Hx: int, Hy: int, x0: int) -> None:
    """HermitianSymmetrizeX (convolve.h:1175-1197) on a dense Lx x Hy array:
    f(-kx,0) = conj f(kx,0), real origin, zero Nyquist row when x0 == Hx."""
    for i in range(1, Hx):
        if x0 - i >= 0 and x0 + i < f.shape[0]:
            f[x0 - i, 0] = np.conj(f[x0 + i, 0])
    f[x0, 0] = f[x0, 0].real
    if x0 == Hx:
        f[0, :] = 0.0


def hermitian_symmetrize_xy(f: np.ndarray, Hx: int, Hy: int, Hz: int,
                            x0: int, y0: int) -> None:
    """HermitianSymmetrizeXY (convolve.h:1207-1258) on a dense
    Lx x Ly x Hz array."""
    Lx, Ly = f.shape[0], f.shape[1]
    for i in range(1, Hx):
        f[x0 - i, y0, 0] = np.conj(f[x0 + i, y0, 0])
    f[x0, y0, 0] = f[x0, y0, 0].real
    for i in range(-Hx + 1, Hx):
        for j in range(1, Hy):
            f[x0 - i, y0 - j, 0] = np.conj(f[x0 + i, y0 + j, 0])
    if x0 == Hx:
        f[0, :y0 + Hy, :] = 0.0
    if y0 == Hy:
        f[:x0 + Hx, 0, :] = 0.0


def conv_flops(kind_lengths: Sequence[int]) -> float:
    """Nominal 5 N log2 N flop count of one padded complex transform."""
    total = 1
    for n in kind_lengths:
        total *= n
    return 5.0 * total * math.log2(max(total, 2))
