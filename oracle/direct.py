"""CPU oracle: O(L^d) direct-sum convolutions restating the reference's
tests/direct.h and tests/direct.cc.

TEST INFRASTRUCTURE ONLY (checker for tests/ and smoke(); never shipped on
the GPU path).  These are the reference's own FP64 direct oracles:

* ``directconv``      -- directconv<T>::convolve   (tests/direct.h:20-27)
* ``directconv_c``    -- directconv<T>::convolveC  (tests/direct.h:28-41),
                         the centred 1D variant
* ``directconvh``     -- directconvh::convolve     (tests/direct.cc:5-14)
* ``directconv2``     -- directconv2<T>::convolve  (tests/direct.h:78-89)
* ``directconvh2``    -- directconvh2::convolve    (tests/direct.cc:16-53)
* ``directconv3``     -- directconv3<T>::convolve  (tests/direct.h:118-133)
* ``directconvh3``    -- directconvh3::convolve    (tests/direct.cc:55-98)

Loops over the shift are kept; the inner sums are vectorised with numpy.
"""
from __future__ import annotations

import numpy as np


def directconv(f: np.ndarray, g: np.ndarray) -> np.ndarray:
    """h[i] = sum_{j<=i} f[j] g[i-j], i < L."""
    L = len(f)
    h = np.zeros(L, dtype=np.result_type(f, g))
    for i in range(L):
        h[i] = np.sum(f[: i + 1] * g[i::-1])
    return h


def directconv_c(f: np.ndarray, g: np.ndarray) -> np.ndarray:
    """Centred 1D convolution: index j carries wavenumber j - floor(L/2)."""
    m = len(f)
    h = np.zeros(m, dtype=np.result_type(f, g))
    for i in range(m // 2):
        j = np.arange(i + 1, m)
        h[i + (m + 1) // 2] = np.sum(f[j] * g[m + i - j])
    for i in range(m // 2, m):
        j = np.arange(0, i + 1)
        h[i - m // 2] = np.sum(f[j] * g[i - j])
    return h


def directconvh(f: np.ndarray, g: np.ndarray) -> np.ndarray:
    """1D Hermitian: f, g hold the m non-negative modes of real functions."""
    m = len(f)
    h = np.zeros(m, dtype=np.complex128)
    for i in range(m):
        s = np.sum(f[: i + 1] * g[i::-1])
        j = np.arange(i + 1, m)
        s += np.sum(f[j] * np.conj(g[j - i]))
        j = np.arange(1, m - i)
        s += np.sum(np.conj(f[j]) * g[i + j])
        h[i] = s
    return h


def directconv2(f: np.ndarray, g: np.ndarray) -> np.ndarray:
    """2D complex: h[i,j] = sum_{k<=i,p<=j} f[k,p] g[i-k,j-p]."""
    mx, my = f.shape
    h = np.zeros((mx, my), dtype=np.result_type(f, g))
    for k in range(mx):
        for p in range(my):
            h[k:, p:] += f[k, p] * g[: mx - k, : my - p]
    return h


def _hget(f: np.ndarray, xorigin: int, kx: np.ndarray, ky: np.ndarray):
    """Value of a 2D half-plane Hermitian array at (kx, ky), ky of any sign."""
    kx, ky = np.broadcast_arrays(kx, ky)
    pos = ky >= 0
    out = np.empty(kx.shape, dtype=np.complex128)
    out[pos] = f[xorigin + kx[pos], ky[pos]]
    neg = ~pos
    out[neg] = np.conj(f[xorigin - kx[neg], -ky[neg]])
    return out


def directconvh2(f: np.ndarray, g: np.ndarray, xcompact: bool) -> np.ndarray:
    """2D centred Hermitian (tests/direct.cc:16-53), inputs already
    symmetrised.  f, g: (2*mx - xcompact) x my with the x origin at
    mx - xcompact; returns the same layout."""
    nx, my = f.shape
    mx = (nx + xcompact) // 2
    xorigin = mx - xcompact
    xstart, xstop = -xorigin, mx
    ystart, ystop = 1 - my, my
    lo = xstart + (0 if xcompact else 1)
    h = np.zeros((nx, my), dtype=np.complex128)
    px = np.arange(lo, xstop)[:, None]
    py = np.arange(ystart, ystop)[None, :]
    fv = _hget(f, xorigin, px, py)
    for kx in range(xstart, xstop):
        for ky in range(0, ystop):
            qx = kx - px
            qy = ky - py
            ok = (qx >= lo) & (qx < xstop) & (qy >= ystart) & (qy < ystop)
            qxc = np.where(ok, qx, 0)
            qyc = np.where(ok, qy, 0)
            gv = _hget(g, xorigin, qxc, qyc)
            h[xorigin + kx, ky] = np.sum(np.where(ok, fv * gv, 0.0))
    return h


def directconv3(f: np.ndarray, g: np.ndarray) -> np.ndarray:
    """3D complex/real direct convolution (tests/direct.h:118-133)."""
    mx, my, mz = f.shape
    h = np.zeros((mx, my, mz), dtype=np.result_type(f, g))
    for r in range(mx):
        for p in range(my):
            for q in range(mz):
                h[r:, p:, q:] += f[r, p, q] * g[: mx - r, : my - p, : mz - q]
    return h


def directconvh3(f: np.ndarray, g: np.ndarray, xcompact: bool,
                 ycompact: bool) -> np.ndarray:
    """3D centred Hermitian (tests/direct.cc:55-98), inputs symmetrised.
    f, g: (2mx-xcompact) x (2my-ycompact) x mz."""
    nx, ny, mz = f.shape
    mx = (nx + xcompact) // 2
    my = (ny + ycompact) // 2
    xo, yo = mx - xcompact, my - ycompact
    xlo = -xo + (0 if xcompact else 1)
    ylo = -yo + (0 if ycompact else 1)
    h = np.zeros((nx, ny, mz), dtype=np.complex128)

    def get(a, kx, ky, kz):
        if kz >= 0:
            return a[xo + kx, yo + ky, kz]
        return np.conj(a[xo - kx, yo - ky, -kz])

    rng = [(px, py, pz) for px in range(xlo, mx) for py in range(ylo, my)
           for pz in range(1 - mz, mz)]
    for kx in range(-xo, mx):
        for ky in range(-yo, my):
            for kz in range(0, mz):
                s = 0.0j
                for px, py, pz in rng:
                    qx, qy, qz = kx - px, ky - py, kz - pz
                    if xlo <= qx < mx and ylo <= qy < my and 1 - mz <= qz < mz:
                        s += get(f, px, py, pz) * get(g, qx, qy, qz)
                h[xo + kx, yo + ky, kz] = s
    return h


def directconv3_at(f: np.ndarray, g: np.ndarray, points) -> np.ndarray:
    """Entries h[i, j, k] of the 3D direct convolution (tests/direct.h:
    118-133, h[i,j,k] = sum f[a,b,c] g[i-a,j-b,k-c] over a <= i, b <= j,
    c <= k) at the given index triples only, for sizes whose full O(L^6)
    sum is out of reach; each entry is one vectorised FP64 sum."""
    out = []
    for idx in points:
        i, j, k = (int(t) for t in idx)
        out.append(np.sum(f[:i + 1, :j + 1, :k + 1] *
                          g[i::-1, j::-1, k::-1]))
    return np.asarray(out)


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    """Relative L2 error |a-b|/|b| as in the reference's tests
    (tests/hybridconv.cc:118-129)."""
    num = np.linalg.norm(np.asarray(a).ravel() - np.asarray(b).ravel())
    den = np.linalg.norm(np.asarray(b).ravel())
    return float(num / den) if den > 0 else float(num)
