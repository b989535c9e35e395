"""GPU: the dot-product and work-array forms of the FFTW++ C interface
(fftwpp_create_*_dot / *_work / *_work_dot, fftwpp_*_convolve_dot / _dotf),
called through the C ABI with host arrays, against the oracle's
sum-of-products convolution.  Sums of more than four products exercise the
chunked device accumulation."""
import ctypes

import numpy as np
import pytest

from oracle import hybrid as H
from oracle.direct import rel_l2

pytestmark = pytest.mark.gpu

# name, axis kinds, data lengths m, multiplier of the oracle
CASES = [
    ("conv1d", [H.PAD], [37], "dot"),
    ("hconv1d", [H.HERMITIAN], [19], "realdot"),
    ("conv2d", [H.PAD, H.PAD], [9, 11], "dot"),
    ("hconv2d", [H.CENTERED, H.HERMITIAN], [15, 15], "realdot"),
    ("conv3d", [H.PAD, H.PAD, H.PAD], [5, 6, 7], "dot"),
    ("hconv3d", [H.CENTERED, H.CENTERED, H.HERMITIAN], [5, 7, 9], "realdot"),
]
NWORK = {"conv1d": 2, "hconv1d": 3, "conv2d": 4, "hconv2d": 5, "conv3d": 6,
         "hconv3d": 7}


def _inputs(kinds, L, n, seed):
    rng = np.random.default_rng(seed)
    shape = list(L)
    if kinds[-1] == H.HERMITIAN:
        shape[-1] = (L[-1] + 1) // 2
    out = []
    for _ in range(n):
        f = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
        if kinds[-1] == H.HERMITIAN and len(kinds) == 1:
            f[0] = f[0].real
        if kinds[-1] == H.HERMITIAN and len(kinds) == 2:
            H.hermitian_symmetrize_x(f, (L[0] + 1) // 2, shape[1], L[0] // 2)
        if kinds[-1] == H.HERMITIAN and len(kinds) == 3:
            H.hermitian_symmetrize_xy(f, (L[0] + 1) // 2, (L[1] + 1) // 2,
                                      shape[2], L[0] // 2, L[1] // 2)
        out.append(np.ascontiguousarray(f))
    return out


def _want(kinds, L, a, b, mult):
    M = [H.default_M(k, l) for k, l in zip(kinds, L)]
    return H.convolve(list(a) + list(b), kinds, L, M, mult=mult)[0]


def _ptrs(arrs):
    return (ctypes.c_void_p * len(arrs))(*[x.ctypes.data for x in arrs])


@pytest.mark.parametrize("pairs", [1, 3, 6])
@pytest.mark.parametrize("name,kinds,L,mult", CASES)
def test_convolve_dot(native_lib, name, kinds, L, mult, pairs):
    lib = native_lib
    fs = _inputs(kinds, L, 2 * pairs, seed=pairs * 10 + len(L))
    a, b = fs[:pairs], fs[pairs:]
    want = _want(kinds, L, a, b, mult)
    h = getattr(lib, f"fftwpp_create_{name}_dot")(*L, pairs)
    assert h, lib.fgb_last_error()
    try:
        aa = [x.copy() for x in a]
        getattr(lib, f"fftwpp_{name}_convolve_dot")(h, _ptrs(aa), _ptrs(b))
        assert rel_l2(aa[0], want) <= 1e-13
        # Inputs other than a[0] are left as they were.
        for x, y in zip(aa[1:], a[1:]):
            assert np.array_equal(x, y)
        if name != "hconv3d":
            fa = np.ascontiguousarray(np.stack(a))
            fb = np.ascontiguousarray(np.stack(b))
            getattr(lib, f"fftwpp_{name}_convolve_dotf")(
                h, fa.ctypes.data, fb.ctypes.data)
            assert rel_l2(fa[0], want) <= 1e-13
    finally:
        getattr(lib, f"fftwpp_{name}_delete")(h)


@pytest.mark.parametrize("name,kinds,L,mult", CASES)
def test_work_forms(native_lib, name, kinds, L, mult):
    """The work-array constructors ignore the caller's host scratch and
    behave like the plain (and dot) forms."""
    lib = native_lib
    work = [np.zeros(4, dtype=np.complex128) for _ in range(NWORK[name])]
    wp = [w.ctypes.data for w in work]
    a, b = _inputs(kinds, L, 2, seed=7)
    want = _want(kinds, L, [a], [b], mult)
    h = getattr(lib, f"fftwpp_create_{name}_work")(*L, *wp)
    assert h, lib.fgb_last_error()
    try:
        aa = a.copy()
        getattr(lib, f"fftwpp_{name}_convolve")(h, aa.ctypes.data,
                                                 b.ctypes.data)
        assert rel_l2(aa, want) <= 1e-13
        # A plain handle in a _dot call computes the single product.
        aa = a.copy()
        getattr(lib, f"fftwpp_{name}_convolve_dot")(h, _ptrs([aa]),
                                                     _ptrs([b]))
        assert rel_l2(aa, want) <= 1e-13
    finally:
        getattr(lib, f"fftwpp_{name}_delete")(h)
    if name != "conv3d":
        fs = _inputs(kinds, L, 10, seed=8)
        want = _want(kinds, L, fs[:5], fs[5:], mult)
        h = getattr(lib, f"fftwpp_create_{name}_work_dot")(*L, *wp, 5)
        assert h, lib.fgb_last_error()
        try:
            aa = [x.copy() for x in fs[:5]]
            getattr(lib, f"fftwpp_{name}_convolve_dot")(h, _ptrs(aa),
                                                         _ptrs(fs[5:]))
            assert rel_l2(aa[0], want) <= 1e-13
        finally:
            getattr(lib, f"fftwpp_{name}_delete")(h)
    assert all(not w.any() for w in work)


def test_dot_rejects_zero_products(native_lib):
    assert not native_lib.fftwpp_create_conv1d_dot(16, 0)
    assert b"positive" in native_lib.fgb_last_error()
