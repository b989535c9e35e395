"""GPU: strided layouts (the reference's fftPad(L, M, app, C, S) with S > C
and the Sx / Sy strides of Convolution2 / Convolution3, convolve.h:515-536,
1274, 1556; tests/hybridconv2.cc, hybridconvh2.cc, hybridconv3.cc) through
fgb_set_strides and the C ABI: the stored entries convolve as the dense
arrays do (against the oracle), the gaps are neither read nor written, on
the device entry in every precision and on the host entry with page-locked
and pageable arrays."""
import ctypes

import numpy as np
import pytest

from oracle import hybrid as H
from oracle.direct import rel_l2

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-13, "ff": 1e-13, "f32": 2e-6}
SENTINEL = 12345.0


def _dense_inputs(kinds, L, seed):
    rng = np.random.default_rng(seed)
    shape = [(l + 1) // 2 if k == H.HERMITIAN else l for k, l in zip(kinds, L)]
    fs = []
    for _ in range(2):
        if kinds[0] == H.REAL:
            f = rng.normal(size=shape)
        else:
            f = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
        if kinds[-1] == H.HERMITIAN and len(kinds) == 2:
            H.hermitian_symmetrize_x(f, (L[0] + 1) // 2, shape[1], L[0] // 2)
        fs.append(f)
    return fs


def _embed(f, strides, dtype):
    """f laid out with the given outer strides, gaps = SENTINEL."""
    if f.ndim == 2:
        buf = np.full(f.shape[0] * strides[0], SENTINEL, dtype=dtype)
        v = buf.reshape(f.shape[0], strides[0])
        v[:, :f.shape[1]] = f
        return buf
    n0, n1, n2 = f.shape
    buf = np.full(n0 * strides[0], SENTINEL, dtype=dtype)
    for i in range(n0):
        for j in range(n1):
            o = i * strides[0] + j * strides[1]
            buf[o:o + n2] = f[i, j]
    return buf


def _extract(buf, shape, strides):
    if len(shape) == 2:
        return buf.reshape(shape[0], strides[0])[:, :shape[1]].copy()
    out = np.empty(shape, dtype=buf.dtype)
    for i in range(shape[0]):
        for j in range(shape[1]):
            o = i * strides[0] + j * strides[1]
            out[i, j] = buf[o:o + shape[2]]
    return out


def _gaps_intact(buf, shape, strides):
    mask = np.ones(buf.size, dtype=bool)
    if len(shape) == 2:
        mask.reshape(shape[0], strides[0])[:, :shape[1]] = False
    else:
        for i in range(shape[0]):
            for j in range(shape[1]):
                o = i * strides[0] + j * strides[1]
                mask[o:o + shape[2]] = False
    return bool(np.all(buf[mask] == SENTINEL))


CASES = [
    ([H.CENTERED, H.HERMITIAN], [31, 31], [46, 46], "realbinary", [16 + 5]),
    ([H.PAD, H.PAD], [16, 12], [31, 23], "binary", [12 + 3]),
    ([H.REAL, H.PAD], [16, 15], [31, 29], "binary", [15 + 1]),
    ([H.PAD, H.PAD, H.PAD], [6, 5, 7], [11, 9, 13], "binary", [5 * 9 + 4, 9]),
    ([H.REAL, H.PAD, H.PAD], [12, 10, 9], [23, 19, 17], "binary",
     [10 * 9 + 7, 9]),
]


def _plan(kinds, L, M, mult, precision, strides):
    from fftwpp_gb300.gpu import HybridConvolution
    conv = HybridConvolution(kinds, L, M, mult=mult, precision=precision)
    arr = (ctypes.c_size_t * len(strides))(*strides)
    assert conv.lib.fgb_set_strides(conv.handle, arr) == 0, \
        conv.lib.fgb_last_error()
    return conv


@pytest.mark.parametrize("precision", ["f64", "ff", "f32"])
@pytest.mark.parametrize("case", CASES, ids=lambda c: "x".join(map(str, c[1]))
                         + "-" + str(c[0][0]))
def test_strided_device(native_lib, case, precision):
    import torch
    kinds, L, M, mult, strides = case
    fs = _dense_inputs(kinds, L, seed=sum(L))
    want = H.convolve(fs, kinds, L, M, mult=mult)[0]
    conv = _plan(kinds, L, M, mult, precision, strides)
    real = kinds[0] == H.REAL
    npdt = {"f64": np.float64 if real else np.complex128,
            "ff": np.float64 if real else np.complex128,
            "f32": np.float32 if real else np.complex64}[precision]
    bufs = [torch.from_numpy(_embed(f.astype(npdt), strides, npdt)).cuda()
            for f in fs]
    out = torch.from_numpy(np.full(bufs[0].numel(), SENTINEL,
                                   dtype=npdt)).cuda()
    vp = ctypes.c_void_p
    pin = (vp * 2)(*[b.data_ptr() for b in bufs])
    pout = (vp * 1)(out.data_ptr())
    rc = conv.lib.fgb_convolve_device(
        conv.handle, pin, pout, vp(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, conv.lib.fgb_last_error()
    h = out.cpu().numpy()
    shape = fs[0].shape
    assert rel_l2(_extract(h, shape, strides).astype(want.dtype),
                  want) <= TOL[precision]
    assert _gaps_intact(h, shape, strides)
    for b in bufs:                        # inputs untouched, gaps included
        assert _gaps_intact(b.cpu().numpy(), shape, strides)


@pytest.mark.parametrize("pinned", [True, False])
def test_strided_host(native_lib, pinned):
    """fgb_convolve_host on strided arrays (in place, as the reference's
    convolve overwrites f[0]): page-locked arrays are addressed by the
    kernels, pageable ones are copied; gaps stay untouched either way."""
    import torch
    kinds, L, M, mult, strides = CASES[0]
    fs = _dense_inputs(kinds, L, seed=77)
    want = H.convolve(fs, kinds, L, M, mult=mult)[0]
    conv = _plan(kinds, L, M, mult, "f64", strides)
    hs = [_embed(f, strides, np.complex128) for f in fs]
    if pinned:
        hs = [torch.from_numpy(h).pin_memory().numpy() for h in hs]
    vp = ctypes.c_void_p
    pin = (vp * 2)(*[h.ctypes.data for h in hs])
    assert conv.lib.fgb_convolve_host(conv.handle, pin, pin) == 0, \
        conv.lib.fgb_last_error()
    assert rel_l2(_extract(hs[0], fs[0].shape, strides), want) <= 1e-13
    assert _gaps_intact(hs[0], fs[0].shape, strides)
    assert np.array_equal(_extract(hs[1], fs[1].shape, strides), fs[1])


def test_strides_validated(native_lib):
    """Strides smaller than the data they step over, and strides on a 1D
    plan, are refused."""
    from fftwpp_gb300.gpu import HybridConvolution
    conv = HybridConvolution([H.PAD, H.PAD, H.PAD], [6, 5, 7], [11, 9, 13])
    bad = [(5 * 7 - 1, 7), (5 * 9, 6)]
    for s in bad:
        arr = (ctypes.c_size_t * 2)(*s)
        assert conv.lib.fgb_set_strides(conv.handle, arr) == -1
    one = HybridConvolution([H.PAD], [16], [31])
    arr = (ctypes.c_size_t * 1)(20)
    assert one.lib.fgb_set_strides(one.handle, arr) == -1
    assert conv.lib.fgb_set_strides(conv.handle, None) == 0
