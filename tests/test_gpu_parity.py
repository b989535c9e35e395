"""GPU parity: the sm_103a kernels (through the C ABI of lib_fftwpp.so)
against the CPU oracle (numpy restatement of FFTW++'s hybrid convolution,
pinned to the compiled reference) on seeded inputs.

Tolerances (relative L2, as the reference's tests measure it,
tests/hybridconv.cc:118-129): 1e-13 in FP64 and in the float-float mode
(FP64 data, hi+lo float arithmetic), 2e-6 in FP32-compensated mode.
"""
import os

import numpy as np
import pytest

from oracle import hybrid as H
from oracle.direct import rel_l2

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-13, "ff": 1e-13, "f32": 2e-6}


def _rand(rng, shape, real):
    if real:
        return rng.normal(size=shape)
    return rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)


def _inputs(kinds, L, A, seed):
    rng = np.random.default_rng(seed)
    shape = [l for l in L]
    if kinds[-1] == H.HERMITIAN:
        shape[-1] = (L[-1] + 1) // 2
    real = kinds[0] == H.REAL
    fs = [_rand(rng, tuple(shape), real) for _ in range(A)]
    if kinds[-1] == H.HERMITIAN:
        for f in fs:
            if len(kinds) == 1:
                f[0] = f[0].real
            elif len(kinds) == 2:
                Lx = L[0]
                H.hermitian_symmetrize_x(f, (Lx + 1) // 2, shape[1], Lx // 2)
            else:
                H.hermitian_symmetrize_xy(f, (L[0] + 1) // 2, (L[1] + 1) // 2,
                                          shape[2], L[0] // 2, L[1] // 2)
    return fs


def _ldexp(a, e):
    """a * 2^e exactly, for real or complex arrays."""
    a = np.asarray(a)
    if np.iscomplexobj(a):
        return np.ldexp(a.real, e) + 1j * np.ldexp(a.imag, e)
    return np.ldexp(a, e)


def run_gpu(kinds, L, M, fs, mult, precision, m=None, B=1):
    import torch
    from fftwpp_gb300.gpu import HybridConvolution
    A = len(fs)
    conv = HybridConvolution(kinds, L, M, m=m, A=A, B=B, mult=mult,
                             precision=precision)
    dt = conv.dtype
    ts = [torch.from_numpy(np.ascontiguousarray(f)).to(dt).cuda() for f in fs]
    out = conv.convolve(*ts)
    torch.cuda.synchronize()
    return [o.cpu().numpy() for o in out], conv


CASES = [
    # (kinds, L, M, mult)
    ([H.PAD], [8], [16], "binary"),
    ([H.PAD], [9], [17], "binary"),
    ([H.PAD], [7], [13], "binary"),
    ([H.PAD], [1024], [2047], "binary"),            # 1D complex workload
    ([H.PAD], [1000], [1999], "correlation"),
    ([H.CENTERED], [8], [16], "binary"),
    ([H.CENTERED], [9], [13], "binary"),
    ([H.CENTERED], [8], [12], "binary"),
    ([H.CENTERED], [7], [10], "binary"),
    ([H.HERMITIAN], [7], [10], "realbinary"),
    ([H.HERMITIAN], [8], [12], "realbinary"),
    ([H.HERMITIAN], [15], [22], "realbinary"),
    ([H.HERMITIAN], [1023], [1534], "realbinary"),
    ([H.REAL], [8], [16], "binary"),
    ([H.REAL], [9], [17], "binary"),
    ([H.REAL], [100], [199], "binary"),
    ([H.PAD, H.PAD], [8, 6], [15, 11], "binary"),
    ([H.PAD, H.PAD], [33, 17], [65, 33], "binary"),
    ([H.CENTERED, H.HERMITIAN], [7, 7], [10, 10], "realbinary"),
    ([H.CENTERED, H.HERMITIAN], [8, 8], [12, 12], "realbinary"),
    ([H.CENTERED, H.HERMITIAN], [9, 7], [13, 10], "realbinary"),
    ([H.CENTERED, H.HERMITIAN], [63, 63], [94, 94], "realbinary"),
    ([H.REAL, H.PAD], [8, 6], [15, 11], "binary"),
    ([H.REAL, H.PAD], [16, 15], [31, 29], "binary"),
    ([H.PAD, H.PAD, H.PAD], [4, 5, 6], [7, 9, 11], "binary"),
    ([H.REAL, H.PAD, H.PAD], [4, 5, 6], [7, 9, 11], "binary"),
    ([H.REAL, H.PAD, H.PAD], [8, 8, 8], [15, 15, 15], "binary"),
    ([H.CENTERED, H.CENTERED, H.HERMITIAN], [5, 5, 5], [7, 7, 7], "realbinary"),
    ([H.CENTERED, H.CENTERED, H.HERMITIAN], [7, 6, 9], [10, 9, 13], "realbinary"),
]


def _ids():
    names = {0: "pad", 1: "cen", 2: "her", 3: "real"}
    return ["-".join(names[k] for k in c[0]) + "-" + "x".join(map(str, c[1]))
            + "-" + c[3] for c in CASES]


@pytest.mark.parametrize("precision", ["f64", "ff", "f32"])
@pytest.mark.parametrize("case", CASES, ids=_ids())
def test_parity(case, precision, native_lib):
    kinds, L, M, mult = case
    fs = _inputs(kinds, L, 2, seed=sum(L) + 7)
    want = H.convolve(fs, kinds, L, M, mult=mult)[0]
    got, conv = run_gpu(kinds, L, M, fs, mult, precision)
    err = rel_l2(got[0], want)
    assert err <= TOL[precision], (err, conv.axes)


@pytest.mark.parametrize("m", [2, 4, 8, 16])
def test_forced_m(m, native_lib):
    """The reference's Application m (convolve.h:103-111): any residue block
    length gives the same dealiased result."""
    kinds, L, M = [H.PAD], [16], [31]
    fs = _inputs(kinds, L, 2, seed=3)
    want = H.convolve(fs, kinds, L, M)[0]
    got, conv = run_gpu(kinds, L, M, fs, "binary", "f64", m=[m])
    assert conv.axes[0]["m"] == m
    assert rel_l2(got[0], want) <= 1e-13


@pytest.mark.parametrize("precision", ["f64", "ff"])
def test_long_1d(native_lib, precision):
    """1D data too long for one CTA takes the column/row/column path."""
    kinds, L, M = [H.PAD], [20000], [39999]
    fs = _inputs(kinds, L, 2, seed=11)
    want = H.convolve(fs, kinds, L, M)[0]
    got, conv = run_gpu(kinds, L, M, fs, "binary", precision)
    assert conv.long_path
    assert rel_l2(got[0], want) <= 1e-13


def test_float_float_large_2d(native_lib):
    """The float-float mode on the 2D centred-Hermitian workload's full
    size (1023 x 512 modes) against the FP64 GPU path, whose parity with
    the oracle the tests above establish."""
    kinds, L, M = [H.CENTERED, H.HERMITIAN], [1023, 1023], [1534, 1534]
    fs = _inputs(kinds, L, 2, seed=21)
    g64, _ = run_gpu(kinds, L, M, fs, "realbinary", "f64")
    gff, conv = run_gpu(kinds, L, M, fs, "realbinary", "ff")
    assert conv.launches == 3
    assert rel_l2(gff[0], g64[0]) <= 1e-13


def test_jacobian_2d(native_lib):
    """A=4 centred-Hermitian inputs, physical-space Jacobian multiplier."""
    kinds, L, M = [H.CENTERED, H.HERMITIAN], [15, 15], [22, 22]
    fs = _inputs(kinds, L, 4, seed=5)
    want = H.convolve(fs, kinds, L, M, mult="realjacobian")[0]
    for prec in ("f64", "ff", "f32"):
        got, _ = run_gpu(kinds, L, M, fs, "realjacobian", prec)
        assert rel_l2(got[0], want) <= TOL[prec]


@pytest.mark.parametrize("precision", ["f64", "ff", "f32"])
def test_host_pointer_entry(native_lib, precision):
    """fgb_convolve_host (copies inside the call) in every mode; host arrays
    of the wrong type or shape are refused before any copy."""
    from fftwpp_gb300.gpu import HybridConvolution
    kinds, L, M = [H.CENTERED, H.HERMITIAN], [31, 31], [46, 46]
    fs = _inputs(kinds, L, 2, seed=9)
    want = H.convolve(fs, kinds, L, M, mult="realbinary")[0]
    conv = HybridConvolution(kinds, L, M, mult="realbinary",
                             precision=precision)
    dt = np.complex64 if precision == "f32" else np.complex128
    hs = [f.astype(dt) for f in fs]
    conv.convolve_host(*hs)
    assert rel_l2(hs[0], want) <= TOL[precision]
    with pytest.raises(TypeError):
        conv.convolve_host(*[f.astype(np.complex64 if dt == np.complex128
                                      else np.complex128) for f in fs])
    with pytest.raises(TypeError):
        conv.convolve_host(*[f[:-1].copy().astype(dt) for f in fs])


@pytest.mark.parametrize("scales", [(1e-25, 1e30), (1e20, 1e-18), (1.0, 0.0),
                                    (2.0 ** -69, 2.0 ** 69), (1e150, 1e-150),
                                    (1e300, 1e-5), (1e-300, 1e5),
                                    (1e150, 1e150), (1e-150, 1e-150)])
def test_float_float_scales(native_lib, scales):
    """FP64 inputs far from 1 (both sides of the fast split's range, far
    beyond a float's exponent range, and zero) in the float-float mode: the
    range guard scales them into range and back."""
    kinds, L, M = [H.CENTERED, H.HERMITIAN], [31, 31], [46, 46]
    fs = _inputs(kinds, L, 2, seed=13)
    fs = [fs[0] * scales[0], fs[1] * scales[1]]
    # A spread of magnitudes inside one array as well.
    fs[0][::3] *= 1e-12
    want = H.convolve(fs, kinds, L, M, mult="realbinary")[0]
    got, _ = run_gpu(kinds, L, M, fs, "realbinary", "ff")
    if not np.any(want):
        assert not np.any(got[0])
    else:
        # Relative error of arrays near 1e300, measured after an exact
        # power-of-two rescale (their squared norm overflows in FP64).
        e = int(np.frexp(np.abs(want).max())[1])
        assert rel_l2(_ldexp(got[0], -e), _ldexp(want, -e)) <= 1e-13


@pytest.mark.parametrize("precision", ["f64", "ff", "f32"])
def test_autotune_changes_schedule_only(native_lib, precision):
    """Autotuned tiles and rows per CTA regroup columns and rows across
    CTAs without changing any arithmetic: results are bit-identical to the
    cost-model plan."""
    kinds, L, M = [H.REAL, H.PAD, H.PAD], [12, 10, 9], [23, 19, 17]
    fs = _inputs(kinds, L, 2, seed=17)
    try:
        native_lib.fgb_set_residue_search(0)
        try:
            native_lib.fgb_set_autotune(0)
            plain, c0 = run_gpu(kinds, L, M, fs, "binary", precision)
        finally:
            native_lib.fgb_set_autotune(1)
        tuned, c1 = run_gpu(kinds, L, M, fs, "binary", precision)
    finally:
        native_lib.fgb_set_residue_search(1)
    assert np.array_equal(plain[0], tuned[0])


@pytest.mark.parametrize("precision", ["f64", "ff", "f32"])
@pytest.mark.parametrize("case", [
    ([H.CENTERED, H.HERMITIAN], [31, 31], [46, 46], "realbinary"),
    ([H.PAD], [300], [599], "binary"),
    ([H.REAL, H.PAD, H.PAD], [12, 10, 9], [23, 19, 17], "binary")])
def test_zero_copy_host_path(native_lib, precision, case):
    """Page-locked host arrays are read and written by the kernels in place
    over the host link, or copied whole by the SMs, each side the way the
    plan measured fastest; the result equals the copying path and every
    forced combination of ways bit for bit."""
    import torch
    from fftwpp_gb300.gpu import HybridConvolution
    kinds, L, M, mult = case
    fs = _inputs(kinds, L, 2, seed=23)
    want = H.convolve(fs, kinds, L, M, mult=mult)[0]
    conv = HybridConvolution(kinds, L, M, mult=mult, precision=precision)
    tdt = conv.dtype

    def pinned():
        return [torch.from_numpy(np.ascontiguousarray(f)).to(tdt).pin_memory()
                .numpy() for f in fs]
    zc = pinned()
    conv.convolve_host(*zc)
    assert rel_l2(zc[0], want) <= TOL[precision]
    try:
        native_lib.fgb_set_zero_copy(0)
        cp = pinned()
        conv.convolve_host(*cp)
    finally:
        native_lib.fgb_set_zero_copy(1)
    assert np.array_equal(zc[0], cp[0])
    assert np.array_equal(zc[1], cp[1])      # the second input is untouched
    try:
        for wi in (0, 1, 2):
            for wo in (0, 1, 2):
                native_lib.fgb_set_host_path(wi, wo)
                h = pinned()
                conv.convolve_host(*h)
                assert np.array_equal(zc[0], h[0]), (wi, wo)
                assert np.array_equal(zc[1], h[1]), (wi, wo)
    finally:
        native_lib.fgb_set_host_path(-1, -1)


@pytest.mark.parametrize("precision", ["f64", "ff", "f32"])
@pytest.mark.parametrize("case", [
    ([H.PAD, H.CENTERED, H.PAD], [12, 10, 9], [23, 19, 17], "binary", 2, 1),
    ([H.CENTERED, H.HERMITIAN], [31, 31], [46, 46], "realjacadj", 5, 4)])
def test_host_path_column_ranges(native_lib, precision, case):
    """Host calls with a complex outer axis copy the outputs out in column
    ranges behind the last outer transform (and the inputs in, ahead of the
    first): every output equals the device call's bit for bit, whichever
    way the inputs take, in 3D and with four outputs."""
    import torch
    from fftwpp_gb300.gpu import HybridConvolution
    kinds, L, M, mult, A, B = case
    fs = _inputs(kinds, L, A, seed=29)
    conv = HybridConvolution(kinds, L, M, A=A, B=B, mult=mult,
                             precision=precision)
    tdt = conv.dtype
    dev = [torch.from_numpy(np.ascontiguousarray(f)).to(tdt).cuda()
           for f in fs]
    want = [o.cpu().numpy() for o in conv.convolve(*dev)]
    try:
        for wi in (0, 1, 2):
            native_lib.fgb_set_host_path(wi, 0)
            h = [torch.from_numpy(np.ascontiguousarray(f)).to(tdt)
                 .pin_memory().numpy() for f in fs]
            conv.convolve_host(*h)
            for b in range(B):
                assert np.array_equal(h[b], want[b]), (wi, b)
    finally:
        native_lib.fgb_set_host_path(-1, -1)


def test_host_path_misaligned_pinned(native_lib):
    """Page-locked arrays that start off a 16-byte boundary take the copying
    path instead of failing."""
    import torch
    from fftwpp_gb300.gpu import HybridConvolution
    kinds, L, M = [H.CENTERED, H.HERMITIAN], [31, 31], [46, 46]
    fs = _inputs(kinds, L, 2, seed=29)
    want = H.convolve(fs, kinds, L, M, mult="realbinary")[0]
    conv = HybridConvolution(kinds, L, M, mult="realbinary")
    hs = []
    for f in fs:
        raw = torch.empty(f.size * 2 + 1, dtype=torch.float64).pin_memory()
        a = raw.numpy()[1:].view(np.complex128).reshape(f.shape)
        a[...] = f
        assert a.ctypes.data % 16 == 8
        hs.append(a)
    conv.convolve_host(*hs)
    assert rel_l2(hs[0], want) <= 1e-13


def _smooth(n):
    for f in (2, 3, 5, 7):
        while n % f == 0:
            n //= f
    return n == 1


@pytest.mark.parametrize("precision", ["f64", "ff", "f32"])
def test_analytic_kat_m_sweep(native_lib, precision):
    """The reference's analytic known answer (tests/hybridconv.cc:13-14,
    50-69: f_j = iF e^{ij}, g_j = iG e^{ij}, h_j = iF iG (j+1) e^{ij}) for
    L = 2^6 .. 2^12, M = 2L, every forced residue block length m the row
    kernel holds (the sweep of tests/accuracy.py:34-50)."""
    import torch
    from fftwpp_gb300.gpu import HybridConvolution
    iF, iG = np.sqrt(3) + 1j * np.sqrt(7), np.sqrt(5) + 1j * np.sqrt(11)
    tol = TOL[precision]
    checked = 0
    for e in range(6, 13):
        L = 2 ** e
        M = 2 * L
        j = np.arange(L)
        f = iF * np.exp(1j * j)
        g = iG * np.exp(1j * j)
        want = iF * iG * (j + 1) * np.exp(1j * j)
        for m in [2 ** k for k in range(2, e + 2)]:
            try:
                conv = HybridConvolution([H.PAD], [L], [M], m=[m],
                                         precision=precision)
            except ValueError:
                continue                  # beyond one CTA's shared memory
            dt = conv.dtype
            got = conv.convolve(torch.from_numpy(f).to(dt).cuda(),
                                torch.from_numpy(g).to(dt).cuda())[0]
            err = rel_l2(got.cpu().numpy().astype(np.complex128), want)
            assert err <= tol, (L, m, err)
            checked += 1
    assert checked >= 30


def test_describe_plan(native_lib):
    from fftwpp_gb300.gpu import HybridConvolution
    conv = HybridConvolution([H.CENTERED, H.HERMITIAN], [63, 63], [94, 94],
                             mult="realbinary")
    text = conv.describe()
    assert "fftPadCentered" in text and "fftPadHermitian" in text
    assert f"m={conv.axes[0]['m']}" in text and "kernels:" in text


@pytest.mark.parametrize("precision,tol", [("f64", 1e-13), ("ff", 1e-13),
                                           ("f32", 2e-6)])
def test_full_size_properties_2d(native_lib, precision, tol):
    """At the 2D benchmark size (1023 x 512 centred-Hermitian modes,
    M = 1534): linearity in each argument and symmetry, properties that hold
    at any size without an oracle run."""
    import torch
    from fftwpp_gb300.gpu import HybridConvolution
    kinds, L, M = [H.CENTERED, H.HERMITIAN], [1023, 1023], [1534, 1534]
    f, g1, g2 = _inputs(kinds, L, 3, seed=41)
    conv = HybridConvolution(kinds, L, M, mult="realbinary",
                             precision=precision)
    dt = conv.dtype

    def run(a, b):
        ta = torch.from_numpy(np.ascontiguousarray(a)).to(dt).cuda()
        tb = torch.from_numpy(np.ascontiguousarray(b)).to(dt).cuda()
        return conv.convolve(ta, tb)[0].cpu().numpy().astype(np.complex128)
    h1, h2, h12 = run(f, g1), run(f, g2), run(f, 2.0 * g1 - 0.5 * g2)
    assert rel_l2(h12, 2.0 * h1 - 0.5 * h2) <= tol
    assert rel_l2(run(g1, f), h1) <= tol


@pytest.mark.parametrize("precision,tol", [("f64", 1e-13), ("ff", 1e-13),
                                           ("f32", 2e-6)])
def test_full_size_properties_3d_real(native_lib, precision, tol):
    """At the 3D benchmark size (two 256^3 real fields, M = 511):
    linearity and symmetry."""
    import torch
    from fftwpp_gb300.gpu import HybridConvolution
    kinds, L, M = [H.REAL, H.PAD, H.PAD], [256, 256, 256], [511, 511, 511]
    rng = np.random.default_rng(43)
    f, g1, g2 = (rng.normal(size=(256, 256, 256)) for _ in range(3))
    conv = HybridConvolution(kinds, L, M, precision=precision)
    dt = conv.dtype

    def run(a, b):
        ta = torch.from_numpy(a).to(dt).cuda()
        tb = torch.from_numpy(b).to(dt).cuda()
        return conv.convolve(ta, tb)[0].cpu().numpy().astype(np.float64)
    h1 = run(f, g1)
    h12 = run(f, g1 + 3.0 * g2)
    h2 = run(f, g2)
    assert rel_l2(h12, h1 + 3.0 * h2) <= tol
    assert rel_l2(run(g1, f), h1) <= tol


@pytest.mark.parametrize("precision", ["f64", "ff", "f32"])
def test_residue_search(native_lib, precision):
    """The timed residue search may pick another m than the cost model; the
    result stays within the tolerance of the oracle either way, and with the
    search off the plan is the cost model's."""
    kinds, L, M = [H.PAD], [1024], [2047]
    fs = _inputs(kinds, L, 2, seed=47)
    want = H.convolve(fs, kinds, L, M, mult="binary")[0]
    try:
        native_lib.fgb_set_residue_search(0)
        plain, c0 = run_gpu(kinds, L, M, fs, "binary", precision)
    finally:
        native_lib.fgb_set_residue_search(1)
    searched, c1 = run_gpu(kinds, L, M, fs, "binary", precision)
    assert rel_l2(plain[0], want) <= TOL[precision]
    assert rel_l2(searched[0], want) <= TOL[precision]
    a0, a1 = c0.axes[0], c1.axes[0]
    assert a0["m"] * a0["q"] >= 2047 and a1["m"] * a1["q"] >= 2047


@pytest.mark.parametrize("case", [
    ([H.CENTERED, H.HERMITIAN], [15, 15], [22, 22], "realjacobian", 4,
     (1e150, 1e150, 1e-140, 1e-140)),
    ([H.REAL, H.PAD, H.PAD], [8, 6, 5], [15, 11, 9], "binary", 2,
     (1e-200, 1e250)),
    ([H.PAD], [300], [599], "binary", 2, (1e280, 1e-250)),
    ([H.PAD], [20000], [39999], "binary", 2, (1e-280, 1e250))])
def test_float_float_range_guard(native_lib, case):
    """Every first/last kernel family of the float-float mode (outer complex
    and real, complex and Hermitian rows, the long 1D path) with inputs far
    outside a float's range, against the oracle; without the guard the
    same inputs overflow or underflow the float exponent."""
    from fftwpp_gb300.gpu import set_ff_range_guard
    kinds, L, M, mult, A, sc = case
    fs = _inputs(kinds, L, A, seed=sum(L) + A)
    fs = [f * s for f, s in zip(fs, sc)]
    want = H.convolve(fs, kinds, L, M, mult=mult)[0]
    e = int(np.frexp(np.abs(want).max())[1])         # exact rescale
    got, _ = run_gpu(kinds, L, M, fs, mult, "ff")
    assert rel_l2(_ldexp(got[0], -e), _ldexp(want, -e)) <= 1e-13
    try:
        set_ff_range_guard(False)
        raw, _ = run_gpu(kinds, L, M, fs, mult, "ff")
    finally:
        set_ff_range_guard(True)
    assert not (rel_l2(_ldexp(raw[0], -e), _ldexp(want, -e)) <= 1e-13)



LONG_CASES = [
    ([H.CENTERED], [20001], None, 1),
    ([H.HERMITIAN], [65536], None, 1),            # hconv1d, L = 65,536
    ([H.REAL], [30000], None, 1),
    ([H.PAD], [20000], [39999], 3),               # a batch of long rows
    ([H.CENTERED, H.HERMITIAN], [15, 8191], None, 1),   # hconv2d, Ly = 8,191
    ([H.PAD, H.PAD], [6, 20000], [11, 39999], 1),
    ([H.CENTERED, H.CENTERED, H.HERMITIAN], [5, 3, 20001], None, 1),
]


@pytest.mark.parametrize("precision", ["f64", "ff", "f32"])
@pytest.mark.parametrize("case", LONG_CASES,
                         ids=lambda c: "-".join(map(str, c[0])) + "-" +
                         "x".join(map(str, c[1])) + f"-b{c[3]}")
def test_long_rows_every_kind(native_lib, case, precision):
    """Innermost rows longer than one CTA's shared memory, of every
    padded-transform kind, in 1D (also batched), 2D and 3D: the long path
    (column DFTs, rows, inverse columns through HBM) against the oracle."""
    import torch
    from fftwpp_gb300.gpu import HybridConvolution, default_M
    kinds, L, M, batch = case
    if M is None:
        M = [default_M(k, l) for k, l in zip(kinds, L)]
    mult = "realbinary" if kinds[-1] == H.HERMITIAN else "binary"
    conv = HybridConvolution(kinds, L, M, mult=mult, precision=precision,
                             batch=batch)
    if precision == "f64":
        assert conv.long_path
    probs = [_inputs(kinds, L, 2, seed=sum(L) + b) for b in range(batch)]
    dt = conv.dtype
    if batch == 1:
        ts = [torch.from_numpy(np.ascontiguousarray(f)).to(dt).cuda()
              for f in probs[0]]
    else:
        ts = [torch.from_numpy(np.stack([p[a] for p in probs])).to(dt).cuda()
              for a in range(2)]
    out = conv.convolve(*ts)[0].cpu().numpy()
    for b, fs in enumerate(probs):
        want = H.convolve(fs, kinds, L, M, mult=mult,
                          workers=os.cpu_count() or 1)[0]
        got = out if batch == 1 else out[b]
        assert rel_l2(got.astype(want.dtype), want) <= TOL[precision], b
