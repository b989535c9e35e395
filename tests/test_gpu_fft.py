"""GPU: the plain FFT classes (fftw++.h's fft1d ... crfft3d names) on the
shared-memory radix kernels, against numpy's FFT (called as the checker)."""
import numpy as np
import pytest

from oracle.direct import rel_l2

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-14, "f32": 2e-6}


def _c(shape, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)


def _dev(a, precision, real=False):
    import torch
    if real:
        dt = torch.float64 if precision == "f64" else torch.float32
    else:
        dt = torch.complex128 if precision == "f64" else torch.complex64
    return torch.from_numpy(np.ascontiguousarray(a)).to(dt).cuda()


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("n", [8, 60, 768, 1000, 2048])
@pytest.mark.parametrize("sign", [-1, 1])
def test_fft1d(native_lib, precision, n, sign):
    from fftwpp_gb300.fft import fft1d
    x = _c(n, n)
    got = fft1d(n, sign, precision=precision).fft(_dev(x, precision))
    want = np.fft.fft(x) if sign < 0 else np.fft.ifft(x) * n
    assert rel_l2(got.cpu().numpy(), want) <= TOL[precision]


@pytest.mark.parametrize("M,stride,dist", [(5, 1, 96), (7, 7, 1), (3, 2, 200)])
def test_mfft1d(native_lib, M, stride, dist):
    from fftwpp_gb300.fft import mfft1d
    n = 96
    t = mfft1d(n, -1, M, stride, dist)
    size = t.in_shape[0]
    x = _c(size, 3)
    got = t.fft(_dev(x, "f64")).cpu().numpy()
    for m in range(M):
        idx = m * dist + np.arange(n) * stride
        assert rel_l2(got[idx], np.fft.fft(x[idx])) <= 1e-14


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("n", [16, 250, 1536])
def test_real_1d(native_lib, precision, n):
    from fftwpp_gb300.fft import crfft1d, rcfft1d
    rng = np.random.default_rng(n)
    x = rng.normal(size=n)
    F = rcfft1d(n, precision=precision).fft(_dev(x, precision, real=True))
    assert rel_l2(F.cpu().numpy(), np.fft.rfft(x)) <= TOL[precision]
    X = np.fft.rfft(rng.normal(size=n))
    Xd = _dev(X, precision)
    y = crfft1d(n, precision=precision).fft(Xd)
    assert rel_l2(y.cpu().numpy(), np.fft.irfft(X, n) * n) <= TOL[precision]
    assert rel_l2(Xd.cpu().numpy(), X) <= TOL[precision]     # input intact


def test_multiple_real_1d(native_lib):
    from fftwpp_gb300.fft import mcrfft1d, mrcfft1d
    rng = np.random.default_rng(4)
    x = rng.normal(size=(6, 120))
    F = mrcfft1d(120, 6).fft(_dev(x, "f64", real=True)).cpu().numpy()
    assert rel_l2(F, np.fft.rfft(x, axis=1)) <= 1e-14
    y = mcrfft1d(120, 6).fft(_dev(F, "f64")).cpu().numpy()
    assert rel_l2(y / 120, x) <= 1e-14


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("nx,ny", [(8, 12), (64, 96), (250, 36)])
def test_2d(native_lib, precision, nx, ny):
    from fftwpp_gb300.fft import crfft2d, fft2d, rcfft2d
    x = _c((nx, ny), 5)
    for sign in (-1, 1):
        got = fft2d(nx, ny, sign, precision=precision).fft(_dev(x, precision))
        want = np.fft.fft2(x) if sign < 0 else np.fft.ifft2(x) * nx * ny
        assert rel_l2(got.cpu().numpy(), want) <= TOL[precision]
    r = np.random.default_rng(6).normal(size=(nx, ny))
    F = rcfft2d(nx, ny, precision=precision).fft(_dev(r, precision, True))
    assert rel_l2(F.cpu().numpy(), np.fft.rfft2(r)) <= TOL[precision]
    back = crfft2d(nx, ny, precision=precision).fftNormalized(F)
    assert rel_l2(back.cpu().numpy(), r) <= TOL[precision]


@pytest.mark.parametrize("shape", [(8, 6, 10), (32, 24, 40)])
def test_3d(native_lib, shape):
    from fftwpp_gb300.fft import crfft3d, fft3d, rcfft3d
    nx, ny, nz = shape
    x = _c(shape, 7)
    got = fft3d(nx, ny, nz, -1).fft(_dev(x, "f64")).cpu().numpy()
    assert rel_l2(got, np.fft.fftn(x)) <= 1e-14
    got = fft3d(nx, ny, nz, 1).fftNormalized(_dev(x, "f64")).cpu().numpy()
    assert rel_l2(got, np.fft.ifftn(x)) <= 1e-14
    r = np.random.default_rng(8).normal(size=shape)
    F = rcfft3d(nx, ny, nz).fft(_dev(r, "f64", True))
    assert rel_l2(F.cpu().numpy(), np.fft.rfftn(r)) <= 1e-14
    back = crfft3d(nx, ny, nz).fftNormalized(F).cpu().numpy()
    assert rel_l2(back, r) <= 1e-14


def test_in_place_complex(native_lib):
    from fftwpp_gb300.fft import fft2d
    x = _c((48, 40), 9)
    t = _dev(x, "f64")
    fft2d(48, 40, -1).fft(t, out=t)
    assert rel_l2(t.cpu().numpy(), np.fft.fft2(x)) <= 1e-14


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("n", [1 << 16, 3 * 5 * 7 * 1024, 1 << 20])
@pytest.mark.parametrize("sign", [-1, 1])
def test_fft1d_two_pass(native_lib, precision, n, sign):
    """Lengths beyond one CTA (two passes through the plan's scratch
    array, the four-step FFT), both signs, in place too."""
    from fftwpp_gb300.fft import fft1d
    x = _c(n, n % 97)
    t = fft1d(n, sign, precision=precision)
    assert t.passes[0].handle
    got = t.fft(_dev(x, precision))
    want = np.fft.fft(x) if sign < 0 else np.fft.ifft(x) * n
    tol = 1e-13 if precision == "f64" else 4e-6
    assert rel_l2(got.cpu().numpy(), want) <= tol
    d = _dev(x, precision)
    t.fft(d, out=d)
    assert rel_l2(d.cpu().numpy(), want) <= tol


def test_mfft1d_two_pass(native_lib):
    """Several long contiguous sequences (dist beyond n)."""
    from fftwpp_gb300.fft import mfft1d
    n, M, dist = 1 << 15, 3, (1 << 15) + 64
    t = mfft1d(n, 1, M, 1, dist)
    x = _c(t.in_shape[0], 4)
    got = t.fft(_dev(x, "f64")).cpu().numpy()
    for m in range(M):
        idx = m * dist + np.arange(n)
        assert rel_l2(got[idx], np.fft.ifft(x[idx]) * n) <= 1e-13


def _shift(r):
    """fftw::Shift of the real side: (-1)^(i (+ j))."""
    i = np.arange(r.shape[0])[:, None]
    if r.ndim == 2:
        return r * (-1.0) ** i
    j = np.arange(r.shape[1])[None, :]
    return r * ((-1.0) ** (i + j))[:, :, None]


@pytest.mark.parametrize("shape", [(8, 12), (64, 30), (8, 6, 10)])
def test_fft0_origin_shift(native_lib, shape):
    """fft0 of rcfft2d/rcfft3d: the Fourier origin at (nx/2, 0) or
    (nx/2, ny/2, 0), i.e. the transform of the shifted input; crfft fft0
    undoes it; the classes without a shift ignore it."""
    from fftwpp_gb300 import fft as F
    r = np.random.default_rng(2).normal(size=shape)
    if len(shape) == 2:
        fwd, bwd = F.rcfft2d(*shape), F.crfft2d(*shape)
        want = np.fft.rfft2(_shift(r))
    else:
        fwd, bwd = F.rcfft3d(*shape), F.crfft3d(*shape)
        want = np.fft.rfftn(_shift(r))
    d = _dev(r, "f64", True)
    got = fwd.fft0(d)
    assert rel_l2(got.cpu().numpy(), want) <= 1e-14
    assert rel_l2(d.cpu().numpy(), _shift(r)) == 0     # shifted in place
    back = bwd.fft0Normalized(got).cpu().numpy()
    assert rel_l2(back, r) <= 1e-14
    c = F.fft2d(8, 12, -1)
    x = _c((8, 12), 3)
    assert rel_l2(c.fft0(_dev(x, "f64")).cpu().numpy(), np.fft.fft2(x)) <= 1e-14
    with pytest.raises(ValueError):
        F.rcfft2d(7, 12).fft0(_dev(np.zeros((7, 12)), "f64", True))
