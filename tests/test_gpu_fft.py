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
