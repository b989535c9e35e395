"""GPU: multipliers written by the caller as device functors
(include/fftwpp_gb300_mult.cuh), the counterpart of the reference's user
multiplier hook with its Indices (convolve.h:48-82).  tests/cpp/user_mult.cu
is compiled here with nvcc into a shared library linked to lib_fftwpp.so;
its functors run inside the library's row kernels.

Checks: the Jacobian written as a functor against the oracle's Jacobian at
the benchmark size (1023 x 512 modes, FP64, 1e-13); position-dependent
functors against the explicit N-grid oracle (oracle/explicit.py) on every
padded-transform kind and dimension, in FP64, float-float (1e-13) and FP32
(2e-6), through the device and the host entries; plan misuse is refused."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from oracle import explicit as E
from oracle import hybrid as H
from oracle.direct import rel_l2

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOL = {"f64": 1e-13, "ff": 1e-13, "f32": 2e-6}


@pytest.fixture(scope="module")
def user_lib(native_lib, tmp_path_factory):
    out = str(tmp_path_factory.mktemp("user") / "libuser_mult.so")
    libdir = os.path.join(ROOT, "fftwpp_gb300")
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
           "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
           "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "user_mult.cu"),
           "-L", libdir, "-l_fftwpp", "-Xlinker", "-rpath=" + libdir,
           "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    lib = ctypes.CDLL(out)
    vp = ctypes.c_void_p
    for name in ("user_jacobian_device", "user_weighted_device",
                 "user_mixed_device"):
        getattr(lib, name).argtypes = [vp, ctypes.POINTER(vp),
                                       ctypes.POINTER(vp), vp]
        getattr(lib, name).restype = ctypes.c_int
    lib.user_weighted_host.argtypes = [vp, ctypes.POINTER(vp),
                                       ctypes.POINTER(vp)]
    lib.user_weighted_host.restype = ctypes.c_int
    return lib


def _inputs(kinds, L, A, seed):
    rng = np.random.default_rng(seed)
    shape = [(l + 1) // 2 if k == H.HERMITIAN else l for k, l in zip(kinds, L)]
    fs = []
    for _ in range(A):
        if kinds[0] == H.REAL:
            f = rng.normal(size=shape)
        else:
            f = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
        if kinds[-1] == H.HERMITIAN:
            if len(kinds) == 1:
                f[0] = f[0].real
            elif len(kinds) == 2:
                H.hermitian_symmetrize_x(f, (L[0] + 1) // 2, shape[1],
                                         L[0] // 2)
            else:
                H.hermitian_symmetrize_xy(f, (L[0] + 1) // 2,
                                          (L[1] + 1) // 2, shape[2],
                                          L[0] // 2, L[1] // 2)
        fs.append(f)
    return fs


def _run(fn, kinds, L, M, fs, B, precision, m=None):
    import torch
    from fftwpp_gb300.gpu import HybridConvolution
    conv = HybridConvolution(kinds, L, M, m=m, A=len(fs), B=B, mult="user",
                             precision=precision)
    ts = [torch.from_numpy(np.ascontiguousarray(f)).to(conv.dtype).cuda()
          for f in fs]
    outs = [torch.empty_like(ts[0]) for _ in range(B)]
    vp = ctypes.c_void_p
    pin = (vp * len(ts))(*[t.data_ptr() for t in ts])
    pout = (vp * B)(*[t.data_ptr() for t in outs])
    rc = fn(vp(conv.handle), pin, pout,
            vp(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, conv.lib.fgb_last_error()
    torch.cuda.synchronize()
    return [o.cpu().numpy().astype(np.complex128 if not conv.real
                                   else np.float64) for o in outs], conv


def _weighted_oracle(fs, kinds, L, Ns):
    def mult(v, ix):
        w = 1.0
        for d, k in enumerate(ix):
            w = w + 0.25 * (d + 1) * np.cos(2 * np.pi * k / Ns[d])
        return [v[0] * v[1] * w]
    return E.convolve(fs, kinds, L, Ns, mult)[0]


def test_jacobian_functor_full_size(user_lib):
    """The Jacobian as a caller's functor (instantiated for FP64 only) on
    the advection workload's size matches the oracle's built-in Jacobian
    (the functor sees one real value per grid point, as the reference's
    real multipliers do)."""
    precision = "f64"
    kinds, L = [H.CENTERED, H.HERMITIAN], [1023, 1023]
    M = [1534, 1534]
    fs = _inputs(kinds, L, 4, seed=61)
    want = H.convolve(fs, kinds, L, M, mult="realjacobian",
                      workers=os.cpu_count() or 1)[0]
    got, _ = _run(user_lib.user_jacobian_device, kinds, L, M, fs, 1,
                  precision)
    assert rel_l2(got[0], want) <= 1e-13


CASES = [
    ([H.PAD], [300], [599], None),
    ([H.PAD], [40], [79], [16]),                 # residues (q > 1)
    ([H.CENTERED], [41], [61], [8]),
    ([H.HERMITIAN], [63], [94], None),
    ([H.REAL], [50], [99], None),
    ([H.PAD], [20000], [39999], None),           # long 1D path
    ([H.PAD, H.PAD], [24, 20], [47, 39], None),
    ([H.CENTERED, H.HERMITIAN], [63, 63], [94, 94], None),
    ([H.CENTERED, H.HERMITIAN], [31, 31], [46, 46], [8, 0]),
    ([H.REAL, H.PAD], [16, 15], [31, 29], None),
    ([H.REAL, H.PAD, H.PAD], [12, 10, 9], [23, 19, 17], None),
    ([H.CENTERED, H.CENTERED, H.HERMITIAN], [9, 7, 9], [13, 10, 13], None),
    ([H.CENTERED, H.HERMITIAN], [7, 8191], [10, 12286], None),  # long rows
]


def _cid(c):
    names = {0: "pad", 1: "cen", 2: "her", 3: "real"}
    return ("-".join(names[k] for k in c[0]) + "-" +
            "x".join(map(str, c[1])) + ("-m" if c[3] else ""))


@pytest.mark.parametrize("precision", ["f64", "ff", "f32"])
@pytest.mark.parametrize("case", CASES, ids=[_cid(c) for c in CASES])
def test_position_dependent_functor(user_lib, case, precision):
    """w(x) f g with w a smooth function of every axis' transformed index:
    the functor receives each point's position on the padded grid of the
    GPU plan, digit-reversed transform orders and residue blocks
    included."""
    kinds, L, M, m = case
    fs = _inputs(kinds, L, 2, seed=sum(L) + 1)
    got, conv = _run(user_lib.user_weighted_device, kinds, L, M, fs, 1,
                     precision, m=m)
    Ns = [ax["N"] for ax in conv.axes]
    want = _weighted_oracle(fs, kinds, L, Ns)
    assert rel_l2(got[0], want) <= TOL[precision], (Ns, conv.axes)


@pytest.mark.parametrize("precision", ["f64", "ff"])
def test_three_output_functor(user_lib, precision):
    """A=3, B=3 functor whose outputs weight different axes."""
    for kinds, L, M in (([H.CENTERED, H.HERMITIAN], [15, 15], [22, 22]),
                        ([H.PAD, H.PAD, H.PAD], [6, 5, 7], [11, 9, 13])):
        fs = _inputs(kinds, L, 3, seed=7)
        got, conv = _run(user_lib.user_mixed_device, kinds, L, M, fs, 3,
                         precision)
        Ns = [ax["N"] for ax in conv.axes]

        def mult(v, ix):
            x = ix[0] / Ns[0]
            y = ix[-1] / Ns[-1]
            return [v[0] * v[1] * (1 + x), v[1] * v[2] * (2 - y),
                    v[0] * v[2]]
        want = E.convolve(fs, kinds, L, Ns, mult)
        for b in range(3):
            assert rel_l2(got[b], want[b]) <= TOL[precision], (kinds, b)


def test_functor_host_entry(user_lib):
    """The host-array entry (fgb_convolve_host_with) gives the device
    entry's result."""
    import torch
    from fftwpp_gb300.gpu import HybridConvolution
    kinds, L, M = [H.CENTERED, H.HERMITIAN], [31, 31], [46, 46]
    fs = _inputs(kinds, L, 2, seed=3)
    dev, conv = _run(user_lib.user_weighted_device, kinds, L, M, fs, 1,
                     "f64")
    hs = [torch.from_numpy(f.copy()).pin_memory().numpy() for f in fs]
    vp = ctypes.c_void_p
    pin = (vp * 2)(*[h.ctypes.data for h in hs])
    rc = user_lib.user_weighted_host(vp(conv.handle), pin, pin)
    assert rc == 0, conv.lib.fgb_last_error()
    assert rel_l2(hs[0], dev[0]) <= 1e-15


def test_functor_plan_misuse(user_lib):
    """A functor on a built-in plan, a plan of the wrong arity, a precision
    the functor was not instantiated for, and a user plan through the
    built-in entry are all refused with an error (nothing launches)."""
    import torch
    from fftwpp_gb300.gpu import HybridConvolution
    vp = ctypes.c_void_p
    kinds, L = [H.PAD], [64]
    t = torch.zeros(64, dtype=torch.complex128, device="cuda")
    ptr = (vp * 4)(*([t.data_ptr()] * 4))
    s = vp(torch.cuda.current_stream().cuda_stream)
    builtin = HybridConvolution(kinds, L, mult="binary")
    assert user_lib.user_weighted_device(vp(builtin.handle), ptr, ptr, s) == -1
    assert b"built-in" in builtin.lib.fgb_last_error()
    three = HybridConvolution(kinds, L, A=3, B=1, mult="user")
    assert user_lib.user_weighted_device(vp(three.handle), ptr, ptr, s) == -1
    assert b"(A, B)" in three.lib.fgb_last_error()
    f32 = HybridConvolution(kinds, L, A=4, B=1, mult="user", precision="f32")
    t32 = torch.zeros(64, dtype=torch.complex64, device="cuda")
    p32 = (vp * 4)(*([t32.data_ptr()] * 4))
    assert user_lib.user_jacobian_device(vp(f32.handle), p32, p32, s) != 0
    plan = HybridConvolution(kinds, L, mult="user")
    with pytest.raises(RuntimeError):
        plan.convolve(t, t)


def test_functor_through_cpp_classes(user_lib):
    """The functor as the Application multiplier of the FFTW++-compatible
    C++ classes (include/convolve.h: Convolution2 over fftPadCentered x
    fftPadHermitian, host arrays with an x stride beyond the stored rows)."""
    fn = user_lib.cpp_weighted_her2
    dp = ctypes.POINTER(ctypes.c_double)
    fn.argtypes = [dp, dp, dp, ctypes.c_size_t, ctypes.c_size_t,
                   ctypes.c_size_t, ctypes.POINTER(ctypes.c_long)]
    fn.restype = ctypes.c_int
    kinds, L = [H.CENTERED, H.HERMITIAN], [31, 31]
    fs = _inputs(kinds, L, 2, seed=19)
    h = np.empty_like(fs[0])
    N = (ctypes.c_long * 2)()
    args = [np.ascontiguousarray(a).ctypes.data_as(dp) for a in (fs[0], fs[1])]
    assert fn(args[0], args[1], h.ctypes.data_as(dp), 31, 31, 16 + 4, N) == 0
    want = _weighted_oracle(fs, kinds, L, [N[0], N[1]])
    assert rel_l2(h, want) <= 1e-13
