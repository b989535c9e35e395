"""GPU: fgb_hconv2d_convolve_noalloc, the 2D centred-Hermitian FP64
convolution for callers that cannot allocate device memory (their own
allocator owns it, or an allocation would synchronise a latency-critical
loop).  It keeps all scratch in one static device array.

Checked through the C ABI against the plan-based entry point
(fgb_convolve_device) on two calls in a row, within the FP64 tolerance of the
other parity tests (1e-13 relative L2).  This file is collected last so that
a failure here does not hide the other tests; it also passes on its own."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _inputs(Lx, Ly, seed):
    from oracle import hybrid as H
    Hy = (Ly + 1) // 2
    rng = np.random.default_rng(seed)
    fs = []
    for _ in range(2):
        f = rng.uniform(-1, 1, (Lx, Hy)) + 1j * rng.uniform(-1, 1, (Lx, Hy))
        H.hermitian_symmetrize_x(f, (Lx + 1) // 2, Hy, Lx // 2)
        fs.append(f)
    return fs


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def test_noalloc_matches_plan_entry_two_calls(native_lib):
    """Two calls in a row (small, then the largest accepted size), then a
    third, small and odd-shaped, that starts on the scratch array the large
    call left dirty."""
    import torch
    from fftwpp_gb300.gpu import HybridConvolution, CENTERED, HERMITIAN
    lib = native_lib
    stream = torch.cuda.current_stream()
    for call, (Lx, Ly, seed) in enumerate([(63, 63, 1), (1023, 1023, 2),
                                           (65, 31, 3)]):
        f, g = _inputs(Lx, Ly, seed)
        tf = torch.from_numpy(f).cuda()
        tg = torch.from_numpy(g).cuda()
        th = torch.empty_like(tf)
        rc = lib.fgb_hconv2d_convolve_noalloc(
            ctypes.c_void_p(tf.data_ptr()), ctypes.c_void_p(tg.data_ptr()),
            ctypes.c_void_p(th.data_ptr()), Lx, Ly,
            ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.fgb_last_error()
        plan = HybridConvolution([CENTERED, HERMITIAN], [Lx, Ly], A=2, B=1,
                                 mult="realbinary", precision="f64")
        want = plan.convolve(tf, tg)[0]
        torch.cuda.synchronize()
        err = _rel(th.cpu().numpy(), want.cpu().numpy())
        assert err <= TOL, (call, Lx, Ly, err)


def test_noalloc_rejects_oversize(native_lib):
    import torch
    lib = native_lib
    t = torch.zeros(4, dtype=torch.complex128, device="cuda")
    p = ctypes.c_void_p(t.data_ptr())
    rc = lib.fgb_hconv2d_convolve_noalloc(p, p, p, 4095, 4095, None)
    assert rc != 0
    assert b"maximum" in lib.fgb_last_error()
