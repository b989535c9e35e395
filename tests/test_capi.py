"""CPU: the C-ABI library loads, exports every symbol include/*.h declares,
and its host-side integer rules match the reference's (golden fixtures).
No compute call is made here; creating a plan without a GPU must fail loudly
(there is no CPU fallback)."""
import ctypes
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_exports_every_declared_symbol(native_lib):
    from fftwpp_gb300 import _native
    syms = _native.header_symbols()
    assert len(syms) >= 35
    missing = [s for s in syms if not hasattr(native_lib, s)]
    assert not missing, missing


def test_reference_abi_names_present(native_lib):
    # wrappers/cfftw++.cc:27-163
    for name in ["create_doubleAlign", "delete_doubleAlign",
                 "create_complexAlign", "delete_complexAlign",
                 "get_fftwpp_maxthreads", "set_fftwpp_maxthreads",
                 "fftwpp_create_conv1d", "fftwpp_conv1d_convolve",
                 "fftwpp_conv1d_delete", "fftwpp_create_hconv1d",
                 "fftwpp_hconv1d_convolve", "fftwpp_hconv1d_delete",
                 "fftwpp_HermitianSymmetrize", "fftwpp_create_conv2d",
                 "fftwpp_conv2d_convolve", "fftwpp_conv2d_delete",
                 "fftwpp_HermitianSymmetrizeX", "fftwpp_create_hconv2d",
                 "fftwpp_hconv2d_convolve", "fftwpp_hconv2d_delete",
                 "fftwpp_create_conv3d", "fftwpp_conv3d_convolve",
                 "fftwpp_conv3d_delete", "fftwpp_HermitianSymmetrizeXY",
                 "fftwpp_create_hconv3d", "fftwpp_hconv3d_convolve",
                 "fftwpp_hconv3d_delete"]:
        assert hasattr(native_lib, name), name


def test_maxthreads_roundtrip(native_lib):
    old = native_lib.get_fftwpp_maxthreads()
    native_lib.set_fftwpp_maxthreads(7)
    assert native_lib.get_fftwpp_maxthreads() == 7
    native_lib.set_fftwpp_maxthreads(old)


def test_parameters_match_reference(native_lib):
    p = np.load(os.path.join(GOLD, "params.npz"))
    sz = ctypes.c_size_t
    a, b, c = sz(), sz(), sz()
    for L, M, m, cen, pp, nn, qq in p["parameters"][::7]:
        native_lib.fgb_parameters(int(L), int(M), int(m), int(cen),
                                  ctypes.byref(a), ctypes.byref(b),
                                  ctypes.byref(c))
        assert (a.value, b.value, c.value) == (pp, nn, qq)
    for m, n in p["nextfftsize"]:
        assert native_lib.fgb_nextfftsize(int(m)) == n


def test_index_matches_reference(native_lib):
    """fgb_index reproduces fftBase::index on every golden layout."""
    from test_oracle import LAYOUTS, layout_stream
    for lay in LAYOUTS:
        stream, (m, p, q, n, D, D0, centered) = layout_stream(lay)
        kind = 1 if centered else 0
        got = [native_lib.fgb_index(kind, m, p, q, n, D, r, k)
               for r, k in stream]
        assert np.array_equal(np.array(got), lay["idx"]), lay["key"]


def _radices(lib, n, prec, inplace, wide):
    buf = (ctypes.c_int * 32)()
    k = lib.fgb_fft_radices(n, prec, int(inplace), int(wide), buf, 32)
    return None if k < 0 else list(buf[:k])


def test_fft_radix_plans(native_lib):
    """The shared-memory transforms' radix sequences: every product equals
    the length, the in-place form puts odd radices (and the radix 6) first
    so every later span is a power of two, and radix 16 / 6 appear only in
    wide FP32 plans, where they save a stage."""
    from fftwpp_gb300._native import PRECISIONS
    f64, f32, ff = PRECISIONS["f64"], PRECISIONS["f32"], PRECISIONS["ff"]
    lengths = [n for n in range(1, 5000)
               if native_lib.fgb_nextfftsize(n) == n]
    for n in lengths:
        for prec in (f64, f32, ff):
            for inplace in (0, 1):
                for wide in (0, 1):
                    r = _radices(native_lib, n, prec, inplace, wide)
                    assert r is not None and int(np.prod(r)) == n, (n, r)
                    w = wide and inplace and prec == f32
                    assert set(r) <= ({2, 3, 4, 5, 6, 7, 8, 16} if w else
                                      {2, 3, 4, 5, 7, 8}), (n, prec, r)
                    if inplace:
                        span = n
                        for k, R in enumerate(r):
                            span //= R
                            if R % 2 == 0 and R != 6:
                                assert all(x % 2 == 0 and x != 6
                                           for x in r[k:]), r
                        assert span == 1
                    if w:
                        base = _radices(native_lib, n, prec, 1, 0)
                        assert len(r) <= len(base), (n, r, base)
                        if 16 in r or 6 in r:
                            assert len(r) < len(base), (n, r, base)
    assert _radices(native_lib, 768, f32, 1, 1) == [3, 16, 16]
    assert _radices(native_lib, 1536, f32, 1, 1) == [6, 16, 16]
    assert _radices(native_lib, 2048, f32, 1, 1) == [16, 16, 8]
    assert _radices(native_lib, 512, f32, 1, 1) == [8, 8, 8]
    assert _radices(native_lib, 768, f64, 0, 0) == [8, 8, 4, 3]
    assert _radices(native_lib, 768, ff, 1, 1) == [3, 8, 8, 4]
    assert _radices(native_lib, 11, f64, 0, 0) is None


def test_hermitian_symmetrize_host(native_lib):
    """fftwpp_HermitianSymmetrizeX/XY agree with the oracle's restatement
    of convolve.h:1175-1258."""
    from oracle import hybrid as H
    rng = np.random.default_rng(4)
    for Lx, Hy in ((7, 4), (8, 5)):
        f = rng.normal(size=(Lx, Hy)) + 1j * rng.normal(size=(Lx, Hy))
        g = f.copy()
        native_lib.fftwpp_HermitianSymmetrizeX((Lx + 1) // 2, Hy, Lx // 2,
                                               ctypes.c_void_p(f.ctypes.data))
        H.hermitian_symmetrize_x(g, (Lx + 1) // 2, Hy, Lx // 2)
        assert np.array_equal(f, g)
    for Lx, Ly, Hz in ((5, 5, 3), (6, 4, 2)):
        f = rng.normal(size=(Lx, Ly, Hz)) + 1j * rng.normal(size=(Lx, Ly, Hz))
        g = f.copy()
        native_lib.fftwpp_HermitianSymmetrizeXY(
            (Lx + 1) // 2, (Ly + 1) // 2, Hz, Lx // 2, Ly // 2,
            ctypes.c_void_p(f.ctypes.data))
        H.hermitian_symmetrize_xy(g, (Lx + 1) // 2, (Ly + 1) // 2, Hz,
                                  Lx // 2, Ly // 2)
        assert np.array_equal(f, g)


def test_no_cpu_fallback(native_lib):
    """Without a GPU, planning fails with an error instead of computing on
    the host."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    sz = ctypes.c_size_t
    k = (ctypes.c_int * 1)(0)
    L = (sz * 1)(16)
    M = (sz * 1)(31)
    h = native_lib.fgb_create(1, k, L, M, None, 2, 1, 1, 0, 1)
    assert not h
    from fftwpp_gb300 import _native
    assert _native.last_error()


def test_missing_library_is_loud(tmp_path, monkeypatch):
    from fftwpp_gb300 import _native
    monkeypatch.setattr(_native, "LIB_PATH", str(tmp_path / "absent.so"))
    monkeypatch.setattr(_native, "_lib", None)
    with pytest.raises(_native.NativeLibraryMissing):
        _native.load()


def test_padded_transform_plans(native_lib):
    """Standalone padded-transform plans (host-side planning only)."""
    from fftwpp_gb300 import _native
    lib = native_lib
    info = (ctypes.c_long * 10)()
    for kind, L, M, C, m in [(0, 1000, 1999, 4, 0), (1, 63, 94, 3, 0),
                             (0, 64, 127, 1, 16), (1, 31, 46, 2, 8),
                             (3, 100, 199, 5, 0)]:
        h = lib.fgb_pad_create(kind, L, M, C, m, 0)
        assert h, _native.last_error()
        try:
            assert lib.fgb_pad_info(h, info) == 0
            mm, p, q, N, LL, CC, rows, c = list(info)[:8]
            assert (LL, CC) == (L, C) and N >= M
            if kind == 3:
                assert rows == N // 2 + 1 and q == 1
                assert lib.fgb_pad_index(h, 0, 7) == 7
            else:
                assert mm * q == N and rows == N and p == -(-L // mm)
                if m:
                    assert mm == m
                assert c == (L // 2 if kind == 1 else 0)
                assert lib.fgb_pad_index(h, 1, 5) == q * 5 + 1
        finally:
            lib.fgb_pad_destroy(h)
    h = lib.fgb_pad_create(2, 15, 22, 3, 0, 0)     # fftPadHermitian
    assert h, _native.last_error()
    try:
        assert lib.fgb_pad_info(h, info) == 0
        mm, p, q, N, LL, CC, rows, c = list(info)[:8]
        assert (q, N % 2, rows, mm) == (1, 0, N, N) and N >= 22
        assert lib.fgb_pad_index(h, 0, 7) == 7
    finally:
        lib.fgb_pad_destroy(h)
    assert not lib.fgb_pad_create(7, 16, 24, 1, 0, 0)
    assert "kind" in _native.last_error()
    assert not lib.fgb_pad_create(0, 16, 8, 1, 0, 0)
    assert "greater than M" in _native.last_error()


def test_plain_fft_plans(native_lib):
    """Plain FFT plans are validated on the host (no GPU needed)."""
    from fftwpp_gb300 import _native
    lib = native_lib
    ok = lib.fgb_fft_create(0, 768, -1, 4, 3, 4, 3072, 4, 3072, 0)
    assert ok
    lib.fgb_fft_destroy(ok)
    for args, msg in [((0, 11, -1, 1, 1, 1, 11, 1, 11, 0), "product of 2"),
                      ((1, 30, -1, 1, 1, 1, 30, 1, 16, 0), None),
                      ((1, 15, -1, 1, 1, 1, 15, 1, 8, 0), "even length"),
                      ((0, 16, 2, 1, 1, 1, 16, 1, 16, 0), "sign"),
                      ((0, 16, 1, 8, 1, 4, 0, 8, 0, 0), "stride >= C"),
                      ((0, 16, 1, 1, 1, 1, 16, 1, 16, 2), "FP64 or FP32"),
                      ((1, 1 << 16, -1, 1, 1, 1, 1 << 16, 1, 1, 0),
                       "too long"),
                      ((0, 1 << 16, 1, 2, 1, 2, 0, 2, 0, 0), "too long")]:
        h = lib.fgb_fft_create(*args)
        if msg is None:
            assert h
            lib.fgb_fft_destroy(h)
        else:
            assert not h
            assert msg in _native.last_error(), _native.last_error()


def test_misaligned_arrays_refused(native_lib):
    """Transform entry points refuse arrays that are not aligned to their
    element size before anything reaches the GPU (the kernels' vector
    accesses would fault on them)."""
    from fftwpp_gb300 import _native
    lib = native_lib
    t = lib.fgb_pad_create(0, 64, 127, 1, 0, 0)
    try:
        assert lib.fgb_pad_forward_device(t, 4096 + 8, 8192, None) == -1
        assert "aligned" in _native.last_error()
        assert lib.fgb_pad_backward_device(t, 4096, 8192 + 8, None) == -1
    finally:
        lib.fgb_pad_destroy(t)
    f = lib.fgb_fft_create(1, 64, -1, 1, 1, 1, 64, 1, 33, 0)     # r2c FP64
    try:
        assert lib.fgb_fft_execute_device(f, 4096 + 4, 8192, None) == -1
        assert "aligned" in _native.last_error()
        assert lib.fgb_fft_execute_device(f, 4096 + 8, 8192 + 8, None) == -1
    finally:
        lib.fgb_fft_destroy(f)
    assert lib.fgb_hconv2d_convolve_noalloc(4096 + 8, 8192, 12288, 63, 63,
                                            None) != 0
    assert "aligned" in _native.last_error()


def test_drop_in_precision_switch(native_lib):
    lib = native_lib
    assert lib.fgb_get_drop_in_precision() == 0
    assert lib.fgb_set_drop_in_precision(1) == -1        # FP32 arrays differ
    assert lib.fgb_set_drop_in_precision(2) == 0
    assert lib.fgb_get_drop_in_precision() == 2
    assert lib.fgb_set_drop_in_precision(0) == 0
    assert lib.fgb_get_drop_in_precision() == 0


def test_python_switches(native_lib):
    """The process-wide planning switches are reachable from Python and
    validate their arguments (no GPU work)."""
    from fftwpp_gb300 import gpu
    gpu.set_autotune(True)
    gpu.set_residue_search(True)
    gpu.set_host_path(-1, -1)
    with pytest.raises(ValueError):
        gpu.set_host_path(3, 0)


def _reference_wrapper_dir():
    ref = (os.environ.get("FFTWPP_REFERENCE") or
           os.path.join(os.sep, "root", "reference"))
    path = os.path.join(ref, "wrappers", "fftwpp.py")
    return path if os.path.exists(path) else None


def test_unchanged_reference_wrapper_binds(native_lib, tmp_path):
    """The reference's own wrappers/fftwpp.py, unmodified, loads this
    library from its own directory and binds every prototype it declares;
    its thread-count calls and host-side Hermitian symmetrisers run (no GPU
    needed) and agree with the oracle.  Skipped where the reference
    checkout is absent (it is not shipped with this package)."""
    import importlib.util
    import shutil
    from fftwpp_gb300 import _native
    from oracle import hybrid as H
    src = _reference_wrapper_dir()
    if src is None:
        pytest.skip("reference checkout not present")
    shutil.copy(src, tmp_path / "fftwpp.py")
    os.symlink(_native.LIB_PATH, tmp_path / "lib_fftwpp.so")
    spec = importlib.util.spec_from_file_location("ref_fftwpp",
                                                  tmp_path / "fftwpp.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    assert hasattr(mod, "Convolution") and hasattr(mod, "HConvolution")
    old = mod.fftwpp_get_maxthreads()
    mod.fftwpp_set_maxthreads(3)
    assert mod.fftwpp_get_maxthreads() == 3
    mod.fftwpp_set_maxthreads(old)
    rng = np.random.default_rng(8)
    Lx, Hy = 9, 5
    f = mod.complex_align([Lx, Hy])
    f[...] = rng.normal(size=(Lx, Hy)) + 1j * rng.normal(size=(Lx, Hy))
    g = f.copy()
    mod.clib.fftwpp_HermitianSymmetrizeX((Lx + 1) // 2, Hy, Lx // 2, f)
    H.hermitian_symmetrize_x(g, (Lx + 1) // 2, Hy, Lx // 2)
    assert np.array_equal(f, g)
