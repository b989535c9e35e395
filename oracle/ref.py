"""ctypes access to the compiled REFERENCE (oracle/_ref/libfftwpp_ref.so).

TEST INFRASTRUCTURE ONLY: used to generate the golden fixtures in
tests/golden/ and to pin the numpy oracle in this container.  The library is
built by oracle/Makefile from the reference's own sources plus the clean-room
FFTW3 backend; it exists only where the reference sources do, so callers must
handle ``available() == False``.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libfftwpp_ref.so")

_lib = None


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(LIB_PATH)
        sz = ctypes.c_size_t
        P = ctypes.POINTER
        _lib.ref_convolve.restype = ctypes.c_int
        _lib.ref_convolve.argtypes = [
            ctypes.c_int, P(ctypes.c_int), P(sz), P(sz), P(sz), P(sz),
            P(ctypes.c_long), sz, sz, ctypes.c_int, P(ctypes.c_double), P(sz),
            ctypes.c_int]
        _lib.ref_forward_layout.restype = ctypes.c_long
        _lib.ref_forward_layout.argtypes = [
            ctypes.c_int, sz, sz, sz, sz, ctypes.c_long,
            P(ctypes.c_double), P(ctypes.c_double), P(sz), sz, P(sz)]
        _lib.ref_forward_layout_hermitian.restype = ctypes.c_long
        _lib.ref_forward_layout_hermitian.argtypes = [
            sz, sz, sz, sz, ctypes.c_long,
            P(ctypes.c_double), P(ctypes.c_double), P(sz), sz, P(sz)]
        _lib.ref_parameters.argtypes = [sz, sz, sz, ctypes.c_int, P(sz), P(sz),
                                        P(sz)]
        _lib.ref_nextfftsize.restype = sz
        _lib.ref_nextfftsize.argtypes = [sz]
    return _lib


MULT_CODES = {"none": 0, "binary": 1, "realbinary": 2, "correlation": 3,
              "realjacobian": 4, "jacobian": 5}


def convolve(inputs, kinds, Ls, Ms, ms=None, Ds=None, Is=None,
             mult="binary", B=1, threads=1):
    """Run the reference Convolution{,2,3}; returns (outputs, info) where
    info[d] = (m, p, q, n, D, inplace) chosen by the reference."""
    dim = len(kinds)
    A = len(inputs)
    real = kinds[0] == 3
    arrs = []
    for f in inputs:
        a = np.ascontiguousarray(f, dtype=np.float64 if real else np.complex128)
        arrs.append(a)
    shape = arrs[0].shape
    words = arrs[0].size * (1 if real else 2)
    N = max(A, B)
    buf = np.zeros(N * words, dtype=np.float64)
    for a, f in enumerate(arrs):
        buf[a * words:(a + 1) * words] = f.view(np.float64).ravel()
    c_int_arr = (ctypes.c_int * dim)(*kinds)
    sz = ctypes.c_size_t
    Larr = (sz * dim)(*Ls)
    Marr = (sz * dim)(*Ms)
    marr = (sz * dim)(*(ms or [0] * dim))
    Darr = (sz * dim)(*(Ds or [0] * dim))
    Iarr = (ctypes.c_long * dim)(*(Is or [-1] * dim))
    info = (sz * (6 * dim))()
    rc = lib().ref_convolve(dim, c_int_arr, Larr, Marr, marr, Darr, Iarr, A, B,
                            MULT_CODES[mult],
                            buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                            info, threads)
    if rc != 0:
        raise RuntimeError(f"ref_convolve failed ({rc})")
    outs = []
    for b in range(B):
        v = buf[b * words:(b + 1) * words].copy()
        outs.append(v.reshape(shape) if real else v.view(np.complex128).reshape(shape))
    inf = [tuple(int(info[6 * d + k]) for k in range(6)) for d in range(dim)]
    return outs, inf


def forward_layout(kind, L, M, m=0, D=0, I=-1, f=None):
    """Forward residue blocks of a 1D fftPad/fftPadCentered and their
    transformed indices (tests/hybrid.cc:69-105)."""
    f = np.ascontiguousarray(f, dtype=np.complex128)
    cap = 8 * M + 64
    F = np.zeros(cap, dtype=np.complex128)
    idx = np.zeros(cap, dtype=np.uintp)
    info = (ctypes.c_size_t * 8)()
    n = lib().ref_forward_layout(
        kind, L, M, m, D, I, f.view(np.float64).ctypes.data_as(
            ctypes.POINTER(ctypes.c_double)),
        F.view(np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
        idx.ctypes.data_as(ctypes.POINTER(ctypes.c_size_t)), cap, info)
    if n < 0 or n > cap:
        return None
    return F[:n].copy(), idx[:n].astype(np.int64), tuple(int(x) for x in info)


def forward_layout_hermitian(L, M, m=0, D=0, I=-1, f=None):
    """Forward real blocks of a 1D fftPadHermitian and their transformed
    indices (tests/hybridh.cc:74-99); f holds the ceil(L/2) stored modes."""
    f = np.ascontiguousarray(f, dtype=np.complex128)
    cap = 8 * M + 64
    F = np.zeros(cap, dtype=np.float64)
    idx = np.zeros(cap, dtype=np.uintp)
    info = (ctypes.c_size_t * 8)()
    n = lib().ref_forward_layout_hermitian(
        L, M, m, D, I, f.view(np.float64).ctypes.data_as(
            ctypes.POINTER(ctypes.c_double)),
        F.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
        idx.ctypes.data_as(ctypes.POINTER(ctypes.c_size_t)), cap, info)
    if n < 0 or n > cap:
        return None
    return F[:n].copy(), idx[:n].astype(np.int64), tuple(int(x) for x in info)


def parameters(L, M, m, centered):
    p, n, q = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
    lib().ref_parameters(L, M, m, int(centered), ctypes.byref(p),
                         ctypes.byref(n), ctypes.byref(q))
    return p.value, n.value, q.value


def nextfftsize(m):
    return lib().ref_nextfftsize(m)
