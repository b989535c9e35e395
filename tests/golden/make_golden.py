"""Generate the golden fixtures in tests/golden/ from the REFERENCE itself.

Runs FFTW++'s own Convolution / Convolution2 / Convolution3 (compiled from
the reference sources by oracle/Makefile into oracle/_ref/libfftwpp_ref.so,
linked against the clean-room FFTW3 backend) on:

* the reference tests' deterministic integer inputs
  (tests/hybridconv.cc:60, hybridconvh.cc:49, hybridconvr.cc:46,
  hybridconv2.cc:55, hybridconvh2.cc:58-61, hybridconvr2.cc:55,
  hybridconv3.cc:61-62, hybridconvh3.cc:67-68, hybridconvr3.cc:61)
  over parameter grids in the spirit of tests/tests.py:561-653, with the
  residue block m, residues per pass D and in-place flag I forced so that
  every forward/backward routine family is exercised;
* seeded uniform/normal inputs;
* the analytic known-answer case of tests/hybridconv.cc:50-69;
* forward residue layouts and transformed indices (tests/hybrid.cc:69-105),
  and the real forward blocks of fftPadHermitian with theirs
  (tests/hybridh.cc:74-99; `--only hlayouts` regenerates just these);
* the parameter rule and nextfftsize over a grid.

Usage (in a checkout where the reference and oracle/_ref exist):
    make -C oracle && python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref  # noqa: E402

PAD, CEN, HER, REAL = 0, 1, 2, 3


def det_inputs(kinds, L, A):
    """The reference tests' integer-valued inputs."""
    dim = len(kinds)
    fs = []
    if dim == 1:
        n = (L[0] + 1) // 2 if kinds[0] == HER else L[0]
        j = np.arange(n)
        for a in range(A):
            if kinds[0] == REAL:
                fs.append((j + a + 1).astype(np.float64))
            else:
                f = (j + a + 1) + 1j * ((a + 1) * j + 3)
                if kinds[0] == HER:
                    f[0] = f[0].real
                fs.append(f.astype(np.complex128))
        return fs
    if dim == 2:
        Lx, Ly = L
        ny = (Ly + 1) // 2 if kinds[1] == HER else Ly
        i = np.arange(Lx)[:, None]
        j = np.arange(ny)[None, :]
        for a in range(A):
            if kinds[0] == REAL:
                fs.append((i + a * j + 1).astype(np.float64))
            elif kinds[1] == HER:
                I = i if Lx % 2 else i - 1
                f = (I + a + 1) + 1j * ((a + 1) * j + 3) + 0 * i
                f = f.astype(np.complex128)
                symmetrize_x(f, (Lx + 1) // 2, ny, Lx // 2)
                fs.append(f)
            else:
                fs.append(((i + a + 1) + 1j * ((a + 1) * j + 3)).astype(
                    np.complex128))
        return fs
    Lx, Ly, Lz = L
    nz = (Lz + 1) // 2 if kinds[2] == HER else Lz
    i = np.arange(Lx)[:, None, None]
    j = np.arange(Ly)[None, :, None]
    k = np.arange(nz)[None, None, :]
    for a in range(A):
        if kinds[0] == REAL:
            fs.append((i + (a + 1) * j + a * k + 1).astype(np.float64))
        elif kinds[2] == HER:
            I = i if Lx % 2 else i - 1
            J = j if Ly % 2 else j - 1
            f = ((I + a * k + 1) + 1j * ((a + 1) * J + 3 + k)).astype(
                np.complex128)
            symmetrize_xy(f, (Lx + 1) // 2, (Ly + 1) // 2, nz, Lx // 2, Ly // 2)
            fs.append(f)
        else:
            fs.append(((i + a * k + 1) + 1j * ((a + 1) * j + 3 + k)).astype(
                np.complex128))
    return fs


def symmetrize_x(f, Hx, Hy, x0):
    for i in range(1, Hx):
        f[x0 - i, 0] = np.conj(f[x0 + i, 0])
    f[x0, 0] = f[x0, 0].real
    if x0 == Hx:
        f[0, :] = 0


def symmetrize_xy(f, Hx, Hy, Hz, x0, y0):
    for i in range(1, Hx):
        f[x0 - i, y0, 0] = np.conj(f[x0 + i, y0, 0])
    f[x0, y0, 0] = f[x0, y0, 0].real
    for i in range(-Hx + 1, Hx):
        for j in range(1, Hy):
            f[x0 - i, y0 - j, 0] = np.conj(f[x0 + i, y0 + j, 0])
    if x0 == Hx:
        f[0, :y0 + Hy, :] = 0
    if y0 == Hy:
        f[:x0 + Hx, 0, :] = 0


def rand_inputs(kinds, L, A, seed):
    rng = np.random.default_rng(seed)
    shape = list(L)
    if kinds[-1] == HER:
        shape[-1] = (L[-1] + 1) // 2
    fs = []
    for _ in range(A):
        if kinds[0] == REAL:
            f = rng.normal(size=shape)
        else:
            f = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
        if kinds[-1] == HER:
            if len(kinds) == 1:
                f[0] = f[0].real
            elif len(kinds) == 2:
                symmetrize_x(f, (L[0] + 1) // 2, shape[1], L[0] // 2)
            else:
                symmetrize_xy(f, (L[0] + 1) // 2, (L[1] + 1) // 2, shape[2],
                              L[0] // 2, L[1] // 2)
        fs.append(f)
    return fs


def mult_for(kinds):
    return "realbinary" if kinds[-1] == HER else "binary"


def conv_cases():
    cases = []
    # 1D grids (tests/tests.py:561-653): complex L=8, M in {16,20},
    # m in {M, L+1, L, L/2, L/4}, D in {1,2,4}, I in {0,1}.
    for M in (16, 20):
        for m in (M, 9, 8, 4, 2):
            for D in (1, 2, 4):
                for I in (0, 1):
                    cases.append(([PAD], [8], [M], [m], [D], [I]))
    for (L, M) in ((8, 16), (9, 13), (8, 12), (7, 10)):
        for m in (M, L, (L + 1) // 2, 4, 2):
            for D in (1, 2):
                for I in (0, 1):
                    cases.append(([CEN], [L], [M], [m], [D], [I]))
    for (L, M) in ((8, 12), (7, 10), (15, 22), (16, 24)):
        for m in (M, (L + 1) // 2, 4, 2):
            for D in (1, 2):
                for I in (0, 1):
                    cases.append(([HER], [L], [M], [m], [D], [I]))
    for (L, M) in ((8, 16), (9, 17), (12, 23)):
        for m in (M, L, (L + 1) // 2, 4, 3, 2):
            for D in (1, 2):
                for I in (0, 1):
                    cases.append(([REAL], [L], [M], [m], [D], [I]))
    # Optimizer-chosen parameters.
    for kinds, L, M in (
            ([PAD], [64], [127]), ([CEN], [63], [94]), ([HER], [63], [94]),
            ([REAL], [64], [127]), ([PAD], [1024], [2047]),
            ([PAD, PAD], [8, 6], [15, 11]), ([PAD, PAD], [16, 16], [31, 31]),
            ([CEN, HER], [7, 7], [10, 10]), ([CEN, HER], [8, 8], [12, 12]),
            ([CEN, HER], [31, 31], [46, 46]), ([REAL, PAD], [8, 6], [15, 11]),
            ([REAL, PAD], [16, 12], [31, 23]),
            ([PAD, PAD, PAD], [4, 5, 6], [7, 9, 11]),
            ([CEN, CEN, HER], [5, 5, 5], [7, 7, 7]),
            ([CEN, CEN, HER], [6, 7, 8], [9, 10, 12]),
            ([REAL, PAD, PAD], [4, 5, 6], [7, 9, 11]),
            ([REAL, PAD, PAD], [8, 8, 8], [15, 15, 15])):
        cases.append((kinds, L, M, None, None, None))
    # Forced 2D parameters (outer m/D/I swept, inner optimised).
    for mx in (16, 8, 4):
        for D in (1, 2):
            cases.append(([PAD, PAD], [8, 6], [16, 11], [mx, 0], [D, 0],
                          [0, -1]))
    for mx in (12, 8, 4):
        for D in (1, 2):
            cases.append(([CEN, HER], [8, 8], [12, 12], [mx, 0], [D, 0],
                          [0, -1]))
    return cases


def main():
    if not ref.available():
        sys.exit("oracle/_ref/libfftwpp_ref.so is missing: run make -C oracle")
    out = {}
    meta = []
    n = 0
    for idx, (kinds, L, M, m, D, I) in enumerate(conv_cases()):
        for src in ("det", "rand"):
            A = 2
            fs = det_inputs(kinds, L, A) if src == "det" else \
                rand_inputs(kinds, L, A, seed=1000 + idx)
            try:
                h, info = ref.convolve(fs, kinds, L, M, ms=m, Ds=D, Is=I,
                                       mult=mult_for(kinds))
            except RuntimeError:
                continue
            key = f"c{n:04d}"
            out[key + "_in0"] = fs[0]
            out[key + "_in1"] = fs[1]
            out[key + "_out"] = h[0]
            out[key + "_info"] = np.array(info, dtype=np.int64)
            meta.append((key, kinds, L, M, m or [0] * len(kinds),
                         D or [0] * len(kinds), I or [-1] * len(kinds),
                         mult_for(kinds), src))
            n += 1
    # Jacobian multiplier (A=4, B=1) on centred-Hermitian 2D data.  Explicit
    # plans (m = M) are forced: the reference's two-pass schedule (loop2,
    # convolve.cc:7538-7549 and convolve.h:1487-1498) overwrites the residue-0
    # product before its backward transform whenever A - B > B, so an
    # optimiser-chosen 2-pass plan returns a wrong result for A=4, B=1.
    for (Lx, Ly) in ((7, 7), (15, 15)):
        kinds = [CEN, HER]
        Mx, My = 3 * ((Lx + 1) // 2) - 2, 3 * ((Ly + 1) // 2) - 2
        fs = rand_inputs(kinds, [Lx, Ly], 4, seed=77 + Lx)
        h, info = ref.convolve(fs, kinds, [Lx, Ly], [Mx, My], ms=[Mx, My],
                               Ds=[1, 1], Is=[0, 0], mult="realjacobian")
        key = f"c{n:04d}"
        for a in range(4):
            out[key + f"_in{a}"] = fs[a]
        out[key + "_out"] = h[0]
        out[key + "_info"] = np.array(info, dtype=np.int64)
        meta.append((key, kinds, [Lx, Ly], [Mx, My], [0, 0], [0, 0], [-1, -1],
                     "realjacobian", "rand"))
        n += 1
    np.savez_compressed(os.path.join(HERE, "conv_cases.npz"), **out)
    with open(os.path.join(HERE, "conv_cases.txt"), "w") as fh:
        fh.write("# key kinds L M m D I mult inputs   (kinds: 0 fftPad, "
                 "1 fftPadCentered, 2 fftPadHermitian, 3 fftPadReal)\n")
        for row in meta:
            fh.write(" ".join(str(x).replace(" ", "") for x in row) + "\n")

    # Analytic known answer (tests/hybridconv.cc:13-14, 50-69).
    kat = {}
    iF = complex(np.sqrt(3.0), np.sqrt(7.0))
    iG = complex(np.sqrt(5.0), np.sqrt(11.0))
    for L in (64, 256, 1024, 4096):
        j = np.arange(L)
        e = np.exp(1j * j)
        f, g = iF * e, iG * e
        exact = iF * iG * (j + 1) * e
        h, info = ref.convolve([f, g], [PAD], [L], [2 * L])
        kat[f"L{L}_ref"] = h[0]
        kat[f"L{L}_exact"] = exact
    np.savez_compressed(os.path.join(HERE, "kat.npz"), **kat)

    # Forward residue layouts (tests/hybrid.cc:69-105).
    lay = {}
    lmeta = []
    k = 0
    for kind in (PAD, CEN):
        for (L, M) in ((8, 16), (9, 13), (8, 12), (16, 31), (7, 20)):
            for m in (0, M, L, (L + 1) // 2, 4, 2):
                for D in (0, 1, 2, 4):
                    for I in (0, 1):
                        f = (np.arange(L) + 1) + 1j * (np.arange(L) + 2)
                        r = ref.forward_layout(kind, L, M, m, D, I, f)
                        if r is None:
                            continue
                        F, idx, info = r
                        key = f"l{k:04d}"
                        lay[key + "_F"] = F
                        lay[key + "_idx"] = idx
                        lay[key + "_info"] = np.array(info, dtype=np.int64)
                        lmeta.append((key, kind, L, M, m, D, I))
                        k += 1
    np.savez_compressed(os.path.join(HERE, "layouts.npz"), **lay)
    with open(os.path.join(HERE, "layouts.txt"), "w") as fh:
        fh.write("# key kind L M m D I   (info: m p q n D I R N)\n")
        for row in lmeta:
            fh.write(" ".join(map(str, row)) + "\n")

    # Parameter rule and nextfftsize.
    par = []
    for L in range(1, 40):
        for M in range(L, 2 * L + 8, 3):
            for m in range(1, M + 3):
                for c in (0, 1):
                    p, nn, q = ref.parameters(L, M, m, c)
                    par.append((L, M, m, c, p, nn, q))
    nf = [(m, ref.nextfftsize(m)) for m in range(1, 5000)]
    np.savez_compressed(os.path.join(HERE, "params.npz"),
                        parameters=np.array(par, dtype=np.int64),
                        nextfftsize=np.array(nf, dtype=np.int64))
    print(f"{n} convolution cases, {len(kat)//2} KAT lengths, {k} layouts, "
          f"{len(par)} parameter rows")


def hermitian_layouts():
    """Forward blocks of a 1D fftPadHermitian (real values at transformed
    indices) for explicit and hybrid plans; the inputs are the reference
    test's (tests/hybridh.cc:58-62: f_0 = 1, f_j = (j+1) + i (j+2))."""
    lay = {}
    meta = []
    k = 0
    for (L, M) in ((15, 22), (16, 24), (31, 46), (63, 94), (20, 30),
                   (511, 766)):
        H = (L + 1) // 2
        f = (np.arange(H) + 1) + 1j * (np.arange(H) + 2)
        f[0] = 1
        for m in (0, M, (M + 2) // 2 * 2, 8, 4, 16, 32):
            for D in (0, 1, 2):
                r = ref.forward_layout_hermitian(L, M, m, D, -1, f)
                if r is None:
                    continue
                F, idx, info = r
                key = f"h{k:04d}"
                lay[key + "_F"] = F
                lay[key + "_idx"] = idx
                lay[key + "_info"] = np.array(info, dtype=np.int64)
                meta.append((key, L, M, m, D))
                k += 1
    np.savez_compressed(os.path.join(HERE, "hlayouts.npz"), **lay)
    with open(os.path.join(HERE, "hlayouts.txt"), "w") as fh:
        fh.write("# key L M m D   (info: m p q n D I R N)\n")
        for row in meta:
            fh.write(" ".join(map(str, row)) + "\n")
    return k


if __name__ == "__main__":
    if sys.argv[1:] == ["--only", "hlayouts"]:
        print(f"{hermitian_layouts()} Hermitian layouts")
    else:
        main()
        print(f"{hermitian_layouts()} Hermitian layouts")
