"""CPU: pin the oracle (numpy restatement + direct sums) to the reference's
own outputs stored in tests/golden/ (generated by tests/golden/make_golden.py
from FFTW++ compiled from its sources)."""
import os

import numpy as np
import pytest

from oracle import direct as Dr
from oracle import hybrid as H

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_cases():
    data = np.load(os.path.join(GOLD, "conv_cases.npz"))
    rows = []
    for line in open(os.path.join(GOLD, "conv_cases.txt")):
        if line.startswith("#"):
            continue
        key, kinds, L, M, m, D, I, mult, src = line.split()
        ev = eval  # literal lists written by make_golden.py
        A = 4 if mult == "realjacobian" else 2
        ins = [data[f"{key}_in{a}"] for a in range(A)]
        rows.append(dict(key=key, kinds=ev(kinds), L=ev(L), M=ev(M), m=ev(m),
                         mult=mult, src=src, ins=ins, out=data[f"{key}_out"],
                         info=data[f"{key}_info"]))
    return rows


CASES = load_cases()


def test_fixture_count():
    assert len(CASES) >= 500


@pytest.mark.parametrize("idx", range(0, len(CASES), 1))
def test_oracle_matches_reference(idx):
    c = CASES[idx]
    got = H.convolve(c["ins"], c["kinds"], c["L"], c["M"], mult=c["mult"])[0]
    err = Dr.rel_l2(got, c["out"])
    # The reference's own test tolerance is 1e-12 (tests/tests.py:223-224).
    assert err < 1e-12, (c["key"], err)


def test_oracle_forced_m_matches_reference():
    """The residue decomposition with the reference's chosen (m, q)
    reproduces the reference's output."""
    n = 0
    for c in CASES:
        if len(c["kinds"]) != 1:
            continue
        m = int(c["info"][0][0])
        got = H.convolve(c["ins"], c["kinds"], c["L"], c["M"], ms=[m],
                         mult=c["mult"])[0]
        assert Dr.rel_l2(got, c["out"]) < 1e-12, c["key"]
        n += 1
    assert n > 100


def _direct(c):
    kinds, f, g = c["kinds"], c["ins"][0], c["ins"][1]
    if kinds == [H.PAD] or kinds == [H.REAL]:
        return Dr.directconv(f, g)
    if kinds == [H.CENTERED]:
        return Dr.directconv_c(f, g)
    if kinds == [H.HERMITIAN]:
        return Dr.directconvh(f, g)
    if kinds in ([H.PAD, H.PAD], [H.REAL, H.PAD]):
        return Dr.directconv2(f, g)
    if kinds == [H.CENTERED, H.HERMITIAN] and c["L"][1] % 2 == 1:
        return Dr.directconvh2(f, g, c["L"][0] % 2 == 1)
    if kinds in ([H.PAD, H.PAD, H.PAD], [H.REAL, H.PAD, H.PAD]):
        return Dr.directconv3(f, g)
    return None


def test_reference_matches_direct_sums():
    """The reference (with the clean-room FFT backend) against the
    reference's own O(L^d) direct oracles (tests/direct.cc)."""
    n = 0
    for c in CASES:
        if c["mult"] not in ("binary", "realbinary"):
            continue
        d = _direct(c)
        if d is None:
            continue
        assert Dr.rel_l2(c["out"], d) < 1e-12, c["key"]
        n += 1
    assert n > 300


def test_known_answer():
    """tests/hybridconv.cc:50-69: f_j = iF e^{ij}, g_j = iG e^{ij} gives
    h_j = iF iG (j+1) e^{ij}."""
    kat = np.load(os.path.join(GOLD, "kat.npz"))
    for L in (64, 256, 1024, 4096):
        exact = kat[f"L{L}_exact"]
        assert Dr.rel_l2(kat[f"L{L}_ref"], exact) < 1e-12
        iF = complex(np.sqrt(3.0), np.sqrt(7.0))
        iG = complex(np.sqrt(5.0), np.sqrt(11.0))
        j = np.arange(L)
        e = np.exp(1j * j)
        got = H.convolve([iF * e, iG * e], [H.PAD], [L], [2 * L])[0]
        assert Dr.rel_l2(got, exact) < 1e-12


def test_parameters_and_nextfftsize():
    p = np.load(os.path.join(GOLD, "params.npz"))
    for L, M, m, c, pp, nn, qq in p["parameters"]:
        assert H.parameters(int(L), int(M), int(m), bool(c)) == (pp, nn, qq)
    for m, n in p["nextfftsize"]:
        assert H.nextfftsize(int(m)) == n


def load_layouts():
    data = np.load(os.path.join(GOLD, "layouts.npz"))
    rows = []
    for line in open(os.path.join(GOLD, "layouts.txt")):
        if line.startswith("#"):
            continue
        key, kind, L, M, m, D, I = line.split()
        rows.append(dict(key=key, kind=int(kind), L=int(L), M=int(M),
                         F=data[key + "_F"], idx=data[key + "_idx"],
                         info=data[key + "_info"]))
    return rows


LAYOUTS = load_layouts()


def layout_stream(lay):
    """(r, k) pairs in the order the reference emits them: residue blocks
    r += increment(r) (convolve.h:394-396), entries k < noutputs(r)
    (convolve.h:435-437) with blocksize l = m*P (convolve.cc:549-557)."""
    m, p, q, n, D, I, R, N = [int(x) for x in lay["info"]]
    centered = lay["kind"] == H.CENTERED
    if q == 1:
        return [(0, k) for k in range(N)], (m, p, q, n, 1, 1, centered)
    if centered:
        conj = D > 1 and (p == 1 or p % 2 == 0)      # convolve.h:653
        P = 1 if p == 2 else p // 2
    else:
        conj = D > 1 and p <= 2                      # convolve.h:384-386
        P = 1 if p == 2 else p
    D0 = n % D or D
    dr = D // 2 if conj else D
    out = []
    r = 0
    while r < R:
        for k in range(m * P * (D0 if r == 0 else D)):
            out.append((r, k))
        r += dr if r > 0 else ((D0 + 1) // 2 if conj else D0)
    return out, (m, p, q, n, D, D0, centered)


def test_layout_index_map():
    """fftBase::index restated in the oracle reproduces the reference's
    transformed index of every entry of every residue block."""
    for lay in LAYOUTS:
        stream, (m, p, q, n, D, D0, centered) = layout_stream(lay)
        assert len(stream) == len(lay["idx"]), lay["key"]
        got = [H.index_base(r, k, m=m, p=p, q=q, n=n, D=D, D0=D0,
                            centered=centered) for r, k in stream]
        assert np.array_equal(np.array(got), lay["idx"]), lay["key"]


def test_layout_values_are_padded_dft():
    """Every forward output F of residue block entry k equals the explicit
    padded DFT (FFTW sign +1) at the transformed index idx[k]; centred data
    carries the extra phase of its origin offset floor(L/2)."""
    for lay in LAYOUTS:
        L, kind = lay["L"], lay["kind"]
        N = int(lay["info"][7])
        f = (np.arange(L) + 1) + 1j * (np.arange(L) + 2)
        s = np.arange(L)
        c = L // 2 if kind == H.CENTERED else 0
        k = lay["idx"]
        full = np.exp(2j * np.pi * (np.outer(k, s - c) % N) / N) @ f
        assert Dr.rel_l2(lay["F"], full) < 1e-12, lay["key"]


@pytest.mark.parametrize("kinds,L,mult,single", [
    ([H.PAD], [23], "dot", "binary"),
    ([H.CENTERED, H.HERMITIAN], [15, 15], "realdot", "realbinary"),
    ([H.PAD, H.PAD], [6, 7], "dot", "binary"),
])
def test_dot_multiplier_is_sum_of_products(kinds, L, mult, single):
    """The dot-product multiplier equals the sum of the pairs' binary
    convolutions (linearity); checks the restated *_dot semantics."""
    rng = np.random.default_rng(4)
    shape = list(L)
    if kinds[-1] == H.HERMITIAN:
        shape[-1] = (L[-1] + 1) // 2
    K = 3
    fs = []
    for _ in range(2 * K):
        f = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
        if kinds[-1] == H.HERMITIAN:
            H.hermitian_symmetrize_x(f, (L[0] + 1) // 2, shape[1], L[0] // 2)
        fs.append(f)
    M = [H.default_M(k, l) for k, l in zip(kinds, L)]
    got = H.convolve(fs, kinds, L, M, mult=mult)[0]
    want = sum(H.convolve([fs[k], fs[K + k]], kinds, L, M, mult=single)[0]
               for k in range(K))
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()


def test_sampled_direct_sum_3d():
    """directconv3_at, the per-entry form the 256^3 parity test uses,
    equals the full direct sum of tests/direct.h:118-133."""
    from oracle.direct import directconv3, directconv3_at
    rng = np.random.default_rng(12)
    f, g = rng.normal(size=(5, 4, 6)), rng.normal(size=(5, 4, 6))
    h = directconv3(f, g)
    pts = [(4, 3, 5), (0, 0, 0), (2, 1, 3), (4, 0, 5), (1, 3, 2)]
    np.testing.assert_allclose(directconv3_at(f, g, pts),
                               [h[p] for p in pts], rtol=0, atol=1e-13)


@pytest.mark.parametrize("case", [
    ([0], [9], [17], "binary"),
    ([1], [9], [13], "binary"),
    ([2], [15], [22], "realbinary"),
    ([3], [9], [17], "binary"),
    ([1, 2], [9, 7], [13, 10], "realbinary"),
    ([0, 0], [6, 5], [11, 9], "binary"),
    ([3, 0, 0], [4, 5, 3], [7, 9, 5], "binary"),
    ([1, 1, 2], [5, 5, 5], [7, 7, 7], "realbinary")])
def test_explicit_oracle_matches_hybrid(case):
    """The explicit N-grid oracle (the checker of position-dependent
    multipliers) equals the hybrid restatement for position-independent
    multipliers, on padded grids larger than M as well."""
    from oracle import explicit as E
    from oracle import hybrid as H
    kinds, L, M, mult = case
    rng = np.random.default_rng(sum(L))
    shape = [(l + 1) // 2 if k == H.HERMITIAN else l for k, l in zip(kinds, L)]
    fs = []
    for _ in range(2):
        if kinds[0] == H.REAL:
            f = rng.normal(size=shape)
        else:
            f = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        if kinds[-1] == H.HERMITIAN:
            if len(kinds) == 1:
                f[0] = f[0].real
            elif len(kinds) == 2:
                H.hermitian_symmetrize_x(f, (L[0] + 1) // 2, shape[1],
                                         L[0] // 2)
            else:
                H.hermitian_symmetrize_xy(f, (L[0] + 1) // 2, (L[1] + 1) // 2,
                                          shape[2], L[0] // 2, L[1] // 2)
        fs.append(f)
    want = H.convolve(fs, kinds, L, M, mult=mult)[0]
    for extra in (0, 3):
        Ns = [m + extra + ((m + extra) % 2 if k in (H.HERMITIAN, H.REAL)
                           else 0) for k, m in zip(kinds, M)]
        got = E.convolve(fs, kinds, L, Ns, lambda v, ix: [v[0] * v[1]])[0]
        err = Dr.rel_l2(got, want)
        assert err <= 1e-13, (Ns, err)


def hermitian_layouts():
    data = np.load(os.path.join(GOLD, "hlayouts.npz"))
    for line in open(os.path.join(GOLD, "hlayouts.txt")):
        if line.startswith("#"):
            continue
        key, L, M, m, D = line.split()
        yield (key, int(L), int(M), int(m), int(D), data[key + "_F"],
               data[key + "_idx"], data[key + "_info"])


def test_hermitian_layouts_pin_explicit_oracle():
    """Every real value the reference's fftPadHermitian forward produced
    (tests/hybridh.cc:74-99, explicit and hybrid plans) equals the explicit
    oracle's complex-to-real transform at its transformed index."""
    from oracle import explicit as E
    n = 0
    for key, L, M, m, D, F, idx, info in hermitian_layouts():
        N = int(info[7])
        H_ = (L + 1) // 2
        f = (np.arange(H_) + 1) + 1j * (np.arange(H_) + 2)
        f[0] = 1
        u = E._forward(f, E.HERMITIAN, L, N, 0)
        assert len(set(idx.tolist())) == len(idx) <= N, key
        np.testing.assert_allclose(F, u[idx], rtol=0,
                                   atol=1e-12 * np.abs(u).max(), err_msg=key)
        n += 1
    assert n >= 100
