"""The CPU oracle against the reference's own known answers (no GPU)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle.oracle import OracleProblem, clebsch, start_vector, sym_eig

CKPOT = os.path.join(GOLDEN, "ckpot.snt")
USDB = os.path.join(GOLDEN, "usdb.snt")


def test_ckpot_be8_known_answer(golden):
    """test/ShellModel_test.jl:8-15: ckpot.snt, 8Be, 10 lowest, (ΔE)² < 1e-6."""
    g = golden["ckpot_Be8"]
    P = OracleProblem(CKPOT, "Be8")
    assert P.mdim == 51 and P.nblocks == 5
    r = P.trl(10, lm=300, ls=20, tol=1e-8)
    assert r["converged"]
    for e, ref in zip(r["evals"], g["energies"]):
        assert (e - ref) ** 2 < g["tolerance_sq"]


def test_mg24_sd_dimension(golden):
    """example/log_sample_script.txt:323: 24Mg in the sd shell has mdim 28503."""
    P = OracleProblem(USDB, "Mg24")
    assert P.mdim == golden["sd_Mg24_mdim"]["mdim"]


@pytest.mark.parametrize("name,mdim,nblocks,maxblk", [("sd2p2n", 640, 9, 14), ("sd4p4n", 28503, 13, 81),
                                                      ("pf4p4n", 1963461, 21, 565)])
def test_config_dimensions(snt_dir, name, mdim, nblocks, maxblk):
    snt, nuc = snt_dir[name]
    P = OracleProblem(snt, nuc)
    assert (P.mdim, P.nblocks, int(P.np_.max()), int(P.nn_.max())) == (mdim, nblocks, maxblk, maxblk)
    assert int(P.tdims[-1]) == mdim
    assert np.all(np.diff(P.Mp) == 2)  # blocks ordered by ascending proton M


@pytest.mark.parametrize("case", ["ckpot", "sd2p2n"])
def test_dense_h_symmetric_and_trl_matches_eigh(snt_dir, case):
    """calc_Hflat's symmetry check (variational_ansatz.jl:582-584) and TRL vs LAPACK."""
    P = OracleProblem(CKPOT, "Be8") if case == "ckpot" else OracleProblem(*snt_dir["sd2p2n"])
    H = P.dense_H()
    assert np.abs(H - H.T).max() < 1e-12
    w = np.linalg.eigvalsh(H)
    r = P.trl(5, lm=60, ls=20, tol=1e-10)
    assert np.allclose(r["evals"], w[:5], rtol=1e-9, atol=0)


def test_jacobi_matches_lapack():
    rng = np.random.default_rng(7)
    A = rng.standard_normal((40, 40))
    A = A + A.T
    w, Z = sym_eig(A)
    assert np.allclose(w, np.linalg.eigvalsh(A), rtol=0, atol=1e-12)
    assert np.allclose(A @ Z, Z * w, atol=1e-11)


def test_clebsch_gordan_orthonormality():
    # Σ_{m1,m2} <j1 m1 j2 m2|J M><j1 m1 j2 m2|J' M> = δ_JJ' for j1=7/2, j2=5/2
    tj1, tj2 = 7, 5
    for tM in range(-12, 13, 2):
        for tJ in range(2, 13, 2):
            for tJp in range(2, 13, 2):
                s = 0.0
                for tm1 in range(-tj1, tj1 + 1, 2):
                    tm2 = tM - tm1
                    if abs(tm2) > tj2:
                        continue
                    s += clebsch(tj1, tm1, tj2, tm2, tJ, tM) * clebsch(tj1, tm1, tj2, tm2, tJp, tM)
                expect = 1.0 if (tJ == tJp and abs(tM) <= tJ) else 0.0
                assert abs(s - expect) < 1e-14
    assert clebsch(1, 1, 1, -1, 0, 0) == pytest.approx(2 ** -0.5, abs=1e-16)
    assert clebsch(1, -1, 1, 1, 0, 0) == pytest.approx(-(2 ** -0.5), abs=1e-16)


def test_start_vector_deterministic():
    a = start_vector(1000, 1234)
    b = start_vector(1000, 1234)
    assert np.array_equal(a, b)
    assert abs(a.mean()) < 0.1 and 0.2 < a.std() < 0.8
    assert not np.array_equal(a, start_vector(1000, 99))


def test_uneven_and_empty_species():
    """Odd A (M=1/2 doubled 1), a zero-particle proton species and an uneven split."""
    for nuc, mdim in (("O19", None), ("Na21", None), ("Al27", None)):
        P = OracleProblem(USDB, nuc)
        assert P.mdim > 0
        assert P.Mtot == P.A % 2
        H = P.dense_H() if P.mdim < 3000 else None
        if H is not None:
            assert np.abs(H - H.T).max() < 1e-12


def _jj_snt_text(orbits, core, A):
    """J^2 written as an snt interaction on the given orbits (one-body
    j(j+1); diagonal two-body J(J+1) - j_a(j_a+1) - j_b(j_b+1) per pair, J
    even for a == b in pp/nn).  The library builds the same operator in C++."""
    k = len(orbits)
    jj1 = [0.25 * o[2] * (o[2] + 2) for o in orbits]
    lines = ["! J^2", f" {k} {k} {core[0]} {core[1]}"]
    for t, tz in ((0, -1), (1, 1)):
        lines += [f" {i + 1 + t * k} {n} {l} {j2} {tz}" for i, (n, l, j2) in enumerate(orbits)]
    lines.append(f" {2 * k} 0")
    lines += [f" {i + 1 + t * k} {i + 1 + t * k} {jj1[i]:.12f}" for t in range(2) for i in range(k)]
    tb = []
    for off in (0, k):
        for a in range(k):
            for b in range(a, k):
                for J in range(abs(orbits[a][2] - orbits[b][2]) // 2, (orbits[a][2] + orbits[b][2]) // 2 + 1):
                    if a == b and J % 2:
                        continue
                    tb.append((a + 1 + off, b + 1 + off, a + 1 + off, b + 1 + off, J, J * (J + 1) - jj1[a] - jj1[b]))
    for a in range(k):
        for b in range(k):
            for J in range(abs(orbits[a][2] - orbits[b][2]) // 2, (orbits[a][2] + orbits[b][2]) // 2 + 1):
                tb.append((a + 1, b + 1 + k, a + 1, b + 1 + k, J, J * (J + 1) - jj1[a] - jj1[b]))
    lines.append(f" {len(tb)} 0 {A}")
    lines += [" %d %d %d %d %d %.12f" % t for t in tb]
    return "\n".join(lines) + "\n"


def test_jj_ladder_operator_on_be8_levels():
    """<J^2> of the ckpot 8Be Ritz vectors is J(J+1) with integer J."""
    P = OracleProblem(CKPOT, "Be8")
    r = P.trl(10, lm=60, ls=20, tol=1e-10, want_vecs=True)
    jj = np.array([P.jj(x) for x in r["evecs"]])
    J = (-1 + np.sqrt(1 + 4 * jj)) / 2
    assert np.abs(J - np.round(J)).max() < 1e-8
    assert list(np.round(J).astype(int)) == [0, 2, 4, 2, 1, 2, 3, 1, 0, 4]


@pytest.mark.parametrize("vp,vn", [(2, 2), (1, 2), (3, 1)])
def test_jj_two_body_form_matches_ladder_operator(tmp_path, vp, vn):
    """The two-body form of J^2 (what the library applies) against the
    ladder-operator form of the oracle, on random vectors and on J^2's own
    spectrum."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(GOLDEN), "..", "nucleartoolkit.jl_gb300"))
    from smgpu import synth
    nuc = synth.nucleus_name("sd", vp, vn)
    f = tmp_path / "jj.snt"
    f.write_text(_jj_snt_text(synth.SD_ORBITS, synth.SD_CORE, 16 + vp + vn))
    Jop = OracleProblem(str(f), nuc)
    # a problem on the same orbits in the same order (usdb.snt lists d3/2 first)
    ref = OracleProblem(synth.write_snt(str(tmp_path / "h.snt"), "sd", 7, vp, vn), nuc)
    assert Jop.mdim == ref.mdim
    ev = np.linalg.eigvalsh(Jop.dense_H())
    twoJ = -1 + np.sqrt(1 + 4 * ev)
    assert np.abs(twoJ - np.round(twoJ)).max() < 1e-9
    rng = np.random.default_rng(vp * 10 + vn)
    for _ in range(3):
        v = rng.standard_normal(ref.mdim)
        two_body = v @ Jop.operate_H(v) / (v @ v)
        assert abs(two_body - ref.jj(v)) < 1e-10 * max(1.0, abs(two_body))
    # eigenvectors of a J-conserving H have integer J in both forms
    r = ref.trl(3, lm=40, ls=15, tol=1e-10, want_vecs=True)
    for x in r["evecs"]:
        a, b = x @ Jop.operate_H(x), ref.jj(x)
        assert abs(a - b) < 1e-8
        assert abs(np.sqrt(1 + 4 * b) - np.round(np.sqrt(1 + 4 * b))) < 1e-6


# --------------------------------------------------------------- moments
def one_orbit_snt(path, n, l, j2, core=(8, 8)):
    """A model space of one orbit (n, l, j) per species and no two-body
    interaction: one valence nucleon is a pure single-particle state."""
    with open(path, "w") as f:
        f.write(f"! one orbit\n 1 1 {core[0]} {core[1]}\n 1 {n} {l} {j2} -1\n 2 {n} {l} {j2} 1\n 2 0\n"
                f" 1 1 0.0\n 2 2 0.0\n 0 0 {sum(core) + 2} -0.3\n")
    return str(path)


def schmidt_mu(l, j2, g_l, g_s):
    """Schmidt value of one nucleon in j = l ± 1/2 (units of mu_N)."""
    j = j2 / 2
    if j2 == 2 * l + 1:
        return g_l * l + g_s / 2
    return j / (j + 1) * ((j + 1.5) * g_l - g_s / 2)


def single_particle_q(n, l, j2, e, A):
    """Q = -(2j-1)/(2j+2) <r^2> e, <r^2> = b^2 (2n + l + 3/2), b from the
    mass formula the reference uses for 16 <= A <= 40."""
    hw = 45.0 * A ** (-1 / 3) - 25.0 * A ** (-2 / 3)
    b2 = 197.32696 ** 2 / (hw * (938.27231 + 939.56563) / 2)
    j = j2 / 2
    return -(2 * j - 1) / (2 * j + 2) * b2 * (2 * n + l + 1.5) * e


@pytest.mark.parametrize("orb", [(0, 2, 5), (0, 2, 3), (1, 0, 1)])
@pytest.mark.parametrize("nuc,species", [("F17", 0), ("O17", 1)])
def test_moment_operators_give_schmidt_values(tmp_path, orb, nuc, species):
    """Known answer for the restatement of prep_obtr_diag / op_obtr_diag /
    eval_moment (transit.jl:82-284,702-765): one nucleon in one orbit has the
    Schmidt magnetic moment and the single-particle quadrupole moment."""
    from oracle.oracle import wigner3j
    import math
    n, l, j2 = orb
    snt = one_orbit_snt(tmp_path / "one.snt", n, l, j2)
    O = OracleProblem(snt, nuc, mtot2=j2)
    assert O.mdim == 1
    v = np.ones((1, 1))
    g = (1.0, 0.0, 5.586, -3.826)
    ec = (1.5, 0.5)
    mu = O.obtr(0, v, gfactors=g, effcharge=ec)[0, 0]
    q = O.obtr(1, v, gfactors=g, effcharge=ec)[0, 0]
    gm = mu * wigner3j(j2, 2, j2, -j2, 0, j2) / wigner3j(j2, 2, j2, -j2, 0, j2) * math.sqrt(4 * math.pi / 3)
    assert abs(gm - schmidt_mu(l, j2, g[species], g[2 + species])) < 1e-12
    if j2 > 1:
        Q = q * math.sqrt(16 * math.pi / 5)
        assert abs(Q - single_particle_q(n, l, j2, ec[species], 17)) < 1e-12
    else:
        assert abs(q) < 1e-14


def test_wigner_symbols_match_sympy():
    """The oracle's 3j / 6j (WignerSymbols.jl stand-ins) against sympy."""
    wig = pytest.importorskip("sympy.physics.wigner")
    from sympy import Rational as R
    from oracle.oracle import wigner3j, wigner6j
    import itertools
    for a, b, c in itertools.product(range(0, 8), range(0, 5), range(0, 8)):
        for ma in range(-a, a + 1, 2):
            for mb in range(-b, b + 1, 2):
                mc = -ma - mb
                ref = float(wig.wigner_3j(R(a, 2), R(b, 2), R(c, 2), R(ma, 2), R(mb, 2), R(mc, 2)))
                assert abs(wigner3j(a, b, c, ma, mb, mc) - ref) < 1e-15
    rng = np.random.default_rng(5)
    for js in rng.integers(0, 9, size=(3000, 6)):
        try:
            ref = float(wig.wigner_6j(*[R(int(j), 2) for j in js]))
        except ValueError:
            ref = 0.0
        assert abs(wigner6j(*js) - ref) < 1e-15


def test_radius_power_is_the_oscillator_r2():
    """radius_power(2, n, l, n, l, b) = b^2 (2n + l + 3/2) (transit.jl:62-80)."""
    from oracle.oracle import radius_power
    for n in range(3):
        for l in range(5):
            assert abs(radius_power(2, n, l, n, l, 1.7) - 1.7 ** 2 * (2 * n + l + 1.5)) < 1e-12


# ------------------------------------------------- eigenvector continuation
def _snt_parts(path):
    L = [x.strip() for x in open(path) if x.strip() and not x.strip().startswith(("!", "#"))]
    lp, ln = map(int, L[0].split()[:2])
    nsp = int(L[1 + lp + ln].split()[0])
    hdr = L[2 + lp + ln + nsp].split()
    nt = int(hdr[0])
    return L[0], L[1:1 + lp + ln], hdr, L[3 + lp + ln + nsp:3 + lp + ln + nsp + nt], lp, ln


def unit_snt(path, u, out):
    """The interaction whose only non-zero entry is unit u: the SPE of orbit
    u (u < lp + ln) or TBME line u - lp - ln, set to 1 without mass scaling."""
    head, orbs, hdr, tb, lp, ln = _snt_parts(path)
    s = [head] + orbs
    if u < lp + ln:
        s += [" 1 0", f" {u + 1} {u + 1} 1.0", f" 0 0 {hdr[2]}"]
    else:
        s += [" 0 0", f" 1 0 {hdr[2]}", " ".join(tb[u - lp - ln].split()[:5] + ["1.0"])]
    with open(out, "w") as f:
        f.write("\n".join(s) + "\n")
    return str(out)


@pytest.mark.parametrize("snt,nuc,mtot2", [("ckpot.snt", "Be8", 0), ("ckpot.snt", "Li7", 1),
                                           ("usdb.snt", "Ne20", 0)])
def test_ec_transition_densities_are_derivatives_of_h(tmp_path, snt, nuc, mtot2):
    """The restated calcOBTD / prepTBTD / calcTBTD (eigenvector_continuation.jl:
    1035-1380) equal <w_i|H_u|w_j> with H_u the Hamiltonian of the unit
    interaction of each orbit SPE and snt line (hermitian partner included):
    the identity the GPU's transition densities are computed from."""
    snt = os.path.join(GOLDEN, snt)
    O = OracleProblem(snt, nuc, mtot2=mtot2)
    V = np.random.default_rng(3).standard_normal((2, O.mdim))
    N, td = O.ec_td(V)
    assert np.allclose(N, V @ V.T, rtol=1e-14, atol=0)
    _, _, _, tb, lp, ln = _snt_parts(snt)
    assert td.shape == (3, lp + ln + len(tb))
    for u in range(td.shape[1]):
        U = OracleProblem(unit_snt(snt, u, tmp_path / "unit.snt"), nuc, mtot2=mtot2)
        W = np.array([U.operate_H(v) for v in V])
        M = V @ W.T
        got = np.array([M[0, 0], M[0, 1], M[1, 1]])
        assert np.abs(got - td[:, u]).max() <= 1e-12 * max(1.0, np.abs(td[:, u]).max()), u
