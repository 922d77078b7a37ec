"""M1 / E2 one-body operators, eval_moment and transit_main on the GPU
against the oracle's restatement of transit.jl (needs a GB300)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from test_oracle import one_orbit_snt, schmidt_mu, single_particle_q

pytestmark = pytest.mark.gpu

CKPOT = os.path.join(GOLDEN, "ckpot.snt")
USDB = os.path.join(GOLDEN, "usdb.snt")
OBTR_RTOL = 1e-11  # FP64 overlaps <l|O|r> vs the oracle, relative to max |entry|
GF = (1.0, 0.0, 5.586, -3.826)
EC = (1.5, 0.5)


@pytest.fixture(scope="module")
def lib():
    from smgpu import _lib
    from smgpu import build as b
    b.build()
    return _lib.load()


def _rand(n, m, seed):
    v = np.random.default_rng(seed).standard_normal((n, m))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _close(a, b, rtol=OBTR_RTOL):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() <= rtol * scale


@pytest.mark.parametrize("snt,nuc,mtot2", [(USDB, "Ne20", 0), (USDB, "Ne20", 4), (USDB, "Na21", 1),
                                           (USDB, "O19", 3), (CKPOT, "Be8", 2), ("sd2p2n", "Ne20", 0)])
def test_expectation_form_matches_oracle(lib, snt_dir, snt, nuc, mtot2):
    """eval_moment's operator (prep_obtr_diag / op_obtr_diag, symmetric
    application with halves on the diagonal): full matrices <a|O|b> over
    seeded vectors, M1 and E2, custom g factors and charges."""
    from oracle.oracle import OracleProblem
    from smgpu import ShellModelProblem
    if snt in snt_dir:
        snt, nuc = snt_dir[snt]
    G = ShellModelProblem(snt, nuc, 0, twoJ=mtot2)
    O = OracleProblem(snt, nuc, mtot2=mtot2)
    v = _rand(3, G.mdim, 11)
    for op in (0, 1):
        for gf, ec in ((GF, EC), ((0.9, -0.1, 4.0, -2.5), (1.3, 0.7))):
            a = G.obtr(op, v, gfactors=gf, effcharge=ec)
            b = O.obtr(op, v, gfactors=gf, effcharge=ec)
            assert _close(a, b), (op, np.abs(a - b).max(), np.abs(b).max())
            assert np.allclose(a, a.T, rtol=0, atol=1e-12 * np.abs(a).max())


@pytest.mark.parametrize("snt,nuc,ml,mr", [(USDB, "Ne20", 2, 0), (USDB, "Ne20", 4, 0), (USDB, "Ne20", 4, 2),
                                           (USDB, "Ne20", 2, 2), (USDB, "Na21", 3, 1), (USDB, "Na21", 5, 1),
                                           (CKPOT, "He6", 4, 0), (CKPOT, "Li7", 3, 1)])
def test_transition_form_matches_oracle(lib, snt, nuc, ml, mr):
    """transit_main's operator (prep_obtr_nondiag / op_obtr_nondiag /
    calc_bifs) from the Mtot = mr basis to the Mtot = ml basis."""
    from oracle.oracle import OracleProblem
    from smgpu import ShellModelProblem
    GL = ShellModelProblem(snt, nuc, 0, twoJ=ml)
    GR = ShellModelProblem(snt, nuc, 0, twoJ=mr)
    OL = OracleProblem(snt, nuc, mtot2=ml)
    OR = OracleProblem(snt, nuc, mtot2=mr)
    vl = _rand(3, GL.mdim, 5)
    vr = _rand(2, GR.mdim, 6)
    for op in (0, 1):
        a = GL.obtr(op, vl, vr, right=GR, symmetric=False)
        b = OL.obtr(op, vl, vr, right=OR, symmetric=False)
        assert _close(a, b), (op, np.abs(a - b).max(), np.abs(b).max())
        if op == 0 and (ml - mr) // 2 > 1:
            assert not a.any()


@pytest.mark.parametrize("orb", [(0, 2, 5), (0, 2, 3), (1, 0, 1), (0, 3, 7)])
@pytest.mark.parametrize("nuc,species", [("F17", 0), ("O17", 1)])
def test_schmidt_moments_on_gpu(lib, tmp_path, orb, nuc, species):
    """Known answer: eval_moment on the GPU gives the Schmidt magnetic moment
    and the single-particle quadrupole moment of one nucleon in one orbit."""
    from smgpu import ShellModelProblem, eval_moment
    n, l, j2 = orb
    snt = one_orbit_snt(tmp_path / "one.snt", n, l, j2)
    P = ShellModelProblem(snt, nuc, 0, twoJ=j2)
    r = eval_moment(P, np.ones((1, 1)), [j2 / 2])
    assert abs(r["mu"][0] - schmidt_mu(l, j2, GF[species], GF[2 + species])) < 1e-12
    if j2 > 1:
        assert abs(r["Q"][0] - single_particle_q(n, l, j2, EC[species], 17)) < 1e-12
        assert f"Q (n=1) {r['Q'][0]:12.5f} " in r["text"]
    else:
        assert np.isnan(r["Q"][0]) and "Q (n=1)" not in r["text"]
    assert r["text"].startswith(f"mu (n=1) {r['mu'][0]:12.5f} \t")


def _oracle_moments(O, vecs, twoJs, m2):
    """eval_moment's composition (transit.jl:702-765) over the oracle's
    operator and 3j symbols."""
    import math
    from oracle.oracle import wigner3j
    mu = O.obtr(0, vecs)
    q = O.obtr(1, vecs)
    out = []
    for k, tJ in enumerate(twoJs):
        sign = -1.0 if ((tJ - m2) // 2) % 2 else 1.0
        s1 = wigner3j(tJ, 2, tJ, -m2, 0, m2)
        s2 = wigner3j(tJ, 4, tJ, -m2, 0, m2)
        g = sign * mu[k, k] * wigner3j(tJ, 2, tJ, -tJ, 0, tJ) / s1 * math.sqrt(4 * math.pi / 3) if s1 else np.nan
        Q = q[k, k] * wigner3j(tJ, 4, tJ, -tJ, 0, tJ) / s2 * math.sqrt(16 * math.pi / 5) * sign if s2 else np.nan
        out.append((g, Q))
    return np.array(out)


def test_main_sm_calc_moment_he6(lib, tmp_path, monkeypatch, capsys):
    """The reference's own case main_sm(ckpot, "He6", 1, [4]; calc_moment =
    true, save_wav = true) (test/ShellModel_test.jl:29): the printed moments
    equal the oracle's on the saved Ritz vector."""
    from smgpu import main_sm
    from smgpu.wav import read_wav_full
    from oracle.oracle import OracleProblem
    monkeypatch.chdir(tmp_path)
    en = main_sm(CKPOT, "He6", 1, [4], calc_moment=True, save_wav=True)
    out = capsys.readouterr().out
    O = OracleProblem(CKPOT, "He6", mtot2=4)
    e, j, v, mt = read_wav_full(str(tmp_path / "He6_ckpot_j4.wav"), O.mdim)
    assert mt == 4 and list(j) == [4] and np.allclose(e, en, rtol=0, atol=0)
    ref = _oracle_moments(O, v, [4], 4)
    assert f"mu (n=1) {ref[0, 0]:12.5f} \tQ (n=1) {ref[0, 1]:12.5f} " in out


def test_eval_moment_sd_states_match_oracle(lib):
    """Moments of the lowest 21Na states (odd A, mixed J) on the GPU against
    the oracle composition on the same Ritz vectors."""
    from smgpu import ShellModelProblem, eval_moment
    from smgpu.shellmodel import J_from_JJ1
    from oracle.oracle import OracleProblem
    G = ShellModelProblem(USDB, "Na21", 0)
    r = G.solve(6, lm=40, ls=15, tol=1e-9, want_vecs=True)
    Js = [J_from_JJ1(x) for x in G.jj(r["evecs"])]
    res = eval_moment(G, r["evecs"], Js)
    O = OracleProblem(USDB, "Na21")
    ref = _oracle_moments(O, r["evecs"], [int(2 * J) for J in Js], G.mtot2)
    for k, J in enumerate(Js):
        if J < 0:
            continue
        for col, key in ((0, "mu"), (1, "Q")):
            if np.isnan(ref[k, col]):
                assert np.isnan(res[key][k])
            else:
                assert abs(res[key][k] - ref[k, col]) < 1e-10 * max(1.0, abs(ref[k, col])), (k, key)


def test_transit_main_he6(lib, tmp_path, monkeypatch, capsys):
    """The reference's transition check (test/ShellModel_test.jl:27-32): J=0
    and J=2 He6 states saved by main_sm, then transit_main(ckpot, "He6", 0,
    4, wavs): E2 reduced matrix elements and B values against the oracle's
    operator on the same vectors; M1 has no 0 -> 2 component."""
    from smgpu import main_sm, transit_main
    from smgpu.wav import read_wav_full
    from oracle.oracle import OracleProblem, wigner3j
    monkeypatch.chdir(tmp_path)
    main_sm(CKPOT, "He6", 1, [0], save_wav=True, verbose=False)
    main_sm(CKPOT, "He6", 1, [4], save_wav=True, verbose=False)
    res = transit_main(CKPOT, "He6", 0, 4, ["He6_ckpot_j0.wav", "He6_ckpot_j4.wav"], calc_EM=True)
    out = capsys.readouterr().out
    OL = OracleProblem(CKPOT, "He6", mtot2=4)
    OR = OracleProblem(CKPOT, "He6", mtot2=0)
    _, _, vl, _ = read_wav_full("He6_ckpot_j4.wav", OL.mdim)
    _, _, vr, _ = read_wav_full("He6_ckpot_j0.wav", OR.mdim)
    sel = wigner3j(4, 4, 0, -4, 4, 0)
    mred = OL.obtr(1, vl, vr, right=OR, symmetric=False) / sel
    assert "Mred_M1" not in res
    assert abs(res["Mred_E2"][0, 0] - mred[0, 0]) < 1e-10 * max(1.0, abs(mred[0, 0]))
    m = mred[0, 0]
    assert f"Mred.(E2) (1,1) {m:9.3f}   B(E2) (1<=1) {m * m / 1:9.3f}  B(E2) (1=>1) {m * m / 5:9.3f} " in out
    assert "mdims J2=4" in out and "wfr: He6_ckpot_j0.wav" in out
