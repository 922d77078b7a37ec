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
