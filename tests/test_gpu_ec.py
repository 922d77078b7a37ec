"""Eigenvector continuation (prepEC / solveEC) on the GPU against the
oracle's restatement of calcOBTD / prepTBTD / calcTBTD (needs a GB300)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CKPOT = os.path.join(GOLDEN, "ckpot.snt")
USDB = os.path.join(GOLDEN, "usdb.snt")
TD_RTOL = 1e-11  # GPU transition densities vs oracle, relative to max |TD| of the pair


@pytest.fixture(scope="module")
def lib():
    from smgpu import _lib
    from smgpu import build as b
    b.build()
    return _lib.load()


@pytest.mark.parametrize("snt,nuc,mtot2", [(CKPOT, "Be8", 0), (CKPOT, "Li7", 1), (USDB, "Ne20", 0),
                                           (USDB, "Na21", 3), (USDB, "O20", 0)])
def test_transition_densities_match_oracle(lib, snt, nuc, mtot2):
    from oracle.oracle import OracleProblem
    from smgpu import ShellModelProblem
    G = ShellModelProblem(snt, nuc, 0, twoJ=mtot2)
    O = OracleProblem(snt, nuc, mtot2=mtot2)
    V = np.random.default_rng(9).standard_normal((3, G.mdim))
    N, td = G.ec_td(V)
    No, tdo = O.ec_td(V)
    assert np.allclose(N, No, rtol=1e-13, atol=0)
    assert td.shape == tdo.shape
    for p in range(td.shape[0]):
        assert np.abs(td[p] - tdo[p]).max() <= TD_RTOL * np.abs(tdo[p]).max(), p


def _perturbed_snts(d, n, seed=2023, rel=0.1):
    """n seeded interactions around usdb: every SPE and TBME value times
    (1 + rel * N(0,1)) (sample interactions of the EC workflow)."""
    rng = np.random.default_rng(seed)
    src = open(USDB).read().splitlines()
    out = []
    for k in range(n):
        lines, sec = [], 0
        body = [x for x in src if x.strip() and not x.strip().startswith(("!", "#"))]
        lp, ln = map(int, body[0].split()[:2])
        nsp = int(body[1 + lp + ln].split()[0])
        first_spe = 2 + lp + ln
        first_tb = first_spe + nsp + 1
        for i, x in enumerate(body):
            t = x.split()
            if first_spe <= i < first_spe + nsp:
                t[2] = f"{float(t[2]) * (1 + rel * rng.standard_normal()):.6f}"
            elif i >= first_tb:
                t[5] = f"{float(t[5]) * (1 + rel * rng.standard_normal()):.6f}"
            lines.append(" ".join(t))
        p = os.path.join(d, f"tmp_{k}.snt")
        with open(p, "w") as f:
            f.write("\n".join(lines) + "\n")
        out.append(p)
        del sec
    return out


def test_prep_ec_and_solve_ec_o20(lib, tmp_path, monkeypatch, capsys):
    """The reference's EC workflow (test/ShellModel_test.jl:37-67) on O20,
    J = 0, 3 states, five seeded sample interactions: sampling writes the
    .wav files, "TD" writes the tdmat file, solveEC with usdb.  Checks: the
    TDs equal the oracle's; Σ ME·TD equals <w_i|H|w_j> from the GPU H·v;
    continuing to a sample interaction reproduces its exact eigenvalues; the
    usdb values are variational upper bounds and the .appwav vectors have
    those Rayleigh quotients."""
    from oracle.oracle import OracleProblem
    from smgpu import ShellModelProblem, prep_ec, solve_ec
    from smgpu.ec import read_snt_mes, read_tdmat
    from smgpu.wav import read_wav_full
    monkeypatch.chdir(tmp_path)
    os.makedirs("wavsamples")
    Hs = _perturbed_snts(str(tmp_path), 5)
    s = prep_ec(Hs, "O20", 3, 1, 0, "sample", path_to_samplewav="wavsamples/", save_wav=True)
    assert len(s["samples"]) == 5
    for smp in s["samples"]:
        e, j, v, mt = read_wav_full(smp["wav"], 81)
        assert mt == 0 and list(j) == [0, 0, 0] and np.allclose(e, smp["evals"], rtol=0, atol=0)
    t = prep_ec(Hs, "O20", 3, 5, 0, "TD", path_to_samplewav="wavsamples/")
    assert t["Dim"] == 15
    Dim, npair, lTD, Nmat, infos, TDs = read_tdmat("tdmat/O20_J0.dat")
    assert (Dim, npair, lTD) == (15, 120, 6 + 158)
    assert os.path.exists("tdmat/wfinfos_O20_J0.dat")
    svecs = np.concatenate([read_wav_full(f"wavsamples/O20_tmp_{k}_j0.wav", 81)[2] for k in range(5)])
    No, tdo = OracleProblem(Hs[0], "O20", mtot2=0).ec_td(svecs)
    assert np.allclose(Nmat, No, rtol=1e-13, atol=1e-15)
    assert np.abs(TDs - tdo).max() <= 1e-11 * np.abs(tdo).max()
    # Σ ME·TD = <w_i|H|w_j> through the GPU H·v
    P = ShellModelProblem(USDB, "O20", 0, twoJ=0)
    HV = P.matvec(svecs)
    Hdirect = svecs @ HV.T
    MEs = np.concatenate(read_snt_mes(USDB, "O20"))
    for (i, j, _), TD in zip(infos, TDs):
        assert abs(TD @ MEs - Hdirect[i - 1, j - 1]) < 1e-10 * max(1.0, abs(Hdirect[i - 1, j - 1]))
    # continuation to a sample interaction reproduces its exact levels
    r0 = solve_ec([Hs[0]], "O20", [[0, 3]], tdmatpath="./tdmat/", quiet=True)
    assert np.allclose(r0[0][2], s["samples"][0]["evals"], rtol=0, atol=1e-8)
    # usdb: variational bounds, .appwav Rayleigh quotients
    rs = solve_ec([USDB], "O20", [[0, 3]], write_appwav=True, wpath="./wavsamples", tdmatpath="./tdmat/")
    assert "vals [" in capsys.readouterr().out
    exact = P.solve(3, lm=60, ls=20, tol=1e-10, twoJ=0)["evals"]
    ec = rs[0][2]
    assert np.all(ec >= exact - 1e-8) and abs(ec[0] - exact[0]) < 0.5
    e, j, R, mt = read_wav_full("appwavs/O20_usdb_j0.appwav", 81)
    assert list(j) == [0, 0, 0] and mt == 0 and np.allclose(e, ec, rtol=0, atol=0)
    assert np.allclose(np.linalg.norm(R, axis=1), 1.0, atol=1e-12)
    rq = np.einsum("ij,ij->i", R, P.matvec(R))
    assert np.allclose(rq, ec, rtol=0, atol=1e-8)
