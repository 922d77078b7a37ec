"""GPU library vs the CPU oracle through the C ABI (needs a GB300)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CKPOT = os.path.join(GOLDEN, "ckpot.snt")
USDB = os.path.join(GOLDEN, "usdb.snt")

# Tolerances (stated here, used below)
MATVEC_FP64_RTOL = 1e-12   # FP64 H·v vs oracle operate_H!, relative to max|w|
MATVEC_MIXED_RTOL = 2e-6   # FP32-mixed H·v vs oracle, relative to max|w|
EIG_FP64_RTOL = 1e-8       # FP64 eigenvalues vs oracle TRL, relative
EIG_MIXED_ATOL = 1e-4      # FP32-mixed eigenvalues vs oracle, MeV


def _cases(snt_dir):
    return {
        "ckpot_Be8": (CKPOT, "Be8"),
        "usdb_Na21": (USDB, "Na21"),   # odd A, uneven vp/vn
        "usdb_O19": (USDB, "O19"),     # zero valence protons
        "sd2p2n": snt_dir["sd2p2n"],
        "sd4p4n": snt_dir["sd4p4n"],
    }


@pytest.fixture(scope="module")
def lib():
    from smgpu import _lib
    from smgpu import build as b
    b.build()
    return _lib.load()


def _oracle(snt, nuc):
    from oracle.oracle import OracleProblem
    return OracleProblem(snt, nuc)


def _gpu(snt, nuc, prec=0):
    from smgpu import ShellModelProblem
    return ShellModelProblem(snt, nuc, prec)


@pytest.mark.parametrize("case", ["ckpot_Be8", "usdb_Na21", "usdb_O19", "sd2p2n", "sd4p4n", "pf4p4n"])
def test_basis_bit_exact(lib, snt_dir, case):
    snt, nuc = snt_dir["pf4p4n"] if case == "pf4p4n" else _cases(snt_dir)[case]
    O, G = _oracle(snt, nuc), _gpu(snt, nuc)
    assert G.mdim == O.mdim and G.nblocks == O.nblocks
    assert np.array_equal(G.tdims, O.tdims)
    assert np.array_equal(G.np_, O.np_) and np.array_equal(G.nn_, O.nn_)
    assert np.array_equal(G.Mp, O.Mp) and np.array_equal(G.Mn, O.Mn)
    gp, gn = G.basis()
    op, on = O.sds()
    assert np.array_equal(gp.astype(np.int64), op) and np.array_equal(gn.astype(np.int64), on)


def _oracle_pn_set(O, which):
    """Distinct (bi, bf, op1, op2, i, f, phase) of the reference's per-V-entry lists."""
    bi, bf, nth, i, f, ph = O.jumps_pn(which)
    delMs, idx, abcd, V = O.vpn()
    # map (bi, bf, nth) -> operator bits: nth indexes Vpn[ΔM] for ΔM = Mps[bf]-Mps[bi]
    starts = np.concatenate([[0], np.cumsum(np.bincount(idx, minlength=len(delMs)))])
    Mps = O.Mp  # block M values; differences equal the reference's Mps differences
    out = set()
    for k in range(len(bi)):
        dm = int(Mps[bf[k] - 1] - Mps[bi[k] - 1])
        di = int(np.where(delMs == dm)[0][0])
        row = abcd[starts[di] + nth[k] - 1]
        ops = (int(row[0]), int(row[2])) if which == 0 else (int(row[1]), int(row[3]))
        out.add((int(bi[k]), int(bf[k])) + ops + (int(i[k]), int(f[k]), int(ph[k])))
    return out


@pytest.mark.parametrize("case", ["ckpot_Be8", "usdb_Na21", "sd2p2n", "sd4p4n"])
def test_jump_tables_match_reference(lib, snt_dir, case):
    snt, nuc = _cases(snt_dir)[case]
    O, G = _oracle(snt, nuc), _gpu(snt, nuc)
    for which in (0, 1):
        g = {tuple(map(int, r)) for r in G.jumps(which)}
        assert g == _oracle_pn_set(O, which), f"pn table {which}"
    for which, ow in ((2, 0), (3, 1)):
        ints, coef = G.jumps(which)
        blk, i, f, c = O.jumps_2b(ow)
        ref = {}
        for k in range(len(blk)):
            key = (int(blk[k]), int(i[k]), int(f[k]))
            ref[key] = ref.get(key, 0.0) + c[k]
        got = {tuple(map(int, r)): v for r, v in zip(ints, coef)}
        ref = {k: v for k, v in ref.items() if v != 0.0}
        got = {k: v for k, v in got.items() if v != 0.0}
        assert set(got) == set(ref)
        scale = max(abs(v) for v in ref.values())
        assert max(abs(got[k] - ref[k]) for k in ref) <= 1e-13 * scale


@pytest.mark.parametrize("case", ["ckpot_Be8", "usdb_Na21", "usdb_O19", "sd2p2n", "sd4p4n"])
def test_matvec_fp64_and_mixed(lib, snt_dir, case):
    snt, nuc = _cases(snt_dir)[case]
    O = _oracle(snt, nuc)
    v = np.random.default_rng(3).standard_normal(O.mdim)
    ref = O.operate_H(v)
    scale = np.abs(ref).max()
    G = _gpu(snt, nuc, 0)
    assert np.abs(G.matvec(v) - ref).max() <= MATVEC_FP64_RTOL * scale
    # accumulate = operate_H!'s "twf += H wf"
    w0 = np.full(O.mdim, 0.25)
    assert np.abs(G.matvec(v, accumulate=True, out=w0.copy()) - (ref + 0.25)).max() <= MATVEC_FP64_RTOL * scale
    M = _gpu(snt, nuc, 1)
    assert np.abs(M.matvec(v) - ref).max() <= MATVEC_MIXED_RTOL * scale


def test_matvec_pf_full_size(lib, snt_dir):
    """48Cr pf (dim 1,963,461): FP64 H·v vs the oracle, mixed vs FP64, and
    the size-independent symmetry <u,Hv> = <Hu,v>."""
    snt, nuc = snt_dir["pf4p4n"]
    O = _oracle(snt, nuc)
    rng = np.random.default_rng(5)
    v = rng.standard_normal(O.mdim)
    u = rng.standard_normal(O.mdim)
    ref = O.operate_H(v)
    G = _gpu(snt, nuc, 0)
    w = G.matvec(v)
    scale = np.abs(ref).max()
    assert np.abs(w - ref).max() <= MATVEC_FP64_RTOL * scale
    hu = G.matvec(u)
    assert abs(u @ w - hu @ v) <= 1e-12 * np.linalg.norm(u) * np.linalg.norm(w)
    M = _gpu(snt, nuc, 1)
    assert np.abs(M.matvec(v) - ref).max() <= MATVEC_MIXED_RTOL * scale


@pytest.mark.parametrize("form", ["tile", "staged"])
@pytest.mark.parametrize("case", ["ckpot_Be8", "usdb_Na21", "usdb_O19", "sd2p2n", "sd4p4n"])
def test_matvec_mixed_each_kernel_form(lib, snt_dir, case, form, monkeypatch):
    """Both FP32-mixed H·v kernels — the row-tile pull kernel and the staged
    pn kernel — against the oracle's operate_H!, and the eigenvalues of a
    solve that runs on the chosen kernel (its double-float epilogue)."""
    snt, nuc = _cases(snt_dir)[case]
    monkeypatch.setenv("SMGPU_HV_FORM", form)
    O = _oracle(snt, nuc)
    v = np.random.default_rng(11).standard_normal(O.mdim)
    ref = O.operate_H(v)
    M = _gpu(snt, nuc, 1)
    assert M.stats()["hv_staged"] == (1 if form == "staged" else 0)
    assert all(c["staged"] == (1 if form == "staged" else 0) for c in M.tune_report())
    assert np.abs(M.matvec(v) - ref).max() <= MATVEC_MIXED_RTOL * np.abs(ref).max()
    lm = min(40, O.mdim - 5)  # O19 has dimension 37
    ro = O.trl(5, lm=lm, ls=15, tol=1e-8)
    rm = M.solve(5, lm=lm, ls=15, tol=1e-8)
    assert rm["converged"]
    assert np.abs(rm["evals"] - ro["evals"]).max() <= EIG_MIXED_ATOL


@pytest.mark.parametrize("form", ["tile", "staged"])
def test_matvec_mixed_each_kernel_form_pf(lib, snt_dir, form, monkeypatch):
    """48Cr pf: each FP32-mixed H·v kernel against the FP64 kernel (which
    equals the oracle to 1e-12, test_matvec_pf_full_size), on two vectors,
    and the symmetry <u,Hv> = <Hu,v> of the mixed form."""
    snt, nuc = snt_dir["pf4p4n"]
    G = _gpu(snt, nuc, 0)
    monkeypatch.setenv("SMGPU_HV_FORM", form)
    M = _gpu(snt, nuc, 1)
    assert M.stats()["hv_staged"] == (1 if form == "staged" else 0)
    rng = np.random.default_rng(12)
    u = rng.standard_normal(G.mdim)
    v = rng.standard_normal(G.mdim)
    ref = G.matvec(v)
    w = M.matvec(v)
    assert np.abs(w - ref).max() <= MATVEC_MIXED_RTOL * np.abs(ref).max()
    hu = M.matvec(u)
    assert abs(u @ w - hu @ v) <= 1e-6 * np.linalg.norm(u) * np.linalg.norm(w)


def _shapes(snt, nuc, prec, form, monkeypatch):
    """The candidate H·v launch shapes of one kernel form for this problem."""
    monkeypatch.delenv("SMGPU_HV_SHAPE", raising=False)
    monkeypatch.setenv("SMGPU_HV_FORM", form)
    shapes = [(c["threads"], c["rows"], c["min_ctas"], c["staged"]) for c in _gpu(snt, nuc, prec).tune_report()]
    monkeypatch.delenv("SMGPU_HV_FORM", raising=False)
    return shapes


@pytest.mark.parametrize("case", ["usdb_Na21", "sd4p4n"])
def test_matvec_every_launch_shape(lib, snt_dir, case, monkeypatch):
    """Every candidate launch shape of every H·v kernel (FP64 row-tile; FP32
    row-tile and staged) against the oracle, not only the autotuner's pick;
    the staged shapes also through a solve (double-float epilogue)."""
    snt, nuc = _cases(snt_dir)[case]
    O = _oracle(snt, nuc)
    v = np.random.default_rng(13).standard_normal(O.mdim)
    ref = O.operate_H(v)
    scale = np.abs(ref).max()
    ro = O.trl(5, lm=30, ls=15, tol=1e-8) if case == "usdb_Na21" else None
    runs = [(0, sh) for sh in _shapes(snt, nuc, 0, "tile", monkeypatch)]
    runs += [(1, sh) for sh in _shapes(snt, nuc, 1, "tile", monkeypatch)]
    runs += [(1, sh) for sh in _shapes(snt, nuc, 1, "staged", monkeypatch)]
    assert len(runs) >= 13 + 13 + 5
    for prec, sh in runs:
        monkeypatch.setenv("SMGPU_HV_SHAPE", ",".join(map(str, sh)))
        G = _gpu(snt, nuc, prec)
        st = G.stats()
        assert (st["hv_threads"], st["hv_rows"], st["hv_min_ctas"], st["hv_staged"]) == sh
        tol = MATVEC_FP64_RTOL if prec == 0 else MATVEC_MIXED_RTOL
        assert np.abs(G.matvec(v) - ref).max() <= tol * scale, sh
        if ro is not None and sh[3] == 1:
            # both epilogues of the staged kernel: FP64 residual (MIXED) and
            # double-float residual (MIXED_DF)
            for H in (G, _gpu(snt, nuc, 2)):
                rm = H.solve(5, lm=30, ls=15, tol=1e-8)
                assert rm["converged"] and np.abs(rm["evals"] - ro["evals"]).max() <= EIG_MIXED_ATOL, sh
    monkeypatch.setenv("SMGPU_HV_SHAPE", "999,1,1,1")
    with pytest.raises(Exception):
        _gpu(snt, nuc, 1)


def test_ckpot_known_answer_on_gpu(lib, golden):
    g = golden["ckpot_Be8"]
    for prec in (0, 1):
        G = _gpu(CKPOT, "Be8", prec)
        r = G.solve(10, lm=300, ls=20, tol=1e-8)
        assert r["converged"]
        for e, ref in zip(r["evals"], g["energies"]):
            assert (e - ref) ** 2 < g["tolerance_sq"]


@pytest.mark.parametrize("case,nev,lm,ls", [("sd2p2n", 5, 300, 20), ("sd4p4n", 10, 30, 15), ("usdb_Na21", 5, 40, 15),
                                            ("sd4p4n", 5, 100, 20)])
def test_eigenvalues_vs_oracle(lib, snt_dir, case, nev, lm, ls):
    snt, nuc = _cases(snt_dir)[case]
    O = _oracle(snt, nuc)
    ro = O.trl(nev, lm=lm, ls=ls, tol=1e-8)
    assert ro["converged"]
    G = _gpu(snt, nuc, 0)
    rg = G.solve(nev, lm=lm, ls=ls, tol=1e-8)
    assert rg["converged"]
    assert np.allclose(rg["evals"], ro["evals"], rtol=EIG_FP64_RTOL, atol=0)
    for prec in (1, 2):  # FP32-mixed with FP64 / double-float Lanczos arithmetic
        M = _gpu(snt, nuc, prec)
        rm = M.solve(nev, lm=lm, ls=ls, tol=1e-8)
        assert rm["converged"], prec
        assert np.abs(rm["evals"] - ro["evals"]).max() <= EIG_MIXED_ATOL, prec


@pytest.mark.parametrize("case", ["sd4p4n", "usdb_Na21"])
def test_mixed_beta_from_norm_before_subtraction_both_paths(lib, snt_dir, case, monkeypatch):
    """The FP32-mixed solve with FP64 re-orthogonalisation takes β from the
    norm before the subtraction when the projections are small, and the norm
    after the subtraction otherwise; SMGPU_FASTNORM=0 forces the latter in
    every iteration.  Both paths against the oracle, with the same iteration
    count."""
    snt, nuc = _cases(snt_dir)[case]
    ro = _oracle(snt, nuc).trl(5, lm=30, ls=15, tol=1e-8)
    res = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("SMGPU_FASTNORM", mode)
        r = _gpu(snt, nuc, 1).solve(5, lm=30, ls=15, tol=1e-8)
        assert r["converged"], mode
        assert np.abs(r["evals"] - ro["evals"]).max() <= EIG_MIXED_ATOL, mode
        res[mode] = r
    assert res["1"]["n_matvec"] == res["0"]["n_matvec"]
    assert np.abs(res["1"]["evals"] - res["0"]["evals"]).max() <= 1e-6


@pytest.mark.parametrize("prec", [1, 2])
def test_ritz_vectors_mixed(lib, snt_dir, prec):
    """Ritz vectors of both FP32-mixed forms (FP64 or double-float Lanczos
    arithmetic): unit norm, small residual, overlap with the oracle's."""
    snt, nuc = snt_dir["sd4p4n"]
    M = _gpu(snt, nuc, prec)
    r = M.solve(3, lm=40, ls=15, tol=1e-10, want_vecs=True)
    O = _oracle(snt, nuc)
    ro = O.trl(3, lm=40, ls=15, tol=1e-10, want_vecs=True)
    for k in range(3):
        x = r["evecs"][k]
        assert abs(np.linalg.norm(x) - 1) < 1e-10
        assert np.linalg.norm(O.operate_H(x) - r["evals"][k] * x) < 1e-2
        assert abs(abs(x @ ro["evecs"][k]) - 1.0) < 1e-5


def test_ritz_vectors(lib, snt_dir):
    snt, nuc = snt_dir["sd4p4n"]
    G = _gpu(snt, nuc, 0)
    r = G.solve(3, lm=40, ls=15, tol=1e-10, want_vecs=True)
    X = r["evecs"]
    for k in range(3):
        x = X[k]
        assert abs(np.linalg.norm(x) - 1) < 1e-12
        res = G.matvec(x) - r["evals"][k] * x
        assert np.linalg.norm(res) < 1e-3
    O = _oracle(snt, nuc)
    ro = O.trl(3, lm=40, ls=15, tol=1e-10, want_vecs=True)
    for k in range(3):
        assert abs(abs(X[k] @ ro["evecs"][k]) - 1.0) < 1e-6


def test_user_start_vector_and_noconv(lib, snt_dir):
    from smgpu import _lib as L
    snt, nuc = snt_dir["sd2p2n"]
    G = _gpu(snt, nuc, 0)
    v1 = np.ones(G.mdim)
    r = G.solve(3, lm=30, ls=10, tol=1e-8, v1=v1)
    O = _oracle(snt, nuc)
    ro = O.trl(3, lm=30, ls=10, tol=1e-8, v1=v1)
    assert np.allclose(r["evals"], ro["evals"], rtol=EIG_FP64_RTOL)
    r2 = G.solve(5, lm=8, ls=3, tol=1e-14, max_restarts=1)
    assert r2["status"] == L.ERR_NOCONV and not r2["converged"]


def test_error_paths(lib, tmp_path):
    from smgpu import SmgpuError, ShellModelProblem
    from smgpu import _lib as L
    with pytest.raises(SmgpuError) as e:
        ShellModelProblem(str(tmp_path / "missing.snt"), "Be8")
    assert e.value.code == L.ERR_IO
    with pytest.raises(SmgpuError) as e:
        ShellModelProblem(CKPOT, "Xx8")
    assert e.value.code == L.ERR_NUCLEUS
    bad = tmp_path / "bad.snt"
    bad.write_text("2 2 2 2\n1 0 1 1 -1\n")
    with pytest.raises(SmgpuError) as e:
        ShellModelProblem(str(bad), "Be8")
    assert e.value.code == L.ERR_PARSE
    with pytest.raises(SmgpuError) as e:
        ShellModelProblem(CKPOT, "He3")  # below the snt core
    assert e.value.code == L.ERR_NUCLEUS
    G = ShellModelProblem(CKPOT, "Be8")
    with pytest.raises(SmgpuError) as e:
        G.solve(0)
    assert e.value.code == L.ERR_ARG


def test_main_sm_mirror(lib, golden):
    from smgpu import main_sm
    en = main_sm(CKPOT, "Be8", 10, [], verbose=False)
    for e, ref in zip(en, golden["ckpot_Be8"]["energies"]):
        assert (e - ref) ** 2 < 1e-6


def test_main_sm_prints_j_labels(lib, capsys):
    """main_sm prints the J of every state before the energies
    (shellmodel_main.jl:226-240,257)."""
    from smgpu import main_sm
    main_sm(CKPOT, "Be8", 10, [], verbose=True)
    out = capsys.readouterr().out
    assert "J [0.0, 2.0, 4.0, 2.0, 1.0, 2.0, 3.0, 1.0, 0.0, 4.0]" in out


def test_jj_on_gpu_matches_oracle(lib, snt_dir):
    """<J^2> of Ritz vectors: GPU (two-body form of J^2) vs the oracle's
    ladder operator, FP64 and mixed forms."""
    from smgpu.shellmodel import J_from_JJ1
    G = _gpu(CKPOT, "Be8", 0)
    r = G.solve(10, lm=60, ls=20, tol=1e-10, want_vecs=True)
    jj = G.jj(r["evecs"])
    O = _oracle(CKPOT, "Be8")
    for x, j in zip(r["evecs"], jj):
        assert abs(j - O.jj(x)) < 1e-9
    assert [J_from_JJ1(x) for x in jj] == [0, 2, 4, 2, 1, 2, 3, 1, 0, 4]
    snt, nuc = snt_dir["sd4p4n"]
    M = _gpu(snt, nuc, 1)
    r = M.solve(3, lm=40, ls=15, tol=1e-10, want_vecs=True)
    O = _oracle(snt, nuc)
    jj = M.jj(r["evecs"])
    for x, j in zip(r["evecs"], jj):
        assert abs(j - O.jj(x)) < 1e-9 * max(1.0, abs(j))
        twoJ = np.sqrt(1 + 4 * j) - 1
        assert abs(twoJ - round(twoJ)) < 1e-4


def test_main_sm_save_wav_and_in_wf(lib, tmp_path, monkeypatch):
    """save_wav writes ./Be8_ckpot.wav (writeRitzvecs, shellmodel_main.jl:
    248-253); in_wf restarts from its first vector (read_appwav, :196-198)."""
    from smgpu import main_sm
    from smgpu.wav import read_wav_full
    monkeypatch.chdir(tmp_path)
    en = main_sm(CKPOT, "Be8", 5, [], save_wav=True, verbose=False)
    e, j, v, mt = read_wav_full(str(tmp_path / "Be8_ckpot.wav"), 51)
    assert mt == 0 and np.allclose(e, en, rtol=0, atol=0)
    assert list(j) == [0, 4, 8, 4, 2]
    assert np.allclose(np.linalg.norm(v, axis=1), 1.0, atol=1e-10)
    en2 = main_sm(CKPOT, "Be8", 5, [], in_wf=str(tmp_path / "Be8_ckpot.wav"), verbose=False)
    assert np.allclose(en2, en, rtol=1e-8, atol=0)


@pytest.mark.parametrize("snt,nuc,twoJ,nev", [(CKPOT, "Be8", 0, 2), (CKPOT, "Be8", 4, 3), (CKPOT, "Be8", 6, 1),
                                              (USDB, "Ne20", 4, 3), (USDB, "Na21", 3, 2)])
def test_j_projected_lanczos_vs_oracle(lib, snt, nuc, twoJ, nev):
    """target_J = [twoJ]: the double Lanczos (lanczos_methods.jl:1-151) on
    the GPU against the oracle's restatement; handles of both precisions
    (the projected solve runs in FP64); the Ritz vectors have <J^2> = J(J+1)."""
    from oracle.oracle import OracleProblem
    J = twoJ / 2
    O = OracleProblem(snt, nuc, mtot2=twoJ)
    ro = O.trl(nev, lm=30, ls=15, tol=1e-8, eval_jj=J * (J + 1))
    assert ro["converged"]
    for prec in (0, 1):
        G = _gpu_J(snt, nuc, prec, twoJ)
        r = G.solve(nev, lm=30, ls=15, tol=1e-8, twoJ=twoJ, want_vecs=True)
        assert r["converged"], prec
        assert np.allclose(r["evals"], ro["evals"], rtol=EIG_FP64_RTOL, atol=0), (prec, r["evals"], ro["evals"])
        jj = G.jj(r["evecs"])
        assert np.abs(jj - J * (J + 1)).max() < 1e-5, jj


def _gpu_J(snt, nuc, prec, twoJ):
    from smgpu import ShellModelProblem
    return ShellModelProblem(snt, nuc, prec, twoJ=twoJ)


def test_main_sm_target_j(lib, golden, capsys):
    """main_sm(..., [0]) gives the J = 0 levels of the ckpot 8Be spectrum
    (levels 1 and 9 of test/ShellModel_test.jl:8-15)."""
    from smgpu import main_sm
    en = main_sm(CKPOT, "Be8", 2, [0])
    ref = golden["ckpot_Be8"]["energies"]
    assert (en[0] - ref[0]) ** 2 < 1e-6 and (en[1] - ref[8]) ** 2 < 1e-6
    assert "2J= 0  En." in capsys.readouterr().out


def test_block_lanczos_ckpot_known_answer(lib, golden):
    """test/ShellModel_test.jl:8-15 runs main_sm(..., "Be8", 10, []; q=2,
    is_block=true): the block Lanczos must reproduce the 10 levels."""
    from smgpu import main_sm
    en = main_sm(CKPOT, "Be8", 10, [], q=2, is_block=True, verbose=False)
    for e, ref in zip(en, golden["ckpot_Be8"]["energies"]):
        assert (e - ref) ** 2 < golden["ckpot_Be8"]["tolerance_sq"]


@pytest.mark.parametrize("q", [2, 3])
def test_block_lanczos_vs_oracle(lib, snt_dir, q):
    """TRBL on the GPU against the oracle's restatement (sd 4p4n, lm=30,
    ls=15), FP64, with Ritz vectors."""
    snt, nuc = snt_dir["sd4p4n"]
    O = _oracle(snt, nuc)
    ro = O.trbl(q, 5, lm=30, ls=15, tol=1e-8)
    assert ro["converged"]
    G = _gpu(snt, nuc, 0)
    r = G.solve(5, lm=30, ls=15, tol=1e-8, block=q, want_vecs=True)
    assert r["converged"] and r["n_matvec"] > 0
    assert np.allclose(r["evals"], ro["evals"], rtol=EIG_FP64_RTOL, atol=0), (r["evals"], ro["evals"])
    for k in range(2):
        x = r["evecs"][k]
        assert abs(np.linalg.norm(x) - 1) < 1e-10
        assert np.linalg.norm(O.operate_H(x) - r["evals"][k] * x) < 1e-3
