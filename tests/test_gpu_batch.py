"""Batches of independent problems (smgpu_batch_*) vs the CPU oracle, problem
by problem, through the C ABI (needs a GB300).

Each problem of a batch must give what its own main_sm call gives
(src/ShellModel/shellmodel_main.jl:89-281): here, what the oracle gives for
the same snt file and nucleus."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

MATVEC_MIXED_RTOL = 2e-6   # batched FP32-mixed H·v vs oracle operate_H!, relative to max|w_p|
EIG_MIXED_ATOL = 1e-4      # FP32-mixed eigenvalues vs oracle TRL, per problem, MeV
RITZ_RESID = 1e-3          # ||H x - λ x|| of a unit Ritz vector (mixed form)

CKPOT = os.path.join(GOLDEN, "ckpot.snt")
USDB = os.path.join(GOLDEN, "usdb.snt")


@pytest.fixture(scope="module")
def lib():
    from smgpu import _lib
    from smgpu import build as b
    b.build()
    return _lib.load()


@pytest.fixture(scope="module")
def mixed_batch(tmp_path_factory):
    """Uneven problems from three interactions and two shells, including a
    dimension-1 problem (no valence particles), odd A and a zero-valence
    species."""
    from smgpu import synth
    d = str(tmp_path_factory.mktemp("batch"))
    probs = [(CKPOT, "Be8"), (USDB, "O16"), (USDB, "F17"), (USDB, "Na21"), (USDB, "O19"), (CKPOT, "Li7")]
    probs += synth.sd_batch_snts(d, 14)[:14]
    return probs


def _oracle(snt, nuc):
    from oracle.oracle import OracleProblem
    return OracleProblem(snt, nuc)


def _batch(probs):
    from smgpu import BatchProblem
    return BatchProblem(probs)


def test_batch_matvec_vs_oracle(lib, mixed_batch):
    G = _batch(mixed_batch)
    assert G.nprob == len(mixed_batch)
    v = np.random.default_rng(13).standard_normal(G.total_mdim)
    w = G.split(G.matvec(v))
    w_acc = G.split(G.matvec(v, accumulate=True, out=np.full(G.total_mdim, 0.25)))
    for p, ((snt, nuc), vp) in enumerate(zip(mixed_batch, G.split(v))):
        O = _oracle(snt, nuc)
        assert O.mdim == G.mdims[p], nuc
        ref = O.operate_H(vp)
        scale = max(np.abs(ref).max(), 1e-30)
        assert np.abs(w[p] - ref).max() <= MATVEC_MIXED_RTOL * scale, (p, nuc)
        assert np.abs(w_acc[p] - (ref + 0.25)).max() <= MATVEC_MIXED_RTOL * scale, (p, nuc)


def test_batch_matvec_every_launch_shape(lib, mixed_batch, monkeypatch):
    """Every candidate launch shape of the batched H·v against the oracle."""
    from smgpu import _lib
    probs = mixed_batch[:8]
    v = None
    refs = None
    ncand = 0
    n_staged = 0
    while True:
        monkeypatch.setenv("SMGPU_BATCH_CAND", str(ncand))
        try:
            G = _batch(probs)
        except _lib.SmgpuError:
            break  # past the last candidate
        if v is None:
            v = np.random.default_rng(19).standard_normal(G.total_mdim)
            refs = [_oracle(snt, nuc).operate_H(vp) for (snt, nuc), vp in zip(probs, G.split(v))]
        w = G.split(G.matvec(v))
        for p, ref in enumerate(refs):
            scale = max(np.abs(ref).max(), 1e-30)
            assert np.abs(w[p] - ref).max() <= MATVEC_MIXED_RTOL * scale, (ncand, p)
        n_staged += G.stats()["hv_staged"]
        ncand += 1
    assert ncand >= 5
    assert n_staged >= 1  # the staged pn row body ran on the batch


def test_batch_solve_vs_oracle(lib, mixed_batch):
    G = _batch(mixed_batch)
    r = G.solve(5, lm=30, ls=15, tol=1e-8, want_vecs=True)
    assert r["converged"] and r["problem_converged"].all()
    assert r["n_matvec"] > 0
    for p, (snt, nuc) in enumerate(mixed_batch):
        O = _oracle(snt, nuc)
        ro = O.trl(5, lm=30, ls=15, tol=1e-8)
        assert ro["converged"]
        nev = len(ro["evals"])
        assert np.abs(r["evals"][p, :nev] - ro["evals"]).max() <= EIG_MIXED_ATOL, (p, nuc)
        assert np.isnan(r["evals"][p, nev:]).all()
        for k in range(min(nev, 2)):
            x = r["evecs"][p][k]
            assert abs(np.linalg.norm(x) - 1.0) < 1e-10, (p, k)
            assert np.linalg.norm(O.operate_H(x) - r["evals"][p, k] * x) < RITZ_RESID, (p, nuc, k)


@pytest.fixture(scope="module")
def golden_runs():
    import json
    with open(os.path.join(GOLDEN, "oracle_runs.json")) as f:
        return json.load(f)


def test_batch_of_128_sd_problems(lib, tmp_path, golden_runs):
    """The uneven batch of 128 sd problems (dims 28 .. 93,710): every problem
    converges; problems spanning the sizes against the oracle."""
    from smgpu import synth
    probs = synth.sd_batch_snts(str(tmp_path), 128)
    G = _batch(probs)
    assert G.nprob == 128 and G.mdims.min() == 28 and G.mdims.max() == 93710
    r = G.solve(5, lm=30, ls=15, tol=1e-8)
    assert r["converged"] and r["problem_converged"].all()
    order = np.argsort(G.mdims)
    for p in [int(order[k]) for k in (0, 20, 60)]:
        ro = _oracle(*probs[p]).trl(5, lm=30, ls=15, tol=1e-8)
        nev = len(ro["evals"])
        assert np.abs(r["evals"][p, :nev] - ro["evals"]).max() <= EIG_MIXED_ATOL, (p, probs[p][1])
    # every problem against the stored oracle run of the same batch
    gb = golden_runs["sd_batch128"]
    for p, q in enumerate(gb["problems"]):
        assert q["mdim"] == G.mdims[p] and q["nucleus"] == probs[p][1]
        ref = np.array(q["evals"])
        assert np.abs(r["evals"][p, :len(ref)] - ref).max() <= EIG_MIXED_ATOL, (p, q["nucleus"])


def test_batch_noconv_and_error_paths(lib, mixed_batch, tmp_path):
    from smgpu import SmgpuError
    from smgpu import _lib as L
    G = _batch(mixed_batch[6:10])
    r = G.solve(5, lm=8, ls=3, tol=1e-14, max_restarts=1)
    assert r["status"] == L.ERR_NOCONV and not r["converged"]
    with pytest.raises(SmgpuError) as e:
        G.solve(0)
    assert e.value.code == L.ERR_ARG
    with pytest.raises(SmgpuError) as e:
        _batch([(CKPOT, "Be8"), (str(tmp_path / "missing.snt"), "Be8")])
    assert e.value.code == L.ERR_IO
    with pytest.raises(SmgpuError) as e:
        _batch([(CKPOT, "Be8"), (CKPOT, "He3")])
    assert e.value.code == L.ERR_NUCLEUS


PERSIST_CANDS = (3, 4, 6, 8, 9, 10)  # batched H·v shapes that have a persistent cycle kernel


def test_batch_persistent_cycle_every_shape(lib, mixed_batch, monkeypatch):
    """The persistent form (one cooperative launch per restart cycle: H·v over
    a device task queue, eigenvalue tests, re-orthogonalisation passes, each
    phase behind a grid barrier) for every H·v shape that has one, against
    the oracle and against the graph form; far fewer launches."""
    probs = mixed_batch[:10]
    refs = []
    for snt, nuc in probs:
        ro = _oracle(snt, nuc).trl(5, lm=30, ls=15, tol=1e-8)
        refs.append(ro["evals"])
    for cand in PERSIST_CANDS:
        monkeypatch.setenv("SMGPU_BATCH_CAND", str(cand))
        G = _batch(probs)
        monkeypatch.setenv("SMGPU_BATCH_PERSIST", "0")
        rg = G.solve(5, lm=30, ls=15, tol=1e-8)
        monkeypatch.delenv("SMGPU_BATCH_PERSIST")
        rp = G.solve(5, lm=30, ls=15, tol=1e-8)
        assert rp["converged"] and rp["problem_converged"].all(), cand
        for p, ref in enumerate(refs):
            nev = len(ref)
            assert np.abs(rp["evals"][p, :nev] - ref).max() <= EIG_MIXED_ATOL, (cand, p)
            assert np.abs(rp["evals"][p, :nev] - rg["evals"][p, :nev]).max() <= EIG_MIXED_ATOL, (cand, p)
        # persistent: per cycle the cycle kernel, the cycle end and 6 restart kernels
        assert rp["kernel_launches"] <= 8 * (rp["n_restart"] + 1) + 3, (cand, rp["kernel_launches"])
        assert rp["kernel_launches"] * 5 < rg["kernel_launches"], cand


def test_batch_beta_from_norm_before_subtraction_both_paths(lib, mixed_batch, monkeypatch):
    """The batched solve takes β from the norm before the subtraction when a
    problem's projections are small; SMGPU_FASTNORM=0 forces the norm after
    the subtraction (and the scaling pass) in every iteration.  Both paths,
    persistent and graph form, against the oracle."""
    probs = mixed_batch[:8]
    refs = [_oracle(snt, nuc).trl(5, lm=30, ls=15, tol=1e-8)["evals"] for snt, nuc in probs]
    for mode in ("1", "0"):
        monkeypatch.setenv("SMGPU_FASTNORM", mode)
        G = _batch(probs)
        for persist in ("1", "0"):
            monkeypatch.setenv("SMGPU_BATCH_PERSIST", persist)
            r = G.solve(5, lm=30, ls=15, tol=1e-8)
            assert r["converged"] and r["problem_converged"].all(), (mode, persist)
            for p, ref in enumerate(refs):
                nev = len(ref)
                assert np.abs(r["evals"][p, :nev] - ref).max() <= EIG_MIXED_ATOL, (mode, persist, p)
    monkeypatch.delenv("SMGPU_BATCH_PERSIST")
    monkeypatch.delenv("SMGPU_FASTNORM")


def test_batch_persistent_barrier_wait_limit(lib, mixed_batch, monkeypatch):
    """Every grid-barrier wait of the persistent kernel is bounded: with a
    wait limit of one poll the kernel gives up at its first barrier, the solve
    reports SMGPU_ERR_DEVICE, and the handle solves normally afterwards."""
    from smgpu import SmgpuError
    from smgpu import _lib as L
    G = _batch(mixed_batch[:6])
    r0 = G.solve(5, lm=30, ls=15, tol=1e-8)
    monkeypatch.setenv("SMGPU_BATCH_SPIN_LIMIT", "1")
    with pytest.raises(SmgpuError) as e:
        G.solve(5, lm=30, ls=15, tol=1e-8)
    assert e.value.code == L.ERR_DEVICE and "wait limit" in str(e.value)
    monkeypatch.delenv("SMGPU_BATCH_SPIN_LIMIT")
    r1 = G.solve(5, lm=30, ls=15, tol=1e-8)
    assert r1["converged"]
    assert np.array_equal(np.nan_to_num(r1["evals"]), np.nan_to_num(r0["evals"]))
