"""Interaction samples sharing one basis (smgpu_multi_*) vs the CPU oracle,
sample by sample, through the C ABI (needs a GB300).

The reference runs such samples one after another (prepEC's sample loop,
src/ShellModel/eigenvector_continuation.jl:140-177); here every sample of a
handle must give the same results as its own oracle problem."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

MATVEC_MIXED_RTOL = 2e-6   # multi-sample FP32-mixed H·V vs oracle operate_H!, relative to max|w_s|
EIG_MIXED_ATOL = 1e-4      # FP32-mixed eigenvalues vs oracle TRL, per sample, MeV
RITZ_RESID = 1e-3          # ||H x - λ x|| of a unit Ritz vector (mixed form)


@pytest.fixture(scope="module")
def lib():
    from smgpu import _lib
    from smgpu import build as b
    b.build()
    return _lib.load()


@pytest.fixture(scope="module")
def samples(tmp_path_factory):
    """sd 4p+4n (24Mg, dim 28,503) and sd 2p+2n (20Ne, dim 640) sample sets:
    base N(0,1.5²) + N(0,0.15²) per sample."""
    from smgpu import synth
    d = str(tmp_path_factory.mktemp("multi"))
    out = {}
    for n in (3, 5, 16):
        out[("sd4p4n", n)] = synth.multi_snts(os.path.join(d, f"mg{n}"), "sd", 4, 4, n, 24000, 1.5, 0.15, "s")
    out[("sd2p2n", 16)] = synth.multi_snts(os.path.join(d, "ne16"), "sd", 2, 2, 16, 20000, 1.5, 0.15, "s")
    return out


NUC = {"sd4p4n": "Mg24", "sd2p2n": "Ne20"}


def _oracle(snt, nuc):
    from oracle.oracle import OracleProblem
    return OracleProblem(snt, nuc)


def _multi(files, nuc):
    from smgpu import MultiSampleProblem
    return MultiSampleProblem(files, nuc)


@pytest.mark.parametrize("n", [3, 5, 16])
def test_multi_matvec_vs_oracle(lib, samples, n):
    files = samples[("sd4p4n", n)]
    G = _multi(files, "Mg24")
    assert G.nsamples == n and G.lanes == (4 if n <= 4 else 8 if n <= 8 else 16)
    v = np.random.default_rng(7).standard_normal((n, G.mdim))
    w = G.matvec(v)
    w_acc = G.matvec(v, accumulate=True, out=np.full((n, G.mdim), 0.5))
    for s, f in enumerate(files):
        ref = _oracle(f, "Mg24").operate_H(v[s])
        scale = np.abs(ref).max()
        assert np.abs(w[s] - ref).max() <= MATVEC_MIXED_RTOL * scale, s
        assert np.abs(w_acc[s] - (ref + 0.5)).max() <= MATVEC_MIXED_RTOL * scale, s


def test_multi_matvec_every_launch_shape(lib, samples, monkeypatch):
    """Every candidate launch shape of the multi-sample H·V (threads, register
    cap, cached neutron entries) against the oracle, 16 samples."""
    from smgpu import _lib
    files = samples[("sd2p2n", 16)]
    v = np.random.default_rng(17).standard_normal((16, 640))
    refs = [_oracle(f, "Ne20").operate_H(v[s]) for s, f in enumerate(files)]
    ncand = 0
    while True:
        monkeypatch.setenv("SMGPU_MULTI_CAND", str(ncand))
        try:
            G = _multi(files, "Ne20")
        except _lib.SmgpuError:
            break  # past the last candidate
        w = G.matvec(v)
        for s in range(16):
            assert np.abs(w[s] - refs[s]).max() <= MATVEC_MIXED_RTOL * np.abs(refs[s]).max(), (ncand, s)
        ncand += 1
    assert ncand >= 5


def test_multi_solve_vs_oracle(lib, samples):
    """5 samples (8 lanes, 3 idle), the pf workload's Lanczos parameters."""
    files = samples[("sd4p4n", 5)]
    G = _multi(files, "Mg24")
    r = G.solve(5, lm=30, ls=15, tol=1e-8)
    assert r["converged"] and r["sample_converged"].all()
    assert r["n_matvec"] > 0 and (r["elit"] > 0).all()
    for s, f in enumerate(files):
        ro = _oracle(f, "Mg24").trl(5, lm=30, ls=15, tol=1e-8)
        assert ro["converged"]
        assert np.abs(r["evals"][s] - ro["evals"]).max() <= EIG_MIXED_ATOL, s


def test_multi_solve_16_samples_with_ritz_vectors(lib, samples):
    files = samples[("sd2p2n", 16)]
    G = _multi(files, "Ne20")
    r = G.solve(5, lm=30, ls=15, tol=1e-8, want_vecs=True)
    assert r["converged"]
    for s, f in enumerate(files):
        O = _oracle(f, "Ne20")
        ro = O.trl(5, lm=30, ls=15, tol=1e-8)
        assert np.abs(r["evals"][s] - ro["evals"]).max() <= EIG_MIXED_ATOL, s
        for k in range(3):
            x = r["evecs"][s, k]
            assert abs(np.linalg.norm(x) - 1.0) < 1e-10
            assert np.linalg.norm(O.operate_H(x) - r["evals"][s, k] * x) < RITZ_RESID, (s, k)


def test_multi_pf_full_size(lib, snt_dir, tmp_path):
    """The 48Cr pf basis (dim 1,963,461) shared by 16 samples: two samples
    against the oracle, and <u,H_s v> = <H_s u,v> for every sample."""
    from smgpu import synth
    files = synth.pf_multi_snts(str(tmp_path))
    G = _multi(files, "Cr48")
    assert G.mdim == 1963461 and G.lanes == 16
    rng = np.random.default_rng(11)
    v = rng.standard_normal((16, G.mdim))
    u = rng.standard_normal((16, G.mdim))
    w = G.matvec(v)
    hu = G.matvec(u)
    for s in (0, 15):
        ref = _oracle(files[s], "Cr48").operate_H(v[s])
        assert np.abs(w[s] - ref).max() <= MATVEC_MIXED_RTOL * np.abs(ref).max(), s
    for s in range(16):
        lhs, rhs = u[s] @ w[s], hu[s] @ v[s]
        assert abs(lhs - rhs) <= 1e-5 * np.linalg.norm(u[s]) * np.linalg.norm(w[s]), s


def test_multi_noconv_and_error_paths(lib, samples, tmp_path):
    from smgpu import SmgpuError, synth
    from smgpu import _lib as L
    files = samples[("sd2p2n", 16)][:4]
    G = _multi(files, "Ne20")
    r = G.solve(5, lm=8, ls=3, tol=1e-14, max_restarts=1)
    assert r["status"] == L.ERR_NOCONV and not r["converged"]
    assert np.isfinite(r["evals"]).all()
    with pytest.raises(SmgpuError) as e:
        G.solve(0)
    assert e.value.code == L.ERR_ARG
    with pytest.raises(ValueError):
        G.matvec(np.zeros((4, G.mdim + 1)))
    # a sample whose matrix elements vanish has another non-zero pattern
    labels, vals = synth.draw_tbmes("sd", 1)
    zero = tmp_path / "zero.snt"
    zero.write_text(synth.snt_text("sd", labels, np.zeros_like(vals), 20))
    with pytest.raises(SmgpuError) as e:
        _multi([files[0], str(zero)], "Ne20")
    assert e.value.code == L.ERR_LIMIT
    with pytest.raises(SmgpuError) as e:
        _multi([files[0], str(tmp_path / "missing.snt")], "Ne20")
    assert e.value.code == L.ERR_IO
    with pytest.raises(SmgpuError) as e:
        _multi([os.path.join(GOLDEN, "ckpot.snt")] * 17, "Be8")
    assert e.value.code == L.ERR_LIMIT
