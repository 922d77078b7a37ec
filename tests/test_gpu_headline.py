"""The headline workload on the GPU: 48Cr, pf shell, 4 protons + 4 neutrons,
M = 0 (dim 1,963,461), 5 lowest eigenvalues, lm = 30, ls = 15, tol = 1e-8.

Eigenvalues and iteration counts of every precision form against the oracle's
FP64 thick-restart Lanczos run of the same seeded interaction (stored in
tests/golden/oracle_runs.json by tests/golden/make_oracle_runs.py: the full
oracle solve takes minutes on a CPU), and the pf jump tables as exact sets
against the oracle's prep_pn / prep_2bjumps (reference:
src/ShellModel/lanczos_methods.jl:1-91 TRL; src/ShellModel/shellmodel_main.jl:
1115-1199 prep_2bjumps, prep_pn).
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

EIG_FP64_RTOL = 1e-8   # FP64 eigenvalues vs the oracle, relative
EIG_MIXED_ATOL = 1e-4  # FP32-mixed eigenvalues vs the FP64 oracle, MeV
COEF_RTOL = 1e-13      # pp/nn jump coefficients, relative to the largest


@pytest.fixture(scope="module")
def ref():
    with open(os.path.join(GOLDEN, "oracle_runs.json")) as f:
        return json.load(f)["pf4p4n"]


@pytest.fixture(scope="module")
def lib():
    from smgpu import _lib
    from smgpu import build as b
    b.build()
    return _lib.load()


def _solve(snt_dir, prec):
    from smgpu import ShellModelProblem
    snt, nuc = snt_dir["pf4p4n"]
    P = ShellModelProblem(snt, nuc, prec)
    r = P.solve(5, lm=30, ls=15, tol=1e-8)
    P.close()
    return r


def test_pf_fp64_eigenvalues_and_counts(lib, snt_dir, ref):
    from smgpu import FP64
    r = _solve(snt_dir, FP64)
    assert r["converged"]
    ev = np.array(ref["evals"])
    assert np.allclose(r["evals"], ev, rtol=EIG_FP64_RTOL, atol=0), (r["evals"], ev)
    # the reference's control flow: same iterations and restarts as the oracle
    assert (r["n_matvec"], r["n_restart"]) == (ref["n_hv"], ref["n_restart"]) == (211, 13)


@pytest.mark.parametrize("form", ["MIXED", "MIXED_DF"])
def test_pf_mixed_eigenvalues_and_counts(lib, snt_dir, ref, form):
    """SMGPU_MIXED (FP64 residual, re-orthogonalisation and restart algebra)
    and SMGPU_MIXED_DF (the same in double-float): |ΔE| <= 1e-4 MeV against
    the FP64 oracle, and the oracle's iteration counts (the FP32 rounding of
    the basis may move convergence by at most one restart cycle)."""
    import smgpu
    r = _solve(snt_dir, getattr(smgpu, form))
    assert r["converged"]
    ev = np.array(ref["evals"])
    assert np.abs(r["evals"] - ev).max() <= EIG_MIXED_ATOL, (r["evals"], ev)
    assert abs(r["n_restart"] - ref["n_restart"]) <= 1, r
    assert abs(r["n_matvec"] - ref["n_hv"]) <= ref["lm"] - ref["ls"], r


def _pn_keys(rows):
    """One int64 key per (bi, bf, op_a, op_c, i, f, phase) row; op masks are
    single m-state bits (bit positions < 32), blocks < 64, SD indices < 2^12."""
    rows = np.asarray(rows, dtype=np.int64)
    ops = rows[:, 2:4]
    assert np.all(ops > 0) and np.all(ops & (ops - 1) == 0), "one-body operator masks are single bits"
    pos = np.log2(ops).astype(np.int64)
    assert rows[:, :2].max() < 64 and rows[:, 4:6].max() < 4096 and pos.max() < 32
    k = rows[:, 0]
    for x, bits in ((rows[:, 1], 6), (pos[:, 0], 5), (pos[:, 1], 5), (rows[:, 4], 12), (rows[:, 5], 12),
                    (rows[:, 6], 1)):
        k = (k << bits) | x
    return k


def _oracle_pn_rows(O, which):
    """The reference's per-V-entry pn jump lists (prep_pn, shellmodel_main.jl:
    1139-1199) as (bi, bf, op_a, op_c, i, f, phase) rows: entry nth of block
    pair (bi, bf) belongs to the nth operator of Vpn[ΔM], ΔM = Mp[bf] - Mp[bi]."""
    bi, bf, nth, i, f, ph = O.jumps_pn(which)
    delMs, idx, abcd, _ = O.vpn()
    starts = np.concatenate([[0], np.cumsum(np.bincount(idx, minlength=len(delMs)))])
    Mp = np.asarray(O.Mp, dtype=np.int64)
    dm = Mp[np.asarray(bf) - 1] - Mp[np.asarray(bi) - 1]
    order = np.argsort(delMs)
    di = order[np.searchsorted(delMs[order], dm)]
    assert np.all(delMs[di] == dm)
    row = abcd[starts[di] + np.asarray(nth) - 1]
    c0, c1 = (0, 2) if which == 0 else (1, 3)
    return np.stack([bi, bf, row[:, c0], row[:, c1], i, f, ph], axis=1)


def test_pf_jump_tables_exact(lib, snt_dir):
    """48Cr pf: the proton and neutron pn jump entries equal the oracle's as
    sets (190,740 distinct proton entries from 8.6 M per-V-entry list items),
    and the pp/nn two-body jumps have the same (block, i, f) set with
    coefficients within 1e-13."""
    from oracle.oracle import OracleProblem
    from smgpu import FP64, ShellModelProblem
    snt, nuc = snt_dir["pf4p4n"]
    O = OracleProblem(snt, nuc)
    G = ShellModelProblem(snt, nuc, FP64)
    for which in (0, 1):
        g = np.unique(_pn_keys(G.jumps(which)))
        o = np.unique(_pn_keys(_oracle_pn_rows(O, which)))
        assert len(o) > 100000
        assert np.array_equal(g, o), f"pn table {which}"
    for which, ow in ((2, 0), (3, 1)):
        ints, coef = G.jumps(which)
        blk, i, f, c = O.jumps_2b(ow)
        ok = (np.asarray(blk, np.int64) << 24) | (np.asarray(i, np.int64) << 12) | np.asarray(f, np.int64)
        uk, inv = np.unique(ok, return_inverse=True)
        osum = np.bincount(inv, weights=np.asarray(c, dtype=np.float64), minlength=len(uk))
        keep = osum != 0.0
        uk, osum = uk[keep], osum[keep]
        gk = (ints[:, 0] << 24) | (ints[:, 1] << 12) | ints[:, 2]
        gkeep = coef != 0.0
        gk, gc = gk[gkeep], coef[gkeep]
        order = np.argsort(gk)
        gk, gc = gk[order], gc[order]
        assert np.array_equal(gk, uk), f"2b table {which}"
        assert np.abs(gc - osum).max() <= COEF_RTOL * np.abs(osum).max(), f"2b coefficients {which}"
