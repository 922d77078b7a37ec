"""Full-size oracle runs recorded as golden data (oracle_runs.json).

For each named workload: the M-scheme dimension, the structural nnz(H)
counted by the oracle, and the oracle's FP64 thick-restart Lanczos result
(eigenvalues, iterations, restarts).  The 48Cr pf eigensolve takes minutes on
a CPU, so its result is computed once here and the GPU tests / bench compare
against the stored values.  Re-run after any change of the synthetic recipe:

    python tests/golden/make_oracle_runs.py [names...]

`sd_batch128` records the uneven batch of 128 sd problems (per problem:
dimension, nnz(H), eigenvalues, iteration counts).
"""
import json
import os
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "nucleartoolkit.jl_gb300"))

from oracle.oracle import OracleProblem, get_threads  # noqa: E402
from smgpu import synth  # noqa: E402

# workload -> (num_ev, lm, ls, tol)
RUNS = {
    "sd2p2n": (5, 300, 20, 1e-8),
    "sd4p4n": (10, 300, 20, 1e-8),
    "pf4p4n": (5, 30, 15, 1e-8),
}


BATCH = ("sd_batch128", 128, (5, 30, 15, 1e-8))


def batch_run():
    """The uneven batch of 128 sd problems: per problem its dimension, nnz(H)
    and the oracle's eigenvalues and iteration counts."""
    n, (nev, lm, ls, tol) = BATCH[1], BATCH[2]
    d = tempfile.mkdtemp()
    out = dict(nprob=n, num_ev=nev, lm=lm, ls=ls, tol=tol, threads=get_threads(), problems=[])
    t0 = time.time()
    for k, (snt, nuc) in enumerate(synth.sd_batch_snts(d, n)):
        P = OracleProblem(snt, nuc)
        r = P.trl(nev, lm=lm, ls=ls, tol=tol)
        out["problems"].append(dict(nucleus=nuc, seed=synth.CONFIG_SEEDS["sd_batch_base"] + k, mdim=P.mdim,
                                    nnz=P.nnz(), evals=[float(x) for x in r["evals"]], n_hv=r["n_hv"],
                                    n_restart=r["n_restart"], converged=r["converged"], t_trl=r["t_total"]))
    out["mdim_total"] = sum(p["mdim"] for p in out["problems"])
    out["nnz_total"] = sum(p["nnz"] for p in out["problems"])
    out["t_total"] = time.time() - t0
    return out


def main(names):
    path = os.path.join(HERE, "oracle_runs.json")
    data = json.load(open(path)) if os.path.exists(path) else {}
    d = tempfile.mkdtemp()
    for name in names:
        if name == BATCH[0]:
            data[name] = batch_run()
            print(name, data[name]["mdim_total"], data[name]["nnz_total"], data[name]["t_total"], flush=True)
            json.dump(data, open(path, "w"), indent=1)
            continue
        nev, lm, ls, tol = RUNS[name]
        snt, nuc = synth.config_snt(d, name)
        t0 = time.time()
        P = OracleProblem(snt, nuc)
        t_setup = time.time() - t0
        t0 = time.time()
        nnz = P.nnz()
        t_nnz = time.time() - t0
        r = P.trl(nev, lm=lm, ls=ls, tol=tol)
        data[name] = dict(nucleus=nuc, seed=synth.CONFIG_SEEDS[name], mdim=P.mdim, nblocks=P.nblocks, nnz=nnz,
                          num_ev=nev, lm=lm, ls=ls, tol=tol, evals=[float(x) for x in r["evals"]],
                          n_hv=r["n_hv"], n_restart=r["n_restart"], elit=r["elit"], converged=r["converged"],
                          t_setup=t_setup, t_nnz=t_nnz, t_trl=r["t_total"], t_hv=r["t_hv"], t_reorth=r["t_reorth"],
                          threads=get_threads())
        print(name, json.dumps(data[name]), flush=True)
        json.dump(data, open(path, "w"), indent=1)


if __name__ == "__main__":
    main(sys.argv[1:] or list(RUNS) + [BATCH[0]])
