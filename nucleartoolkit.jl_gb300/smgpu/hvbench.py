"""Time the H·v kernel on a named workload (CUDA events on the library stream).

    python nucleartoolkit.jl_gb300/smgpu/hvbench.py --workload pf4p4n --precision mixed --reps 20
    python nucleartoolkit.jl_gb300/smgpu/hvbench.py --workload pf4p4n --samples 16 --reps 10 --solve
    python nucleartoolkit.jl_gb300/smgpu/hvbench.py --batch 128 --reps 10 --solve

Prints one JSON line: mean ms per launch, multiply-adds per launch and the
CSR-equivalent bandwidth (algorithmic bytes nnz·(s_c+4) + 4·(mdim+1) +
2·mdim·s_v over the launch time; with --samples S the S coefficient sets
share the indices: nnz·(4 + S·4) + 2·S·mdim·4).  --samples S times the
multi-sample H·V on S seeded interaction samples of the workload's basis
(FP32-mixed).  --solve adds one eigensolve (5 lowest, lm=30, ls=15,
tol=1e-8).  --batch N times the batched H·v over the first N problems of
the uneven sd batch (FP32-mixed; the bandwidth figure then needs --nnz of the
whole batch).  Used for kernel profiling.
"""
import argparse
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import smgpu  # noqa: E402
from smgpu import synth  # noqa: E402

VALENCE = {"sd2p2n": ("sd", 2, 2, "Ne20"), "sd4p4n": ("sd", 4, 4, "Mg24"), "pf4p4n": ("pf", 4, 4, "Cr48")}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="pf4p4n", choices=sorted(VALENCE))
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed", "mixed_df"])
    ap.add_argument("--samples", type=int, default=0, help="interaction samples sharing the basis (multi-sample H·V)")
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--no-flush", action="store_true")
    ap.add_argument("--batch", type=int, default=0, help="problems of the uneven sd batch (batched H·v)")
    ap.add_argument("--solve", action="store_true", help="also run one eigensolve")
    ap.add_argument("--nnz", type=int, default=0, help="structural nnz(H) for the bandwidth figure")
    a = ap.parse_args()
    d = tempfile.mkdtemp()
    out = {"workload": a.workload}
    if a.batch:
        P = smgpu.BatchProblem(synth.sd_batch_snts(d, a.batch))
        out.update(workload=f"sd batch of {a.batch}", precision="mixed", problems=a.batch)
    elif a.samples:
        shell, vp, vn, nuc = VALENCE[a.workload]
        if a.workload == "pf4p4n":
            files = synth.pf_multi_snts(d, a.samples)
        else:
            files = synth.multi_snts(d, shell, vp, vn, a.samples, 77000, synth.SHELLS[shell][3], 0.1, "s")
        P = smgpu.MultiSampleProblem(files, nuc)
        out.update(precision="mixed", samples=a.samples)
    else:
        snt, nuc = synth.config_snt(d, a.workload)
        prec = {"mixed": smgpu.MIXED, "mixed_df": smgpu.MIXED_DF, "fp64": smgpu.FP64}[a.precision]
        P = smgpu.ShellModelProblem(snt, nuc, prec)
        out.update(precision=a.precision)
    ms = P.time_matvec(reps=a.reps, flush_l2=not a.no_flush)
    out.update(mdim=int(getattr(P, "total_mdim", 0) or P.mdim), ms=ms)
    out.update(P.stats())
    if hasattr(P, "tune_report"):
        out["tune"] = P.tune_report()
    if a.nnz:
        if a.batch:
            b = a.nnz * 8 + 4 * (P.total_mdim + a.batch) + 2 * P.total_mdim * 4
        elif a.samples:
            b = a.nnz * (4 + a.samples * 4) + 2 * a.samples * P.mdim * 4
        else:
            s = 8 if a.precision == "fp64" else 4
            b = a.nnz * (s + 4) + 4 * (P.mdim + 1) + 2 * P.mdim * s
        out["csr_equiv_GBs"] = b / (ms * 1e-3) / 1e9
    if a.solve:
        r = P.solve(5, lm=30, ls=15, tol=1e-8)
        out.update(solve_s=P.timings()["lanczos"], n_matvec=r["n_matvec"], n_restart=r["n_restart"],
                   converged=bool(r["converged"]), kernel_launches=r["kernel_launches"])
    print(json.dumps(out))


if __name__ == "__main__":
    main()
