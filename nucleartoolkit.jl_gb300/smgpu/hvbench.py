"""Time the H·v kernel on a named workload (CUDA events on the library stream).

    python nucleartoolkit.jl_gb300/smgpu/hvbench.py --workload pf4p4n --precision mixed --reps 20

Prints one JSON line: mean ms per launch, multiply-adds per launch and the
CSR-equivalent bandwidth (algorithmic bytes nnz·(s_c+4) + 4·(mdim+1) +
2·mdim·s_v over the launch time).  Used for kernel profiling.
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="pf4p4n", choices=["sd2p2n", "sd4p4n", "pf4p4n"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--no-flush", action="store_true")
    ap.add_argument("--nnz", type=int, default=0, help="structural nnz(H) for the bandwidth figure")
    a = ap.parse_args()
    d = tempfile.mkdtemp()
    snt, nuc = synth.config_snt(d, a.workload)
    prec = smgpu.MIXED if a.precision == "mixed" else smgpu.FP64
    P = smgpu.ShellModelProblem(snt, nuc, prec)
    ms = P.time_matvec(reps=a.reps, flush_l2=not a.no_flush)
    st = P.stats()
    out = {"workload": a.workload, "precision": a.precision, "mdim": P.mdim, "ms": ms, "updates": st["updates"],
           "table_bytes": st["table_bytes"], "links": st["links"], "hv_threads": st["hv_threads"],
           "hv_rows": st["hv_rows"], "hv_min_ctas": st["hv_min_ctas"]}
    if a.nnz:
        s = 4 if prec == smgpu.MIXED else 8
        b = a.nnz * (s + 4) + 4 * (P.mdim + 1) + 2 * P.mdim * s
        out["csr_equiv_GBs"] = b / (ms * 1e-3) / 1e9
    print(json.dumps(out))


if __name__ == "__main__":
    main()
