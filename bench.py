"""Benchmark: 48Cr pf-shell M=0 (dim 1,963,461), time to the 5 lowest eigenvalues.

One step = one thick-restart Lanczos eigensolve (lm=30, ls=15, tol=1e-8) of
the seeded synthetic pf interaction, FP32-mixed form, problem resident on the
GPU.  The line also carries the plain FP64 GPU form, the per-eigenvalue error
of both forms against the FP64 oracle, the H·v roofline and the CPU baseline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the CPU restatement of the reference's path (the
oracle: operate_H! + TRL with OpenMP over blocks) on all host cores instead;
each step is a bounded sample (the first restart cycle: lm TRL iterations and
one thick restart) projected to the oracle's full iteration and restart counts
(tests/golden/oracle_runs.json).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "nucleartoolkit.jl_gb300"))

METRIC = "pf M=0 time-to-5-eigvals & H·v HBM GB/s: FP32-mixed vs FP64 GPU, ΔE≤1e-4 MeV"
WORKLOAD = "pf4p4n"
NEV, LM, LS, TOL = 5, 30, 15, 1e-8
HBM_FALLBACK = 6800.0


def load_json(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def golden_run():
    g = load_json(os.path.join(ROOT, "tests", "golden", "oracle_runs.json")) or {}
    return g.get(WORKLOAD)


def config_dict(extra=None):
    c = {"workload": "48Cr pf-shell 4p4n M=0, dim 1963461, 21 (Mp,Mn) blocks, 5 lowest eigenvalues, "
                     "thick-restart Lanczos lm=30 ls=15 tol=1e-8",
         "interaction": "synthetic seeded snt: TBMEs N(0,1.0^2) MeV seed 4848, SPE -8.6/-6.0/-2.0/-4.0",
         "mdim": 1963461, "num_ev": NEV, "lm": LM, "ls": LS, "tol": TOL,
         "l2": "flushed (256 MB write) between timed steps; Krylov basis 236 MB > L2"}
    if extra:
        c.update(extra)
    return c


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,utilization.gpu,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = tempfile.mktemp(suffix=".csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 10:
                    rows.append(parts)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        load = [r for r in rows if (num(r[4]) or 0) >= 20] or rows
        sm = [num(r[1]) for r in load if num(r[1]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[6 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": num(rows[0][2]),
                "reasons": reasons, "samples": len(rows), "samples_under_load": len(load)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ------------------------------------------------------------------ CPU arm
SAMPLE_HV = LM  # the first restart cycle (lm-1 iterations), one thick restart, one more iteration


def oracle_setup(snt, nuc):
    from oracle.oracle import OracleProblem
    t0 = time.perf_counter()
    O = OracleProblem(snt, nuc)
    return O, time.perf_counter() - t0


def oracle_sample(O, max_hv=SAMPLE_HV):
    """Time the oracle's TRL (operate_H! + α + MGS re-orthogonalisation + β,
    thick restart) on the full problem for its first `max_hv` iterations."""
    from oracle.oracle import get_threads
    r = O.trl_sample(NEV, LM, LS, TOL, max_hv)
    t_iter = (r["t_total"] - r["t_restart"]) / max(r["n_hv"], 1)
    t_rs = r["t_restart"] / max(r["n_restart"], 1) if r["n_restart"] else 0.0
    return dict(t_iter=t_iter, t_restart=t_rs, t_hv=r["t_hv"] / max(r["n_hv"], 1), n=r["n_hv"],
                n_restart=r["n_restart"], threads=get_threads(), t_total=r["t_total"])


def project(t_setup, s, g):
    """Full-solve time from the sample: set-up + n_hv iterations + n_restart
    restarts, with the oracle's own counts for this workload."""
    if not g:
        return None
    return t_setup + g["n_hv"] * s["t_iter"] + g["n_restart"] * s["t_restart"]


def sample_text(t_setup, s, g):
    return (f"oracle (C++ restatement of operate_H!/TRL, OpenMP over blocks, {s['threads']} threads) on the full "
            f"48Cr problem: set-up {t_setup:.2f} s + the first {s['n']} TRL iterations incl. {s['n_restart']} thick "
            f"restart ({s['t_iter']:.3f} s/iteration, H·v {s['t_hv']:.3f} s, restart {s['t_restart']:.2f} s), "
            f"projected to the oracle's full run: n_hv={g['n_hv']}, n_restart={g['n_restart']}")


def run_reference(args, dist, rank):
    if rank != 0:
        return
    from smgpu import synth
    d = tempfile.mkdtemp()
    snt, nuc = synth.config_snt(d, WORKLOAD)
    g = golden_run()
    if not g:
        print(json.dumps({"impl": "reference", "unavailable": "oracle iteration count for the projection is missing "
                                                              "(tests/golden/oracle_runs.json)"}))
        return
    O, t_setup = oracle_setup(snt, nuc)
    for _ in range(args.warmup):  # warm-up: two iterations each (untimed)
        oracle_sample(O, max_hv=2)
    vals = []
    s = None
    t_wall0 = time.perf_counter()
    for _ in range(args.steps):
        s = oracle_sample(O)
        vals.append(project(t_setup, s, g))
    wall = time.perf_counter() - t_wall0
    v = statistics.mean(vals)
    threads = s["threads"]
    sample = "per step: " + sample_text(t_setup, s, g)
    line = {"metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict({"impl": "CPU restatement (oracle) of operate_H!/TRL, OpenMP over blocks"}),
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ------------------------------------------------------------------ multi-sample leg
MULTI_WORKLOAD = ("48Cr pf-shell 4p4n M=0 basis (dim 1963461) shared by 16 interaction samples "
                  "(base TBMEs N(0,1.0^2) seed 48000, per-sample N(0,0.1^2) seeds 48001..48016), 5 lowest "
                  "eigenvalues each, lm=30 ls=15 tol=1e-8: one 16-sample FP32-mixed solve vs 16 FP64 solves")


def multi_leg(flush, g):
    """16 samples on the 48Cr basis: one multi-sample FP32-mixed solve against
    16 independent plain FP64 solves of the same samples (device-resident,
    set-up excluded on both sides), per-sample |ΔE| against the FP64 solves,
    and the multi-sample H·V roofline."""
    import numpy as np
    import smgpu
    from smgpu import synth

    d = tempfile.mkdtemp()
    files = synth.pf_multi_snts(d)
    t0 = time.perf_counter()
    G = smgpu.MultiSampleProblem(files, "Cr48")
    t_create = time.perf_counter() - t0
    G.solve(NEV, lm=LM, ls=LS, tol=TOL)
    flush()
    r = G.solve(NEV, lm=LM, ls=LS, tol=TOL)
    t_multi = G.timings()["lanczos"]
    hv_ms = G.time_matvec(reps=10, flush_l2=True)
    st = G.stats()
    G.close()
    t_loop, t_loop_create, dE = 0.0, 0.0, []
    for s, f in enumerate(files):
        t0 = time.perf_counter()
        F = smgpu.ShellModelProblem(f, "Cr48", smgpu.FP64)
        t_loop_create += time.perf_counter() - t0
        flush()
        rf = F.solve(NEV, lm=LM, ls=LS, tol=TOL)
        t_loop += F.timings()["lanczos"]
        dE.append(float(np.abs(r["evals"][s] - rf["evals"]).max()))
        F.close()
    mdim = 1963461
    out = {"workload": MULTI_WORKLOAD, "value": t_multi, "unit": "s", "fp64_loop_s": t_loop,
           "speedup_vs_fp64_loop": t_loop / t_multi, "max_abs_dE_vs_fp64_MeV": max(dE), "dE_per_sample_MeV": dE,
           "n_matvec": r["n_matvec"], "n_restart": r["n_restart"], "converged": r["converged"],
           "kernel_launches": r["kernel_launches"], "create_s": t_create, "fp64_loop_create_s": t_loop_create,
           "hv_ms": hv_ms, "hv_launch_shape": [st["hv_threads"], st["hv_min_ctas"], st["hv_entry_cache"]],
           "sample_matvecs_per_s": 16 * r["n_matvec"] / t_multi}
    if g:
        b_alg = g["nnz"] * (4 + 16 * 4) + 2 * 16 * mdim * 4
        out["hv_algorithmic_bytes"] = b_alg
        out["hv_achieved_GBs"] = b_alg / (hv_ms * 1e-3) / 1e9
    return out


# ------------------------------------------------------------------ batch leg
BATCH_WORKLOAD = ("uneven batch of 128 sd-shell problems (vp, vn cycling through 1..6, M = A mod 2, dims 28..93710, "
                  "total 2235778), each with its own seeded TBMEs N(0,1.5^2) (seeds 128000..128127), 5 lowest "
                  "eigenvalues each, lm=30 ls=15 tol=1e-8: one batched FP32-mixed solve vs a loop of 128 FP64 solves")


def batch_leg(flush):
    """128 independent sd problems: one batched FP32-mixed solve against a
    loop of single plain FP64 solves (device-resident, set-up excluded on
    both sides), per-problem |ΔE| against the loop and against the stored
    oracle eigenvalues, and the batched H·v roofline."""
    import numpy as np
    import smgpu
    from smgpu import synth

    gb = (load_json(os.path.join(ROOT, "tests", "golden", "oracle_runs.json")) or {}).get("sd_batch128")
    d = tempfile.mkdtemp()
    probs = synth.sd_batch_snts(d, 128)
    t0 = time.perf_counter()
    G = smgpu.BatchProblem(probs)
    t_create = time.perf_counter() - t0
    G.solve(NEV, lm=LM, ls=LS, tol=TOL)
    flush()
    r = G.solve(NEV, lm=LM, ls=LS, tol=TOL)
    t_batch = G.timings()["lanczos"]
    hv_ms = G.time_matvec(reps=10, flush_l2=True)
    st = G.stats()
    mdims = [int(x) for x in G.mdims]
    G.close()
    t_loop, t_loop_create, dE, dE_oracle = 0.0, 0.0, [], []
    for p, (snt, nuc) in enumerate(probs):
        t0 = time.perf_counter()
        F = smgpu.ShellModelProblem(snt, nuc, smgpu.FP64)
        t_loop_create += time.perf_counter() - t0
        rf = F.solve(NEV, lm=LM, ls=LS, tol=TOL)
        t_loop += F.timings()["lanczos"]
        nev = len(rf["evals"])
        dE.append(float(np.abs(r["evals"][p, :nev] - rf["evals"]).max()))
        if gb:
            ref = np.array(gb["problems"][p]["evals"])
            dE_oracle.append(float(np.abs(r["evals"][p, :len(ref)] - ref).max()))
        F.close()
    out = {"workload": BATCH_WORKLOAD, "value": t_batch, "unit": "s", "fp64_loop_s": t_loop,
           "speedup_vs_fp64_loop": t_loop / t_batch, "max_abs_dE_vs_fp64_MeV": max(dE),
           "max_abs_dE_vs_oracle_MeV": max(dE_oracle) if dE_oracle else None,
           "n_matvec": r["n_matvec"], "n_restart": r["n_restart"], "converged": r["converged"],
           "kernel_launches": r["kernel_launches"], "create_s": t_create, "fp64_loop_create_s": t_loop_create,
           "hv_ms": hv_ms, "hv_launch_shape": [st["hv_threads"], st["hv_rows"], st["hv_min_ctas"]],
           "mdim_total": sum(mdims), "problem_matvecs_per_s": 128 * r["n_matvec"] / t_batch}
    if gb:
        b_alg = sum(q["nnz"] * (4 + 4) + 4 * (q["mdim"] + 1) + 2 * q["mdim"] * 4 for q in gb["problems"])
        out["hv_algorithmic_bytes"] = b_alg
        out["hv_achieved_GBs"] = b_alg / (hv_ms * 1e-3) / 1e9
    return out


# ------------------------------------------------------------------ GPU arm
def run_gpu(args, dist, rank, local):
    import numpy as np
    import torch
    import smgpu
    from smgpu import synth

    torch.cuda.set_device(0)
    flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def flush():
        flush_buf.fill_(1)
        torch.cuda.synchronize()

    d = tempfile.mkdtemp()
    snt, nuc = synth.config_snt(d, WORKLOAD)
    g = golden_run()

    # ---- device-resident solves (value)
    M = smgpu.ShellModelProblem(snt, nuc, smgpu.MIXED)
    st = M.stats()
    for _ in range(args.warmup):
        M.solve(NEV, lm=LM, ls=LS, tol=TOL)
    times, launches, res = [], 0, None
    barrier(dist)
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush()
            res = M.solve(NEV, lm=LM, ls=LS, tol=TOL)
            times.append(M.timings()["lanczos"])
            launches += res["kernel_launches"]
    barrier(dist)
    t_mixed = max_over_ranks(dist, statistics.mean(times))
    clocks = clk.summary()
    ev_mixed = res["evals"]

    # ---- H·v kernel timing (CUDA events on the library stream)
    hv_ms_mixed = M.time_matvec(reps=20, flush_l2=True)
    M.close()

    # ---- plain FP64 form
    F = smgpu.ShellModelProblem(snt, nuc, smgpu.FP64)
    F.solve(NEV, lm=LM, ls=LS, tol=TOL)
    t64 = []
    for _ in range(max(1, min(args.steps, 2))):
        flush()
        rf = F.solve(NEV, lm=LM, ls=LS, tol=TOL)
        t64.append(F.timings()["lanczos"])
    t_fp64 = statistics.mean(t64)
    ev_fp64 = rf["evals"]
    hv_ms_fp64 = F.time_matvec(reps=10, flush_l2=True)
    F.close()

    # ---- end to end through the C ABI: snt file -> set-up -> solve -> eigenvalues
    e2e_times = []
    h2d = d2h = 0
    for _ in range(max(1, min(args.steps, 3))):
        flush()
        t0 = time.perf_counter()
        E = smgpu.ShellModelProblem(snt, nuc, smgpu.MIXED)
        re = E.solve(NEV, lm=LM, ls=LS, tol=TOL)
        e2e_times.append(time.perf_counter() - t0)
        h2d = E.stats()["table_bytes"]
        d2h = 8 * NEV + 32 * (re["n_restart"] + 1)
        E.close()
    t_e2e = max_over_ranks(dist, statistics.mean(e2e_times))

    # ---- roofline of the H·v kernel (FP32-mixed): CSR-equivalent algorithmic bytes
    mdim = 1963461
    nnz = g["nnz"] if g else None
    peaks = load_json(os.path.join(ROOT, "MEASURED_PEAKS.json"))
    peak = (peaks or {}).get("hbm_gbs") or HBM_FALLBACK
    peak_src = "measured" if peaks and peaks.get("hbm_gbs") else "fallback"
    prof = load_json(os.path.join(ROOT, "profiles", "hv_pf4p4n_traffic.json")) or {}
    staged = bool(st.get("hv_staged"))
    kname = "hv_staged_kernel" if staged else "hv_tile_kernel"
    roof = None
    if nnz:
        b_alg = nnz * (4 + 4) + 4 * (mdim + 1) + 2 * 1 * mdim * 4
        achieved = b_alg / (hv_ms_mixed * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": (prof.get(kname) or {}).get("mixed_bytes_per_launch"),
                "kernel": f"{kname} (FP32-mixed H·v, launch shape {st['hv_threads']}x{st['hv_rows']}"
                          f" min {st['hv_min_ctas']} CTAs/SM)",
                "peak_source": peak_src, "algorithmic_bytes": b_alg,
                "hv_ms": hv_ms_mixed, "hv_fp64_ms": hv_ms_fp64,
                "hv_fp64_achieved": (nnz * (8 + 4) + 4 * (mdim + 1) + 2 * mdim * 8) / (hv_ms_fp64 * 1e-3) / 1e9}

    # ---- CPU baseline (rank 0, N=1 only)
    cpu = None
    if rank == 0 and args.gpus == 1 and not args.no_cpu:
        O, t_setup = oracle_setup(snt, nuc)
        s = oracle_sample(O)
        cpu = {"value": project(t_setup, s, g), "unit": "s", "cores": s["threads"], "kind": "port",
               "sample": sample_text(t_setup, s, g) if g else "golden oracle run missing"}
        del O

    peak_m = (load_json(os.path.join(ROOT, "MEASURED_PEAKS.json")) or {}).get("hbm_gbs") or HBM_FALLBACK
    multi = None
    if not args.no_multi:
        multi = multi_leg(flush, g)
        if "hv_achieved_GBs" in multi:
            multi["hv_frac_of_hbm_peak"] = multi["hv_achieved_GBs"] / peak_m
    batch = None
    if not args.no_batch:
        batch = batch_leg(flush)
        if "hv_achieved_GBs" in batch:
            batch["hv_frac_of_hbm_peak"] = batch["hv_achieved_GBs"] / peak_m

    dE = None
    if g:
        ref = np.array(g["evals"])
        dE = {"mixed_vs_oracle_MeV": [float(x) for x in (ev_mixed - ref)],
              "fp64_vs_oracle_MeV": [float(x) for x in (ev_fp64 - ref)],
              "max_abs_mixed_MeV": float(np.abs(ev_mixed - ref).max()),
              "max_rel_fp64": float(np.abs((ev_fp64 - ref) / ref).max())}
    if rank == 0:
        line = {"metric": METRIC, "value": t_mixed, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_mixed * 1e3, "higher_is_better": False, "scaling": "weak",
                "vs_baseline": None, "dtype": "fp32-mixed (f32 H·v, f64 Lanczos)", "data": "synthetic",
                "config": config_dict({"parallelism": f"replicas x{args.gpus}"}),
                "e2e": {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                        "path": "smgpu_problem_create_from_snt + smgpu_solve (snt file to eigenvalues)"},
                "roofline": roof, "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": int(launches),
                "fp64_plain": {"value": t_fp64, "unit": "s", "evals": [float(x) for x in ev_fp64]},
                "speedup_mixed_vs_fp64": t_fp64 / t_mixed,
                "evals_mixed": [float(x) for x in ev_mixed], "dE": dE,
                "lanczos": {"n_matvec": res["n_matvec"], "n_restart": res["n_restart"],
                            "second_pass": res["n_second_pass"]},
                "matvecs_per_s": res["n_matvec"] / t_mixed, "hv_updates": st["updates"],
                "multi_sample": multi, "batch": batch}
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-multi", action="store_true", help="skip the 16-sample leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the 128-problem batch leg")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dist = init_dist(world)
    if args.impl == "reference":
        run_reference(args, dist, rank)
    else:
        run_gpu(args, dist, rank, local)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
