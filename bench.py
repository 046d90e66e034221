#!/usr/bin/env python3
"""Benchmark of the steady LU-SGS iteration of RocketCombustor on GB300.

One step = one lu_sgs_stage (TimeStep, reconstruction, flux_sourceterm,
LU_SGS_steady with the Newton update) over the whole mesh, launched as one
captured CUDA graph.  Default workload: the large single case of the
roofline configuration, the reacting viscous nozzle at 2,000,000 triangles
(4 species, T-dependent cp, global H2/O2 reaction), plain FP64, with the mixed
form timed beside it.

  value   cell-iters/s = NE * K / (sum of device-timed steps), state resident in
          HBM, L2 flushed (256 MB write) between timed steps;
  e2e     the same metric through the C ABI with the state in pinned host
          memory: each step copies PA, WA host->device, runs the stage, reads the
          residual norms and copies PA, WA device->host;
  roofline  the dominant subroutine timed live with CUDA events, and per
          subroutine its fraction of the measured HBM bandwidth and of the
          FP64 rate measured on this GPU by rc_fp64_rate;
  cpu_baseline  the FP64 CPU oracle on all host threads, bounded sample.

--impl reference times the CPU restatement of the reference (the oracle) on
the host cores on the same workload; the Fortran reference itself cannot be
built (no Fortran compiler, MPI or LAPACK).
Multi-GPU: replicas only (each rank runs its own copy of the case).
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

# Algorithmic bytes per cell-iteration of each reference subroutine, FP64,
# triangles (NF/NE ~ 1.5), V = NVar: the per-kernel table of the design notes.
def algo_bytes_per_cell(V: int, nf_ne: float, viscous: bool, combustion: bool) -> dict:
    b = {
        "timestep": 8 * V + 16 + nf_ne * 32,
        "reconstruction": (24 * V + 84) + (40 * V + 56 + nf_ne * 16),
        "flux_sourceterm": (32 * V + 32 + nf_ne * 40) + ((40 * V + 32 + nf_ne * 40) if viscous else 0)
        + ((24 * V + 8) if combustion else 0),
        "lu_sgs_steady": 2 * (24 * V + 28 + nf_ne * 32) + (32 * V + 8),
    }
    b["stage"] = sum(b.values())
    return b


# DRAM bytes and FP64-pipe warp instructions per cell of each subroutine's
# kernels in one FP64 iteration of the reacting viscous nozzle at 500,000 cells
# (a working set above the 129 MB L2; ncu dram__bytes_read.sum +
# dram__bytes_write.sum and sm__inst_executed_pipe_fp64.sum over the
# subroutine's launches, divided by the cells: profiles/c4_500k_fp64_counters.md).
# Both grow with the cells.
NCU_DRAM_PER_CELL = {"timestep": 199.5, "reconstruction": 339.2, "flux_sourceterm": 685.7,
                     "lu_sgs_steady": 640.3}
NCU_FP64_INST_PER_CELL = {"timestep": 46.72, "reconstruction": 46.00, "flux_sourceterm": 128.92,
                          "lu_sgs_steady": 76.62}
NCU_TRAFFIC_SOURCE = ("ncu capture of one FP64 iteration of the same physics at 500,000 cells (compact dataflow "
                      "LU-SGS; profiles/c4_500k_fp64_counters.md), scaled by cells")


def read_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def fp64_rate(rc, stream, torch, iters: int = 4000, repeats: int = 3) -> dict:
    """The FP64 rate of this GPU (rc_fp64_rate: DADD/DMUL chains on every SM),
    best of `repeats` CUDA-event-timed launches, SM clock sampled meanwhile."""
    import ctypes
    L = rc.load()
    best, secs = 0.0, []
    with ClockSampler(gpu_id(torch)) as clk:
        for _ in range(repeats):
            ops, sec = ctypes.c_double(0.0), ctypes.c_double(0.0)
            st = L.rc_fp64_rate(ctypes.c_void_p(stream.cuda_stream), iters, ctypes.byref(ops), ctypes.byref(sec))
            if st != 0:
                raise RuntimeError(f"rc_fp64_rate failed with status {st}")
            best = max(best, ops.value)
            secs.append(sec.value)
    return {"ops_per_s": best, "warp_inst_per_s": best / 32.0, "unit": "FP64 ops/s (DADD, DMUL)",
            "seconds_per_launch": secs, "clocks": clk.summary(),
            "source": "measured here: rc_fp64_rate, 8 blocks x 256 threads per SM, 8 independent DADD/DMUL "
                      "chains per thread, best of 3 launches (CUDA events)"}


def roofline(dom, sub_ms, ab, NE, peak, peak_kind, fp64) -> dict:
    """The dominant subroutine against the HBM roofline, and every subroutine
    against both the HBM bandwidth and the measured FP64 rate, with the one
    that binds."""
    per = {}
    for name, ms in sub_ms.items():
        t = ms * 1e-3
        hbm = ab[name] * NE / t / 1e9
        e = {"ms": ms, "algorithmic_bytes_per_cell": ab[name], "hbm_gbs": hbm, "hbm_frac": hbm / peak}
        c = NCU_FP64_INST_PER_CELL.get(name)
        if c is not None and fp64:
            rate = c * NE / t
            e.update({"fp64_warp_inst_per_cell": c, "fp64_warp_inst_per_s": rate,
                      "fp64_frac": rate / fp64["warp_inst_per_s"]})
        if name == "lu_sgs_steady":
            e["binds"] = "latency: the dependent chain of one pass per level, level after level"
        elif e.get("fp64_frac", 0.0) > e["hbm_frac"]:
            e["binds"] = "fp64"
        else:
            e["binds"] = "hbm"
        per[name] = e
    d = per[dom]
    return {"bound": "hbm", "kernel": dom, "achieved": d["hbm_gbs"], "peak": peak, "unit": "GB/s",
            "frac": d["hbm_frac"], "peak_source": peak_kind, "algorithmic_bytes_per_cell": ab[dom],
            "traffic": NCU_DRAM_PER_CELL[dom] * NE if dom in NCU_DRAM_PER_CELL else None,
            "traffic_source": NCU_TRAFFIC_SOURCE,
            "binds": d["binds"], "fp64_frac": d.get("fp64_frac"),
            "fp64_peak": fp64, "per_subroutine": per,
            "note": "the face and cell kernels are bound by the FP64 pipe (fp64_frac of the FP64 rate measured "
                    "here), not by HBM; LU-SGS is latency bound (a pass of a few cells per level, level after "
                    "level along the reference cell order)"}


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.out = None

    def __enter__(self):
        if shutil.which("nvidia-smi"):
            self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.out:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.out.flush()
        rows = []
        with open(self.out.name) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 9:
                    rows.append(p)
        os.unlink(self.out.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def case_overrides(args) -> dict:
    over = {}
    for k in ("order", "nx", "ny"):
        if getattr(args, k) is not None:
            over[k] = getattr(args, k)
    return over


def make_workload(name: str, tmp: str, **over):
    from rocketcombustor_gb300 import cases
    d = os.path.join(tmp, name)
    cfg = cases.make_case(d, name, **over)
    return d, cfg


def cpu_baseline(case_dir: str, budget_s: float = 15.0, threads: int = 0):
    """Oracle on the host cores, parallel mode, as many whole iterations as fit
    in about `budget_s` seconds (at least 2)."""
    import oracle
    threads = threads or oracle.Oracle.max_threads()
    o = oracle.Oracle(case_dir, threads=threads)
    t0 = time.perf_counter()
    o.run(1)
    one = time.perf_counter() - t0
    n = max(2, int(budget_s / max(one, 1e-6)))
    t0 = time.perf_counter()
    o.run(n)
    dt = time.perf_counter() - t0
    ne = o.NE
    o.close()
    return {"value": ne * n / dt, "unit": "cell-iters/s", "cores": threads, "kind": "port",
            "sample": f"{n} whole LU-SGS iterations of the same case after 1 warm-up iteration ({dt:.1f} s)"}


def run_reference(args, rank, world):
    import oracle
    if rank != 0:
        return 0
    with tempfile.TemporaryDirectory() as tmp:
        d, cfg = make_workload(args.case, tmp, **case_overrides(args))
        threads = oracle.Oracle.max_threads()
        o = oracle.Oracle(d, threads=threads)
        o.run(args.warmup)
        t0 = time.perf_counter()
        o.run(args.steps)
        dt = time.perf_counter() - t0
        v = o.NE * args.steps / dt
        line = {"impl": "reference", "metric": "cell-iters/s", "value": v, "unit": "cell-iters/s",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": workload_config(cfg, o.NE, o.NF, par_label(world)),
                "cpu_baseline": {"value": v, "unit": "cell-iters/s", "cores": threads, "kind": "port",
                                 "sample": f"{args.steps} whole iterations after {args.warmup} warm-up"},
                "e2e": {"value": v, "unit": "cell-iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
    return 0


def par_label(world: int) -> str:
    """The `parallelism` entry, the same for both arms: one case per process."""
    return "single" if world == 1 else f"replicas x{world}"


def workload_config(cfg, ne, nf, par):
    return {"workload": f"{cfg.name}: steady LU-SGS, nozzle {ne} triangles / {nf} faces, "
                        f"{cfg.nsp} species, {'viscous' if cfg.viscous else 'inviscid'}, "
                        f"{'reacting' if cfg.combustion else 'frozen'}, cell order {cfg.order}",
            "cells": ne, "faces": nf, "species": cfg.nsp, "viscous": cfg.viscous, "combustion": cfg.combustion,
            "cfl": cfg.cfl, "cell_order": cfg.order, "l2": "flushed between timed steps (256 MB write)",
            "parallelism": par}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--case", default="c4")
    ap.add_argument("--order", default=None)
    ap.add_argument("--nx", type=int, default=None, help="override the preset's cells along the axis")
    ap.add_argument("--ny", type=int, default=None, help="override the preset's cells across")
    ap.add_argument("--precision", default="both", choices=["fp64", "mixed", "both"],
                    help="both: FP64 headline plus the mixed form with its error against FP64")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--chem", default="explicit", choices=["explicit", "integrated"],
                    help="chemical source: the reference's explicit rate or the per-cell integrator")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the batched form (64 uneven reacting cases in one context)")
    ap.add_argument("--batch-cases", type=int, default=None,
                    help="cases of the batched form (64 for the throughput line, 16 for --converge)")
    ap.add_argument("--no-surrogate", action="store_true",
                    help="skip the surrogate form (network trained here on integrator pairs)")
    ap.add_argument("--sur-samples", type=int, default=None,
                    help="integrator pairs for the surrogate (10M for the throughput line, 2M for --converge)")
    ap.add_argument("--sur-steps", type=int, default=None,
                    help="training steps of the surrogate (8000 for the throughput line, 4000 for --converge)")
    ap.add_argument("--no-bdf2", action="store_true",
                    help="skip the unsteady form (dual-time BDF2, the reference's shipped time scheme)")
    ap.add_argument("--bdf2-steps", type=int, default=10)
    ap.add_argument("--converge", action="store_true",
                    help="instead of the throughput line: wall time to the steady state (--tol) of the plain FP64 "
                         "path and each form on a steady-state preset (default s2), errors against the FP64 "
                         "converged state, and the oracle to the same criterion")
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--max-iters", type=int, default=40000)
    ap.add_argument("--every", type=int, default=10)
    ap.add_argument("--mlp-infer", type=int, default=0,
                    help="instead of the throughput line: the surrogate network's inference kernel alone on this "
                         "many synthetic samples (10 timed calls), with its error against the FP64 reference")
    ap.add_argument("--mlp-train", type=int, default=0,
                    help="instead of the throughput line: this many Adam steps of the surrogate network "
                         "(rc_mlp_train, batches of 8,192 from 1,048,576 synthetic pairs), wall clock")
    ap.add_argument("--dc-window", type=int, default=20,
                    help="norm reads without a 1%% improvement before the mixed form switches to defect correction")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    for k, thr, conv in (("batch_cases", 64, 16), ("sur_samples", 10_000_000, 2_000_000), ("sur_steps", 8000, 4000)):
        if getattr(args, k) is None:
            setattr(args, k, conv if args.converge else thr)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        rc_ = run_reference(args, rank, world)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return rc_

    import torch
    import rocketcombustor_gb300 as rc

    if args.converge:
        return converge(args, rc, torch)
    if args.mlp_infer:
        return mlp_infer(args, torch)
    if args.mlp_train:
        return mlp_train(args, torch)
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream(device=local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    forms_req = ["fp64", "mixed"] if args.precision == "both" else [args.precision]
    fp64 = fp64_rate(rc, stream, torch)
    with tempfile.TemporaryDirectory() as tmp:
        d, cfg = make_workload(args.case, tmp, **case_overrides(args))
        case = rc.Case(d)
        NE, NF, V = case.NE, case.NF, case.NVar
        results = {}
        states = {}
        clk = None
        for form in forms_req:
            prec = rc.RC_PREC_MIXED if form == "mixed" else rc.RC_PREC_FP64
            s = rc.Solver(case, precision=prec, device=local, stream=stream.cuda_stream)
            if args.chem == "integrated":
                s.set_chemistry(rc.RC_CHEM_INTEGRATED)
            tune = s.autotune(3) if not os.environ.get("RC_LUSGS_SCHEDULE") else "fixed by RC_LUSGS_SCHEDULE"
            r, clk_f = time_form(s, args, stream, flush, dist, torch, rc)
            r["autotune"] = tune
            if clk is None:
                clk = clk_f
            states[form] = s.get_state()
            r.update(subroutine_times(s, args, stream, flush, torch))
            r["e2e"] = e2e_through_abi(s, args, NE, V, torch)
            r["levels"] = {k: v for k, v in s.stats().items() if k != "kernel_launches"}
            if args.chem == "integrated":
                ns = s.chem_substeps()
                r["chem_substeps"] = {"min": int(ns.min()), "mean": float(ns.mean()), "max": int(ns.max())}
            s.close()
            results[form] = r
        head = results[forms_req[0]]
        t_max = max_over_ranks(head["t_local"], dist)
        if rank != 0:
            dist.barrier()
            dist.destroy_process_group()
            return 0
        value = job_throughput(world, NE, args.steps, t_max)
        peak, peak_kind = read_peaks()
        ab = algo_bytes_per_cell(V, NF / NE, cfg.viscous, cfg.combustion)
        sub_ms = head["subroutine_ms"]
        dom = max(sub_ms, key=sub_ms.get)
        line = {
            "metric": "cell-iters/s", "value": value, "unit": "cell-iters/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if forms_req[0] == "fp64" else "f32+f64", "data": "synthetic",
            "config": workload_config(cfg, NE, NF, par_label(world)),
            "e2e": head["e2e"],
            "gpu_launches": head["launches"],
            "roofline": roofline(dom, sub_ms, ab, NE, peak, peak_kind, fp64),
            "subroutine_ms": sub_ms,
            "stage_algorithmic_gbs": ab["stage"] * NE / (t_max / args.steps) / 1e9,
            "levels": head["levels"],
            "autotune": head.get("autotune"),
        }
        if args.chem == "integrated":
            line["config"]["chemistry"] = "integrated (per-cell linearly implicit substeps, tol 0.05)"
            line["chem_substeps"] = head.get("chem_substeps")
        if len(forms_req) > 1:
            ref = states["fp64"][0]
            forms = {}
            for form in forms_req:
                r = results[form]
                f = {"value": NE * args.steps / r["t_local"], "ms_per_step": 1e3 * r["t_local"] / args.steps,
                     "e2e": r["e2e"]["value"], "gpu_launches": r["launches"], "autotune": r.get("autotune"),
                     "subroutine_ms": r["subroutine_ms"]}
                if form != "fp64":
                    st = states[form][0]
                    den = np.maximum(np.abs(ref).max(axis=0), 1e-300)
                    e = np.abs(st - ref).max(axis=0) / den
                    f["rel_linf_vs_fp64"] = {"p": float(e[0]), "T": float(e[3]),
                                             "Y": [float(x) for x in e[4:]],
                                             "after_iterations": args.warmup + args.steps}
                forms[form] = f
            line["forms"] = forms
        bat = None
        if not args.no_batch and world == 1:
            bat = batched_form(args, stream, flush, torch, rc, tmp)
            line.setdefault("forms", {})["batched"] = bat[0]
        if not args.no_surrogate and world == 1 and cfg.combustion and cfg.nsp == 4:
            # trained and compared on the 120k-cell reacting nozzle (and the
            # batched cases' states): the trajectories the surrogate is made for
            if cfg.name == "c2":
                case_s = case
            else:
                d_s, _ = make_workload("c2", tmp)
                case_s = rc.Case(d_s)
            extra = torch.tensor(bat[2].T.copy(), device="cuda") if bat else None
            sur, net = surrogate_form(args, stream, flush, torch, rc, case_s, extra)
            sur["workload"] = f"c2: {case_s.NE} triangles, reacting viscous"
            line.setdefault("forms", {})["surrogate"] = sur
            if bat:
                bat[0]["surrogate"] = batched_surrogate(args, stream, flush, torch, rc, bat[1], bat[2], net)
            net.close()
        if not args.no_bdf2 and world == 1:
            line.setdefault("forms", {})["bdf2"] = bdf2_form(args, stream, torch, rc, tmp)
        line["clocks"] = clk
        if not args.no_cpu:
            line["cpu_baseline"] = cpu_baseline(d, args.cpu_budget)
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def gpu_id(torch):
    """nvidia-smi --id for the current device (its UUID when torch exposes it)."""
    dev = torch.cuda.current_device()
    try:
        u = str(torch.cuda.get_device_properties(dev).uuid)
        return u if u.startswith("GPU-") else "GPU-" + u
    except Exception:
        return str(dev)


def rank_barrier(dist):
    """All ranks meet here (no-op on one rank)."""
    if dist:
        dist.barrier()


def max_over_ranks(t_local: float, dist) -> float:
    """The slowest rank's timed region, on every rank (gloo all-reduce MAX)."""
    if not dist:
        return t_local
    import torch
    tt = torch.tensor([t_local], dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt[0])


def job_throughput(world: int, units_per_rank: int, steps: int, t_max: float) -> float:
    """Whole-job units per second: every rank processed units_per_rank per step."""
    return world * units_per_rank * steps / t_max


def time_form(s, args, stream, flush, dist, torch, rc):
    """W warm-up iterations, then K device-timed iterations (L2 flushed between)."""
    with torch.cuda.stream(stream):
        for it in range(args.warmup):
            s.lu_sgs_stage(it + 1)
        s.sync()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        torch.cuda.synchronize()
        rank_barrier(dist)
        l0 = s.stats()["kernel_launches"]
        with ClockSampler(gpu_id(torch)) as clk:
            for it in range(args.steps):
                flush.zero_()
                ev[it][0].record(stream)
                s.lu_sgs_stage(args.warmup + it + 1)
                ev[it][1].record(stream)
            s.sync()
            torch.cuda.synchronize()
        rank_barrier(dist)
        launches = s.stats()["kernel_launches"] - l0
        ms = [a.elapsed_time(b) for a, b in ev]
    return {"t_local": sum(ms) / 1e3, "launches": int(launches)}, clk.summary()


def batched_form(args, stream, flush, torch, rc, tmp):
    """The batched workload: `--batch-cases` independent reacting viscous
    nozzles of uneven size (2k-60k triangles, 1-10 MPa, O/F 4-8, area ratio
    4-25, seed 5) in one context, with the per-cell chemistry integrator, in
    FP64 and mixed precision; launch configuration chosen by the autotuner."""
    from rocketcombustor_gb300 import cases
    dirs = cases.make_batch(os.path.join(tmp, "batch"), args.batch_cases, 5)
    cs = [rc.Case(d) for d in dirs]
    ne = sum(c.NE for c in cs)
    out = {"workload": f"{len(cs)} cases, {ne} triangles in total ({min(c.NE for c in cs)}-"
                       f"{max(c.NE for c in cs)} per case), integrated chemistry",
           "cells": ne}
    states = {}
    for form, prec in (("fp64", rc.RC_PREC_FP64), ("mixed", rc.RC_PREC_MIXED)):
        b = rc.BatchSolver(cs, precision=prec, stream=stream.cuda_stream)
        b.set_chemistry(rc.RC_CHEM_INTEGRATED)
        tune = b.autotune(3)
        r, _ = time_form(b, args, stream, flush, None, torch, rc)
        ns = b.chem_substeps()
        states[form] = b.get_state()[0]
        out[form] = {"value": ne * args.steps / r["t_local"], "ms_per_step": 1e3 * r["t_local"] / args.steps,
                     "gpu_launches": r["launches"], "autotune": tune,
                     "chem_substeps": {"min": int(ns.min()), "mean": float(ns.mean()), "max": int(ns.max())}}
        out[form].update(subroutine_times(b, args, stream, flush, torch))
        b.close()
    den = np.maximum(np.abs(states["fp64"]).max(axis=0), 1e-300)
    e = np.abs(states["mixed"] - states["fp64"]).max(axis=0) / den
    out["mixed"]["rel_linf_vs_fp64"] = {"p": float(e[0]), "T": float(e[3]), "Y": [float(x) for x in e[4:]],
                                        "after_iterations": args.warmup + args.steps}
    return out, cs, states["fp64"]


def bdf2_form(args, stream, torch, rc, tmp):
    """The reference's shipped time scheme (flow_solver_info.in: dual-time
    BDF2, CFL 10, dt = 1e-8 s, up to 10 inner iterations to relTol 1e-3) on
    the 120k-cell reacting viscous nozzle: physical steps through
    Solver.bdf2_stage (one graph launch per inner iteration, a host read of
    the inner residual after each), the BDF2_LU_SGS pieces timed alone, and
    one step of the CPU oracle on all host threads beside it."""
    import time as _time
    d, cfg = make_workload("c2u", tmp)
    case = rc.Case(d)
    u = case.unsteady
    s = rc.Solver(case, stream=stream.cuda_stream)
    s.set_p_out(u["p_static"])
    warm = 2
    for i in range(1, warm + 1):
        s.bdf2_stage(i, u["dt"], u["inner_loop"], u["rel_tol"])
    s.sync()
    l0 = s.stats()["kernel_launches"]
    inner = []
    t0 = _time.perf_counter()
    for i in range(warm + 1, warm + args.bdf2_steps + 1):
        inner.append(s.bdf2_stage(i, u["dt"], u["inner_loop"], u["rel_tol"]))
    s.sync()
    wall = _time.perf_counter() - t0
    launches = s.stats()["kernel_launches"] - l0
    # one inner iteration's BDF2_LU_SGS alone, device-timed (residual assembled first)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    with torch.cuda.stream(stream):
        s.timestep(); s.reconstruction(); s.flux_sourceterm()
        s.sync()
        ev[0].record(stream)
        s.flux_sourceterm()
        ev[1].record(stream)
        s.bdf2_lusgs(2, 0.5, u["dt"])
        ev[2].record(stream)
        s.sync()
    n_inner = sum(inner)
    out = {"workload": f"c2u: {case.NE} triangles, reacting viscous, BDF2 dt {u['dt']:.3g} s, "
                       f"InnerLoop {u['inner_loop']}, relTol {u['rel_tol']:g}",
           "physical_steps": args.bdf2_steps, "inner_iterations": inner,
           "ms_per_step": 1e3 * wall / args.bdf2_steps, "ms_per_inner_iteration": 1e3 * wall / n_inner,
           "cell_inner_iters_per_s": case.NE * n_inner / wall, "gpu_launches": int(launches),
           "timing": "wall clock around the steps (the stage reads the inner residual on the host "
                     "after every inner iteration)",
           "subroutine_ms": {"flux_sourceterm": ev[0].elapsed_time(ev[1]),
                             "bdf2_lu_sgs": ev[1].elapsed_time(ev[2])},
           "levels": {k: v for k, v in s.stats().items() if k != "kernel_launches"}}
    s.close()
    if not args.no_cpu:
        import oracle
        o = oracle.Oracle(d, threads=oracle.Oracle.max_threads())
        t0 = _time.perf_counter()
        n_cpu = o.unsteady_step(1)[0]
        t_cpu = _time.perf_counter() - t0
        out["cpu_oracle"] = {"ms_per_inner_iteration": 1e3 * t_cpu / n_cpu, "inner_iterations": n_cpu,
                             "threads": oracle.Oracle.max_threads(),
                             "cell_inner_iters_per_s": case.NE * n_cpu / t_cpu}
        o.close()
    case.close()
    return out


def batched_surrogate(args, stream, flush, torch, rc, cs, ref_state, net):
    """The batched workload with the surrogate chemistry (FP64 otherwise),
    against the batched FP64 run with the integrator after the same
    iterations."""
    b = rc.BatchSolver(cs, stream=stream.cuda_stream)
    b.set_surrogate(net)
    b.set_chemistry(rc.RC_CHEM_SURROGATE)
    tune = b.autotune(3)
    r, _ = time_form(b, args, stream, flush, None, torch, rc)
    st = b.get_state()[0]
    n_net, n_fb = b.surrogate_stats()
    ne = b.NE
    den = np.maximum(np.abs(ref_state).max(axis=0), 1e-300)
    e = np.abs(st - ref_state).max(axis=0) / den
    out = {"value": ne * args.steps / r["t_local"], "ms_per_step": 1e3 * r["t_local"] / args.steps,
           "gpu_launches": r["launches"], "autotune": tune, "cells_network": n_net, "cells_integrator": n_fb,
           "rel_linf_vs_integrated_fp64": {"p": float(e[0]), "T": float(e[3]), "Y": [float(x) for x in e[4:]],
                                           "after_iterations": args.warmup + args.steps}}
    b.close()
    return out


def rel_err(st, ref) -> dict:
    """Relative L-infinity difference per field (p, T, Y_k) of a state against
    a reference state, each field relative to the reference field's maximum."""
    den = np.maximum(np.abs(ref).max(axis=0), 1e-300)
    e = np.abs(st - ref).max(axis=0) / den
    return {"p": float(e[0]), "T": float(e[3]), "Y": [float(x) for x in e[4:]]}


def steady_run(s, args, dc_window=0, freeze_window=0):
    """run_to_steady with wall time (set-up excluded: the solver exists and its
    state is set; the timed loop includes the graph launches and the host reads
    of the norms)."""
    s.sync()
    t0 = time.perf_counter()
    r = s.run_to_steady(args.tol, args.max_iters, args.every, dc_window=dc_window, freeze_window=freeze_window)
    wall = time.perf_counter() - t0
    reached = r["reached"]
    out = {"iterations": r["iterations"], "wall_s": wall,
           "reached_tol_at": reached[0] if len(reached) == 1 else reached,
           "final_level": float(np.max(r["levels"])),
           "lowest_level": float(min(float(np.max(lv)) for _, lv in r["history"])),
           "ms_per_iteration": 1e3 * wall / r["iterations"]}
    if dc_window:
        out["switched_to_dc_at"] = r["switched_at"]
    if freeze_window:
        out["surrogate_choice_frozen_at"] = r["frozen_at"]
    return out, r


def converge(args, rc, torch):
    """Wall time to the steady state, max_k Res_k(n)/Res_k(1) <= tol (the
    step_residual columns), for the plain FP64 path and each form, with each
    form's final state against the FP64 converged state, and the oracle's
    time to the same criterion on all host threads."""
    out = {"mode": "converge", "metric": "wall time to steady", "tol": args.tol, "every": args.every,
           "criterion": "max_k Res_k(n)/Res_k(1) <= tol, Res_k = sum(vol*|dU_k|)/V_tot after LU-SGS "
                        "(the step_residual columns), Res_k(1) after the first iteration"}
    case_name = args.case if args.case not in ("c4", "c2") else "s2"
    with tempfile.TemporaryDirectory() as tmp:
        d, cfg = make_workload(case_name, tmp, **case_overrides(args))
        case = rc.Case(d)
        out["config"] = workload_config(cfg, case.NE, case.NF, par_label(1))
        forms = {}
        # plain FP64 (the reference's operation order, explicit chemical source)
        s = rc.Solver(case)
        f, r64 = steady_run(s, args)
        P64 = s.get_state()[0]
        it64 = r64["iterations"]
        s.close()
        forms["fp64"] = f
        # mixed precision alone: FP32 residual, stalls at its rounding level
        s = rc.Solver(case, precision=rc.RC_PREC_MIXED)
        a2 = argparse.Namespace(**{**vars(args), "max_iters": it64})
        f, _ = steady_run(s, a2)
        f["rel_linf_vs_fp64_converged"] = rel_err(s.get_state()[0], P64)
        s.close()
        forms["mixed"] = f
        # mixed precision switching to defect correction when it stalls
        s = rc.Solver(case, precision=rc.RC_PREC_MIXED)
        f, _ = steady_run(s, args, dc_window=args.dc_window)
        f["rel_linf_vs_fp64_converged"] = rel_err(s.get_state()[0], P64)
        s.close()
        forms["mixed_dc"] = f
        if not args.no_batch:
            forms["batched"] = converge_batched(args, rc, tmp)
        if not args.no_surrogate and cfg.combustion and cfg.nsp == 4:
            forms["surrogate"] = converge_surrogate(args, rc, torch, case)
        out["forms"] = forms
        if not args.no_cpu:
            import oracle
            th = oracle.Oracle.max_threads()
            o = oracle.Oracle(d, threads=th)
            t0 = time.perf_counter()
            h = o.run(it64, history=True)
            wall = time.perf_counter() - t0
            res = h[:, :-1]
            m = res[0] > 0
            lv = np.where(m, res / np.where(m, res[0], 1.0), 0.0).max(axis=1)
            hit = np.nonzero(lv <= args.tol)[0]
            out["cpu_baseline"] = {"kind": "port", "cores": th, "iterations": it64, "wall_s": wall,
                                   "reached_tol_at": int(hit[0] + 1) if hit.size else None,
                                   "final_level": float(lv[-1]),
                                   "state_equals_gpu_fp64": bool(np.array_equal(o.array("PA"), P64)),
                                   "sample": f"the oracle's {it64} iterations (as many as the FP64 GPU run took)"}
            o.close()
        case.close()
    print(json.dumps(out), flush=True)
    return 0


def converge_batched(args, rc, tmp):
    """The batched form to steady: `--batch-cases` uneven cases of the steady
    spread (500-5000 cells each) in one context, FP64 and mixed with the
    defect-correction switch; each case's iteration to tol, and the mixed
    batch's states against the FP64 batch's."""
    from rocketcombustor_gb300 import cases
    cfgs = cases.steady_batch_configs(args.batch_cases)
    dirs = []
    for c in cfgs:
        dd = os.path.join(tmp, "steady_batch", c.name)
        cases.write_case(dd, c)
        dirs.append(dd)
    cs = [rc.Case(x) for x in dirs]
    res = {"cases": len(cs), "cells": int(sum(c.NE for c in cs)),
           "cells_per_case": [int(c.NE) for c in cs]}
    b = rc.BatchSolver(cs)
    f, _ = steady_run(b, args)
    ref = b.get_state()[0]
    b.close()
    res["fp64"] = f
    b = rc.BatchSolver(cs, precision=rc.RC_PREC_MIXED)
    f, _ = steady_run(b, args, dc_window=args.dc_window)
    st = b.get_state()[0]
    off = b.offsets
    f["rel_linf_vs_fp64_converged"] = [rel_err(st[off[k]:off[k + 1]], ref[off[k]:off[k + 1]])
                                       for k in range(len(cs))]
    b.close()
    res["mixed_dc"] = f
    for c in cs:
        c.close()
    return res


def converge_surrogate(args, rc, torch, case):
    """The surrogate form to steady on the same case: the network trained here
    on integrator pairs from this case's states, then the steady runs with the
    integrated source (FP64) and with the surrogate source (FP64, cells the
    error indicator rejects sent to the integrator), and the surrogate's
    converged state against the integrated one."""
    from rocketcombustor_gb300 import surrogate
    s = rc.Solver(case)
    s.set_chemistry(rc.RC_CHEM_INTEGRATED)
    t0 = time.perf_counter()
    pool = surrogate.collect_pool(s, iters=200, every=20)
    x, t, nsub = surrogate.build_dataset(s, pool, args.sur_samples, seed=7)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    s.close()
    ntr = x.shape[0] - min(1 << 18, x.shape[0] // 10)
    net = surrogate.MLP(seed=7)
    net.fit_norm(x[:ntr])
    t0 = time.perf_counter()
    net.train(x[:ntr], t[:ntr], steps=args.sur_steps, batch=8192, lr=2e-3, lr_end=3e-5)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    out = {"training": {"samples": int(x.shape[0]), "data_s": t_data, "steps": args.sur_steps, "train_s": t_train,
                        "validation_vs_integrator": surrogate.validate(net, x[ntr:], t[ntr:])}}
    s = rc.Solver(case)
    s.set_chemistry(rc.RC_CHEM_INTEGRATED)
    f, _ = steady_run(s, args)
    ref = s.get_state()[0]
    s.close()
    out["integrated_fp64"] = f
    s = rc.Solver(case)
    s.set_surrogate(net)
    s.set_chemistry(rc.RC_CHEM_SURROGATE)
    f, _ = steady_run(s, args, freeze_window=args.dc_window)
    f["rel_linf_vs_integrated_converged"] = rel_err(s.get_state()[0], ref)
    a, b_ = s.surrogate_stats()
    f["cells_network"], f["cells_integrator"] = a, b_
    s.close()
    out["surrogate_fp64"] = f
    net.close()
    return out


def surrogate_form(args, stream, flush, torch, rc, case, extra_pool=None):
    """The learned-surrogate workload on the same nozzle: pairs from the FP64
    integrator on states of this case's trajectory (integrated source) and,
    when given, the batched cases' states, the network trained on the GPU by
    the project's kernels, its inference throughput, and the steady iteration
    with the surrogate source against the one with the integrated source.
    Returns (results, network)."""
    from rocketcombustor_gb300 import surrogate
    out = {}
    ref = rc.Solver(case, stream=stream.cuda_stream)
    ref.set_chemistry(rc.RC_CHEM_INTEGRATED)
    t0 = time.perf_counter()
    pool = surrogate.collect_pool(ref, iters=20, every=5)
    if extra_pool is not None:
        pool = torch.cat([pool, extra_pool], 1).contiguous()
    x, t, nsub = surrogate.build_dataset(ref, pool, args.sur_samples, seed=7)
    torch.cuda.synchronize()
    out["data"] = {"samples": int(x.shape[0]), "seconds": time.perf_counter() - t0,
                   "integrator_substeps": {"mean": float(nsub.float().mean()), "max": int(nsub.max())},
                   "domain": {"T": surrogate.T_RANGE, "p": surrogate.P_RANGE, "dt": surrogate.DT_RANGE}}
    ntr = x.shape[0] - min(1 << 20, x.shape[0] // 10)
    net = surrogate.MLP(seed=7)
    net.fit_norm(x[:ntr])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = net.train(x[:ntr], t[:ntr], steps=args.sur_steps, batch=8192, lr=2e-3, lr_end=3e-5,
                     log_every=max(1, args.sur_steps // 4))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    flops_sample = 2 * (7 * 128 + 3 * 128 * 128 + 128 * 4)
    out["training"] = {"steps": args.sur_steps, "batch": 8192, "seconds": t_train,
                       "loss": [[int(a), float(b)] for a, b in hist],
                       "tflops": 3 * flops_sample * 8192 * args.sur_steps / t_train / 1e12}
    out["validation_vs_integrator"] = surrogate.validate(net, x[ntr:], t[ntr:])
    xi = x[:min(1 << 22, x.shape[0])].contiguous()
    net.forward(xi)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    torch.cuda.synchronize()
    ev[0].record()
    for _ in range(10):
        net.forward(xi)
    ev[1].record()
    torch.cuda.synchronize()
    t_inf = ev[0].elapsed_time(ev[1]) / 1e3 / 10
    peak = read_peaks_tensor()
    out["inference"] = {"samples": int(xi.shape[0]), "samples_per_s": xi.shape[0] / t_inf,
                        "tflops": flops_sample * xi.shape[0] / t_inf / 1e12, "peak_bf16_tflops": peak,
                        "note": "k_mlp_fwd16: all five layers on tcgen05 (F16 operands, FP32 accumulation in "
                                "TMEM, packed-half GELU epilogue); FLOP counted for the whole network"}
    # steady iterations: integrated source vs surrogate source, same start
    forms = {}
    states = {}
    for name in ("integrated", "surrogate"):
        s = rc.Solver(case, stream=stream.cuda_stream)
        if name == "surrogate":
            s.set_surrogate(net)
            s.set_chemistry(rc.RC_CHEM_SURROGATE)
        else:
            s.set_chemistry(rc.RC_CHEM_INTEGRATED)
        s.autotune(3)
        r, _ = time_form(s, args, stream, flush, None, torch, rc)
        states[name] = s.get_state()[0]
        forms[name] = {"value": case.NE * args.steps / r["t_local"], "ms_per_step": 1e3 * r["t_local"] / args.steps,
                       "gpu_launches": r["launches"]}
        if name == "surrogate":
            a, b = s.surrogate_stats()
            forms[name]["cells_network"], forms[name]["cells_integrator"] = a, b
        s.close()
    den = np.maximum(np.abs(states["integrated"]).max(axis=0), 1e-300)
    e = np.abs(states["surrogate"] - states["integrated"]).max(axis=0) / den
    forms["surrogate"]["rel_linf_vs_integrated"] = {"p": float(e[0]), "T": float(e[3]),
                                                    "Y": [float(v) for v in e[4:]],
                                                    "after_iterations": args.warmup + args.steps}
    out["steady"] = forms
    ref.close()
    return out, net


def mlp_infer(args, torch):
    """Inference of the surrogate network (random weights, seed 3) on
    `--mlp-infer` samples of a fixed synthetic spread of states: samples/s and
    TFLOP/s over 10 CUDA-event-timed calls, and the largest output difference
    from the FP64 reference forward (oracle/mlp_ref.py, no rounding) on 1,000
    of them."""
    from oracle import mlp_ref
    from rocketcombustor_gb300 import surrogate
    mean = np.array([0.6, 6.0, -1.8, -1.8, -0.05, -2.3, -7.0], dtype=np.float32)
    std = np.array([0.5, 0.7, 0.5, 0.5, 0.02, 0.8, 1.2], dtype=np.float32)
    rng = np.random.default_rng(9)
    n = args.mlp_infer
    x = np.stack([rng.uniform(300, 3800, n), 10 ** rng.uniform(4.7, 7, n), rng.uniform(0, .05, n),
                  rng.uniform(0, .05, n), rng.uniform(.85, .95, n), rng.uniform(0, .02, n),
                  10 ** rng.uniform(-9, -5, n)], 1).astype(np.float32)
    net = surrogate.MLP(seed=3)
    net.set_norm(mean, std)
    xd = torch.tensor(x, device="cuda")
    y = net.forward(xd[:1000]).cpu().numpy()
    yr, _ = mlp_ref.forward(net.get_params(), x[:1000], mean, std, bf=False)
    net.forward(xd)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(10):
        net.forward(xd)
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / 10
    flops = 2 * (7 * 128 + 3 * 128 * 128 + 128 * 4)
    print(json.dumps({"mode": "mlp_infer", "samples": n, "samples_per_s": n / t,
                      "tflops": flops * n / t / 1e12, "peak_bf16_tflops": read_peaks_tensor(),
                      "max_abs_err_vs_fp64": float(np.abs(y - yr).max()), "output_scale": float(np.abs(yr).max())}),
          flush=True)
    net.close()
    return 0


def mlp_train(args, torch):
    """`--mlp-train` Adam steps of the surrogate network (random weights, seed
    7) on 1,048,576 synthetic pairs (the states of mlp_infer, smooth targets of
    T), through rc_mlp_train (one CUDA graph per step): wall clock around the
    call after a 20-step warm-up, TFLOP/s at 3 x the forward FLOP per sample."""
    from rocketcombustor_gb300 import surrogate
    rng = np.random.default_rng(9)
    n = 1 << 20
    x = np.stack([rng.uniform(300, 3800, n), 10 ** rng.uniform(4.7, 7, n), rng.uniform(0, .05, n),
                  rng.uniform(0, .05, n), rng.uniform(.85, .95, n), rng.uniform(0, .02, n),
                  10 ** rng.uniform(-9, -5, n)], 1).astype(np.float32)
    f = (x[:, 0:1] - 2000) / 1000 * 0.5
    t = np.concatenate([np.tanh(f), f * f, np.sin(3 * f), 0 * f + 1], 1).astype(np.float32)
    xd, td = torch.tensor(x, device="cuda"), torch.tensor(t, device="cuda")
    net = surrogate.MLP(seed=7)
    net.fit_norm(xd)
    net.train(xd, td, steps=20, batch=8192)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = net.train(xd, td, steps=args.mlp_train, batch=8192, lr=2e-3, lr_end=3e-5, log_every=args.mlp_train)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    flops = 3 * 2 * (7 * 128 + 3 * 128 * 128 + 128 * 4) * 8192
    print(json.dumps({"mode": "mlp_train", "steps": args.mlp_train, "batch": 8192, "seconds": dt,
                      "ms_per_step": 1e3 * dt / args.mlp_train, "tflops": flops * args.mlp_train / dt / 1e12,
                      "loss_first_last": [hist[0][1], hist[-1][1]]}), flush=True)
    net.close()
    return 0


def read_peaks_tensor():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["bf16_tflops"])
    return 1900.0


def subroutine_times(s, args, stream, flush, torch):
    """Each reference subroutine timed with CUDA events on the solver stream."""
    subs = (("timestep", s.timestep), ("reconstruction", s.reconstruction),
            ("flux_sourceterm", s.flux_sourceterm), ("lu_sgs_steady", s.lu_sgs_steady))
    rec = {k: [] for k, _ in subs}
    with torch.cuda.stream(stream):
        for _ in range(max(3, min(args.steps, 20))):
            for name, fn in subs:
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fn()
                b.record(stream)
                rec[name].append((a, b))
        s.sync()
        torch.cuda.synchronize()
    return {"subroutine_ms": {k: float(np.mean([a.elapsed_time(b) for a, b in v])) for k, v in rec.items()}}


def e2e_through_abi(s, args, NE, V, torch):
    """Per step: PA, WA host->device from pinned memory, the stage, the residual
    norms and PA, WA device->host into pinned memory (wall clock)."""
    PA_h = torch.empty((NE, V), dtype=torch.float64, pin_memory=True).numpy()
    WA_h = torch.empty((NE, V), dtype=torch.float64, pin_memory=True).numpy()
    s.get_state(PA_h, WA_h)
    t0 = time.perf_counter()
    for it in range(args.e2e_steps):
        s.set_state(PA_h, WA_h)
        s.lu_sgs_stage(it + 1)
        s.residual()
        s.get_state(PA_h, WA_h)
    dt = time.perf_counter() - t0
    return {"value": NE * args.e2e_steps / dt, "unit": "cell-iters/s",
            "h2d_bytes_per_step": 2 * NE * V * 8, "d2h_bytes_per_step": 2 * NE * V * 8 + (V + 1) * 8}


if __name__ == "__main__":
    sys.exit(main())
