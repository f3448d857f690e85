#!/usr/bin/env python
"""Benchmark of the GB300 tet-FEM Newton path.

Default workload (the one the headline metric's target is stated on): the
batched uneven stream -- 512 independent 6-tet box meshes, nx, ny in [3, 12],
nz in [6, 48], hex edge 1 cm, Neo-Hookean or StVK 50/50, E log-uniform in
[1e4, 1e6] Pa, nu in [0.2, 0.45], one face clamped and the opposite face under
a traction of 1e2..1e3 Pa (seeded synthetic inputs).  One "step" solves every
instance of the batch to static equilibrium at ||g|| <= 1e-6 ||g0||.

  value     batched FP32+refinement solves/s, positions reset on the device,
            everything resident in HBM (device-timed with CUDA events)
  e2e       the same solves through the public C ABI from host meshes:
            instance creation (pattern + upload), solve, download, destroy
  plain_gpu the plain FP64 device-resident drop-in, one instance per solve
            call like the reference's per-object solver, on a bounded sample
  cpu_baseline / --impl reference
            the CPU restatement of the reference's Newton path (LDLT Newton,
            the reference's default linear solver), all host threads, on a
            bounded sample of the same instances

Other workloads: --workload cantilever (8x8x32, FP64 plain vs the CPU
reference), large (48x48x192 single instance), serve (Poisson stream),
dynamics (implicit Euler, 32^3 blocks).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS_FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------
def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return PEAKS_FALLBACK, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return world, rank, local, dist


def dist_max(dist, value):
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_sum(dist, value):
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def dist_barrier(dist):
    if dist is not None:
        dist.barrier()


def percentile(a, q):
    a = sorted(a)
    if not a:
        return None
    k = (len(a) - 1) * q / 100.0
    f, c = math.floor(k), math.ceil(k)
    return a[f] if f == c else a[f] + (a[c] - a[f]) * (k - f)


# ---------------------------------------------------------------------------
# CPU reference arm: the oracle restatement of the reference's Newton path
# ---------------------------------------------------------------------------
def cpu_reference(meshes, budget_s, tol_rel, threads):
    import oracle
    t0 = time.perf_counter()
    done = 0
    sols = {}
    for i, m in enumerate(meshes):
        orc = oracle.Oracle(m)
        x0 = orc.rest()
        g0 = float(np.linalg.norm(orc.gradient(x0)))
        x, rep = orc.solve_static(x0, tol_max_error=tol_rel * g0, tol_min_impr=0.0, tol_min_step=0.0,
                                  threads=threads)
        sols[i] = (x, rep)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return done, dt, sols


def _oracle_batch_instance(job):
    """One batch instance through the oracle (LDLT Newton, one thread): run in a spawned worker."""
    seed, i, tol_rel = job
    import oracle
    from physim_gb300 import mesh as M
    m = M.batch_instance(seed, i)
    orc = oracle.Oracle(m)
    x0 = orc.rest()
    g0 = float(np.linalg.norm(orc.gradient(x0)))
    t0 = time.perf_counter()
    x, r = orc.solve_static(x0, tol_max_error=tol_rel * g0, tol_min_impr=0.0, tol_min_step=0.0, threads=1)
    keep = {k: r[k] for k in ("result_name", "iterations", "bisections", "obj", "opt", "opt0")}
    return i, x, keep, time.perf_counter() - t0


def oracle_batch_parity(seed, sizes, tol_rel, gpu_x, gpu_reps, workers):
    """Every batch instance solved by the oracle on the host cores (outside any timed region,
    one single-threaded solve per worker process, largest first) and compared with the GPU's
    result: relative displacement error where both succeed, and the outcome of each instance
    that does not end SUCCESS on either side."""
    import multiprocessing as mp
    import oracle.build
    oracle.build.build_oracle()  # built once here, not by every worker
    order = sorted(range(len(sizes)), key=lambda i: -sizes[i])
    t0 = time.perf_counter()
    cpu = {}
    with mp.get_context("spawn").Pool(workers) as pool:
        for i, x, rep, secs in pool.imap_unordered(_oracle_batch_instance, [(seed, i, tol_rel) for i in order]):
            cpu[i] = (x, rep, secs)
    wall = time.perf_counter() - t0
    errs, failures = [], []
    for i in range(len(sizes)):
        xr, rr, _ = cpu[i]
        g = gpu_reps[i]
        x0 = None
        if rr["result_name"] == "SUCCESS" and g["result_name"] == "SUCCESS":
            from physim_gb300 import mesh as M
            x0 = M.batch_instance(seed, i).X0.ravel()
            errs.append(float(np.linalg.norm(gpu_x[i] - xr) / max(np.linalg.norm(xr - x0), 1e-300)))
        else:
            failures.append({"instance": i, "tets": int(sizes[i]), "gpu": g["result_name"], "cpu": rr["result_name"],
                             "gpu_rel_residual": g["opt"] / g["opt0"] if g["opt0"] > 0 else None,
                             "cpu_rel_residual": rr["opt"] / rr["opt0"] if rr["opt0"] > 0 else None,
                             "gpu_iterations": g["iterations"], "cpu_iterations": rr["iterations"]})
    gpu_bad = [f for f in failures if f["gpu"] != "SUCCESS"]
    agree = sum(f["cpu"] != "SUCCESS" for f in gpu_bad)
    return {"compared": len(sizes), "success_both": len(errs),
            "rel_displacement_err_max": max(errs) if errs else None,
            "rel_displacement_err_median": statistics.median(errs) if errs else None,
            "non_success_cpu_agree": f"{agree}/{len(gpu_bad)}",
            "gpu_only_failures": [f["instance"] for f in failures if f["gpu"] != "SUCCESS" and f["cpu"] == "SUCCESS"],
            "cpu_only_failures": [f["instance"] for f in failures if f["gpu"] == "SUCCESS" and f["cpu"] != "SUCCESS"],
            "failures": failures,
            "oracle": f"LDLT Newton (reference default linear solver), one thread per instance, {workers} "
                      f"processes, {wall:.1f} s wall, {sum(v[2] for v in cpu.values()):.1f} s CPU"}


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def batch_meshes(count, seed):
    from physim_gb300 import mesh as M
    return [M.batch_instance(seed, i) for i in range(count)]


def pinned_copy(a):
    """A copy of `a` in page-locked host memory (through torch), or a plain copy."""
    try:
        import torch
        t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)), pin_memory=True)
        out = t.numpy()
        out[...] = a
        return out, True
    except Exception:
        return np.array(a, copy=True), False


def pinned_mesh(m):
    """The mesh with every array the library uploads in pinned host memory."""
    pm = m.copy()
    ok = True
    for name in ("X0", "T", "lame", "rho", "model", "fixed", "force"):
        arr = np.ascontiguousarray(getattr(m, name))
        if name == "T":
            arr = arr.astype(np.int32)
        cp, good = pinned_copy(arr)
        setattr(pm, name, cp)
        ok = ok and good
    return pm, ok


LSEARCH = {"none": 0, "simple": 1, "armijo": 2, "wolfe-weak": 3, "wolfe-strong": 4}  # LSearchType


def served_options(px, args):
    """Served path: FP32 Hessian + PCG with FP64 refinement; the same PCG budget per Newton step
    as the plain path (served_sweeps x served_pcg_max = plain_pcg_max), fewer, longer sweeps."""
    return px.options(precision=px.PREC_FP32_REFINE, tol_rel=args.tol_rel, tol_max_error=0.0, tol_min_impr=0.0,
                      tol_min_step=0.0, pcg_chunk=args.pcg_chunk, inner_tol=args.inner_tol,
                      ls_num_max_iters=args.served_pcg_max, max_refine_sweeps=args.served_sweeps,
                      lsearch_type=LSEARCH[args.lsearch], negative_curvature=args.curvature)


def batch_config(args, count, tets):
    return {"workload": f"batched uneven boxes: {count} instances, 6-tet hexes, {tets} tets", "instances": count,
            "tets": tets, "tol_rel": args.tol_rel, "line_search": args.lsearch,
            "l2": "inputs larger than L2 (per-step working set well above 129 MB)",
            "inner_tol": args.inner_tol, "pcg_chunk": args.pcg_chunk, "negative_curvature": args.curvature,
            "plain_pcg_max_per_newton_step": args.plain_pcg_max,
            "served_pcg_per_sweep_x_sweeps": [args.served_pcg_max, args.served_sweeps]}


def run_batch(args, world, rank, dist):
    import physim_gb300 as px
    from physim_gb300 import build
    build.build()
    count = args.count
    meshes = batch_meshes(count, seed=3 + 1000 * rank)
    tets = sum(m.m for m in meshes)
    ctx = px.Context(args.device, arena_bytes=int(args.arena_gb * (1 << 30)))
    if args.pcg_grid >= 0:
        ctx.launch_settings(pcg_grid=args.pcg_grid)
    insts = ctx.create_instances(meshes)  # host parts built in parallel; same instances as one by one
    if args.no_graph:
        ctx.launch_settings(graph=0)
    served = served_options(px, args)
    plain = px.options(precision=px.PREC_FP64, tol_rel=args.tol_rel, tol_max_error=0.0, tol_min_impr=0.0,
                       tol_min_step=0.0, pcg_chunk=args.pcg_chunk, ls_num_max_iters=args.plain_pcg_max,
                       lsearch_type=LSEARCH[args.lsearch])

    def step():
        for it in insts:
            it.reset()
        return ctx.batch_solve(insts, served)[0]

    # launch settings tuned for this batch mix (untimed set-up; cached in the context)
    for it in insts:
        it.reset()
    tuner = ctx.tune_batch(insts, served) if not args.no_tune else None
    for _ in range(args.warmup):
        reps = step()
    bad = [r for r in reps if r["result_name"] != "SUCCESS"]
    # timed region: device events on the library stream around the K steps, clocks sampled
    # meanwhile; no per-launch events (the solve loop runs as graph launches)
    clocks = ClockSampler(0)
    clocks.start()
    dist_barrier(dist)
    launches0 = ctx.kernel_launches()
    ctx.mark(0)
    for _ in range(args.steps):
        reps = step()
    ctx.mark(1)
    ms = ctx.elapsed_ms(0, 1)
    launches = ctx.kernel_launches() - launches0
    clk = clocks.stop()
    # the same K steps again with per-launch events and stage clocks (host-driven loop), for
    # the per-kernel figures and the roofline
    kinds = ["control", "vecop", "elem_eg", "gather", "elem_hess", "assemble", "jacobi", "linsetup", "resid",
             "spmv", "pcg_update", "accum", "pcg_cluster"]
    ctx.profile(True)
    ctx.profile_reset()
    plaunch0 = ctx.kernel_launches()
    ctx.mark(4)
    for _ in range(args.steps):
        step()
    ctx.mark(5)
    ms_profiled = ctx.elapsed_ms(4, 5)
    plaunches = ctx.kernel_launches() - plaunch0
    prof = {}
    for k in kinds:
        n, t = ctx.profile_read(k)
        prof[k] = {"launches": n, "ms": t, "bytes": ctx.profile_bytes(k)}
    eng_launches, eng_event_ms = ctx.profile_read("engine")
    ctx.profile(False)
    ms = dist_max(dist, ms)
    total = dist_sum(dist, float(count * args.steps))
    value = total / (ms / 1e3)
    n_success = sum(r["result_name"] == "SUCCESS" for r in reps)
    value_success = dist_sum(dist, float(n_success * args.steps)) / (ms / 1e3)
    rel_res = [r["opt"] / r["opt0"] for r in reps if r["opt0"] > 0 and r["result_name"] == "SUCCESS"]
    final_x = [it.positions() for it in insts]  # the last timed step's results, for the oracle comparison
    newton = [r["iterations"] for r in reps]
    pcg = [r["pcg_iterations"] for r in reps]

    # roofline of the dominant kernel.  A solve alternates two kinds of launch: the persistent
    # engine k_engine (every stage but the cluster PCG; CUDA events around each launch, its
    # stages split by the device global timer between the grid barriers) and the cluster PCG
    # kernel k_pcg_cg (one 8-CTA cluster per waiting FP32 instance; CUDA events around it).
    peaks, peaks_kind = load_peaks()
    eng_kinds = [k for k in kinds if k != "pcg_cluster"]
    eng = {"ms": eng_event_ms, "bytes": sum(prof[k]["bytes"] for k in eng_kinds)}
    cl = prof["pcg_cluster"]
    cl_steps = cl["launches"]
    cl_launches = plaunches - 2 * eng_launches  # k_prep + k_engine per engine launch, the rest cluster kernels
    tj = {}
    tfile = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tfile):
        with open(tfile) as f:
            tj = json.load(f)

    def roof(name, nbytes, ms, nl, key):
        per = nbytes / max(1, nl)
        ach = nbytes / (ms / 1e3) / 1e9 if ms > 0 else 0.0
        tr = tj.get(key, {}).get("dram_over_algorithmic")
        return {"kernel": name, "bound": "hbm", "achieved": round(ach, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": round(ach / peaks["hbm_gbs"], 4), "traffic": None if tr is None else round(tr * per),
                "algorithmic_bytes_per_launch": round(per), "avg_launch_ms": round(ms / max(1, nl), 4),
                "launches": int(nl), "share": round(ms / max(1e-9, cl["ms"] + eng["ms"]), 3),
                "peak_kind": peaks_kind + " (hbm_gbs, copy bandwidth)"}

    r_cl = roof("k_pcg_cg<8,512>", cl["bytes"], cl["ms"], cl_steps, "pcg_cluster")
    r_cl["kernel_launches"] = int(cl_launches)
    r_eng = roof("k_engine<float>", eng["bytes"], eng["ms"], eng_launches, "engine")
    roofline, other = (r_cl, r_eng) if cl["ms"] >= eng["ms"] else (r_eng, r_cl)
    roofline["second_kernel"] = other
    r_eng["bound_note"] = ("the engine's largest stage is the FP64 element energy + gradient: FP64-pipe bound "
                           "(31 % of the FP64 pipe's peak in the ncu capture of a 32-instance batch), "
                           "so its HBM fraction is small by construction")
    roofline["traffic_note"] = ("traffic = DRAM bytes per launch from an ncu capture of a 32-instance batch, scaled "
                                "by algorithmic bytes; per-instance working sets fit in L2, so DRAM << algorithmic")
    spmv = prof["spmv"]
    spmv_gbs = spmv["bytes"] / (spmv["ms"] / 1e3) / 1e9 if spmv["ms"] > 0 else None
    # FP32 instances run SpMV fused with the PCG updates inside k_pcg_cluster
    pcg_gbs = r_cl["achieved"] if cl["ms"] > 0 else None
    eh = prof["elem_hess"]

    # e2e through the public API from host meshes: create, solve, download, destroy
    e2e_ms = []
    h2d = 0
    d2h = 0
    sub = meshes[: max(1, count // 4)] if args.e2e_sample else meshes  # the headline's own workload
    # inputs and result buffers in pinned host memory, staged before the timed region
    pinned_sub = [pinned_mesh(m) for m in sub]
    pinned_ok = all(p[1] for p in pinned_sub)
    for rep in range(4):  # one untimed warm-up, then the median of three
        xs = [pinned_copy(m.X0.ravel())[0] for m in sub]
        t0 = time.perf_counter()
        tmp = ctx.create_instances([pm for pm, _ in pinned_sub])
        r2, xo = ctx.batch_solve(tmp, served, xs, inplace=True)
        for it in tmp:
            it.close()
        if rep > 0:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
        h2d = sum(m.X0.nbytes + m.T.nbytes + m.lame.nbytes + m.rho.nbytes + m.model.nbytes + m.fixed.nbytes +
                  m.force.nbytes for m in sub) + sum(x.nbytes for x in xs)
        d2h = sum(x.nbytes for x in xo)
    e2e_value = len(sub) / (statistics.median(e2e_ms) / 1e3)

    # plain FP64 drop-in on a bounded sample (one solve call per instance)
    order = np.argsort([m.m for m in meshes])
    pick = order[np.linspace(0, len(order) - 1, min(args.plain_sample, len(order))).astype(int)]
    t0 = time.perf_counter()
    plain_reps = []
    for i in pick:
        insts[i].reset()
        _, r = insts[i].solve_static(plain)
        plain_reps.append(r)
    plain_s = time.perf_counter() - t0
    # the same sample through the served path, batched, for a like-for-like ratio
    for i in pick:
        insts[i].reset()
    ctx.mark(2)
    served_sample = ctx.batch_solve([insts[i] for i in pick], served)[0]
    ctx.mark(3)
    served_sample_ms = ctx.elapsed_ms(2, 3)
    plain_value = len(pick) / plain_s
    # the plain FP64 path batched through the same engine (its PCG in the engine's stages: the
    # cluster PCG is FP32 only), on the same sample and on the whole batch: what the FP32 +
    # refinement path buys at equal batching
    for i in pick:
        insts[i].reset()
    ctx.mark(2)
    plain_b_sample = ctx.batch_solve([insts[i] for i in pick], plain)[0]
    ctx.mark(3)
    plain_b_sample_ms = ctx.elapsed_ms(2, 3)
    plain_batched = {"sample": {"value": round(len(pick) / (plain_b_sample_ms / 1e3), 3), "unit": "solves/s",
                                "instances": len(pick),
                                "non_success": sum(r["result_name"] != "SUCCESS" for r in plain_b_sample)}}
    if not args.no_plain_batch:
        for it in insts:
            it.reset()
        ctx.mark(2)
        plain_b_all = ctx.batch_solve(insts, plain)[0]
        ctx.mark(3)
        plain_b_all_ms = ctx.elapsed_ms(2, 3)
        plain_batched["all"] = {"value": round(count / (plain_b_all_ms / 1e3), 3), "unit": "solves/s",
                                "instances": count, "ms": round(plain_b_all_ms, 1),
                                "non_success": sum(r["result_name"] != "SUCCESS" for r in plain_b_all),
                                "served_over_plain_batched": round(value / (count / (plain_b_all_ms / 1e3)), 2)}
    plain_batched["served_over_plain_batched_sample"] = round(plain_b_sample_ms / served_sample_ms, 2)

    out = {
        "metric": "static solves/s @1e-6 rel residual: served batched FP32+refine (value) vs plain FP64 GPU drop-in",
        "value": round(value, 3), "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32 (Hessian, PCG) + fp64 (gradient, residual, energy)",
        "data": "synthetic (seeded)",
        "config": batch_config(args, count, tets),
        "e2e": {"value": round(e2e_value, 3), "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "sample": f"{len(sub)} instances created from host meshes "
                "(phx_instances_create), solved, downloaded and destroyed per step; median of 3 after 1 warm-up",
                "host_memory": "pinned" if pinned_ok else "pageable (torch pinned allocation unavailable)"},
        "roofline": roofline,
        "plain_gpu": {"value": round(plain_value, 3), "unit": "solves/s",
                      "sample": f"{len(pick)} instances across the size range, one FP64 solve call each",
                      "served_same_sample": round(len(pick) / (served_sample_ms / 1e3), 3),
                      "ratio_served_over_plain": round((len(pick) / (served_sample_ms / 1e3)) / plain_value, 2),
                      "results": sorted(set(r["result_name"] for r in plain_reps))},
        "plain_gpu_batched": plain_batched,
        "elements_per_s": round(sum(r["hessian_evals"] * m.m for r, m in zip(reps, meshes)) * args.steps /
                                (eh["ms"] / 1e3), 1) if eh["ms"] > 0 else None,
        "elem_hess": {"launches": eh["launches"], "ms": round(eh["ms"], 3)},
        "spmv_gbs": None if spmv_gbs is None else round(spmv_gbs, 1),
        "pcg_cluster_gbs": pcg_gbs,
        "kernels_ms": {k: round(v["ms"], 3) for k, v in prof.items()},
        "kernels_n": {k: int(v["launches"]) for k, v in prof.items()},
        "kernel_launches": {"k_engine": int(eng_launches), "k_pcg_cg": int(cl_launches), "cluster_steps": int(cl_steps),
                            "note": "profiled pass (host-driven loop with per-launch events): "
                                    "ms_per_step_profiled"},
        "ms_per_step_profiled": round(ms_profiled / args.steps, 3),
        "tuner": tuner,
        "algorithmic_bytes": {k: v["bytes"] for k, v in prof.items()},
        "value_success": round(value_success, 3),
        "value_note": ("value counts every instance's solve; value_success only those that end SUCCESS (the "
                       "others end as the oracle's LDLT Newton does on the same instance: accuracy.oracle_all)"),
        "accuracy": {"rel_residual_max_success": max(rel_res) if rel_res else None,
                     "non_success": len(bad), "newton_median": statistics.median(newton),
                     "pcg_iters_median": statistics.median(pcg)},
        "clocks": clk, "gpu_launches": int(launches),
    }
    # CPU baseline on a bounded sample (rank 0 only): a fixed sample spaced evenly over the size
    # range, every instance solved (no time cut-off, which would drop the largest)
    if rank == 0 and not args.no_cpu:
        cpu_pick = list(order[np.linspace(0, len(order) - 1, args.cpu_sample).astype(int)])
        done, secs, sols = cpu_reference([meshes[i] for i in cpu_pick], math.inf, args.tol_rel, os.cpu_count())
        out["cpu_baseline"] = {"value": round(done / secs, 4), "unit": "solves/s", "cores": os.cpu_count(),
                               "kind": "port", "sample": f"{done} instances spaced evenly over the size range, all "
                                                         f"solved, LDLT Newton (reference default linear solver), "
                                                         f"{secs:.1f} s"}
        # accuracy of the served results against the FP64 oracle on those instances
        errs = []
        both_failed = 0
        for j, i in enumerate(cpu_pick[:done]):
            x0 = meshes[i].X0.ravel()
            xg = final_x[i]  # the served result (the instances were solved again in FP64 since)
            xr, rr = sols[j]
            if rr["result_name"] != "SUCCESS" or reps[i]["result_name"] != "SUCCESS":
                both_failed += rr["result_name"] != "SUCCESS" and reps[i]["result_name"] != "SUCCESS"
                continue
            errs.append(float(np.linalg.norm(xg - xr) / max(np.linalg.norm(xr - x0), 1e-300)))
        out["accuracy"]["rel_displacement_err_max"] = max(errs) if errs else None
        out["accuracy"]["rel_displacement_err_median"] = statistics.median(errs) if errs else None
        out["accuracy"]["compared"] = len(errs)
        out["accuracy"]["failed_on_both_cpu_and_gpu"] = int(both_failed)
    ctx.close()
    out["_parity_inputs"] = (3 + 1000 * rank, [m.m for m in meshes], final_x, reps)
    return out


def run_reference(args, world, rank):
    """--impl reference: the CPU restatement of the reference path, all host threads."""
    if rank != 0:
        return None
    meshes = batch_meshes(args.count, seed=3)
    order = np.argsort([m.m for m in meshes])
    vals = []
    samples = []
    for _ in range(args.warmup):
        cpu_reference([meshes[order[len(order) // 2]]], 1e9, args.tol_rel, os.cpu_count())
    # each step: four instances spread over the size range (every fourth of 16 spaced evenly by
    # size, the four sets in turn), all solved; no time cut-off, which would drop the largest
    pick16 = list(order[np.linspace(0, len(order) - 1, 16).astype(int)])
    for s in range(args.steps):
        pick = pick16[s % 4::4]
        done, secs, _ = cpu_reference([meshes[i] for i in pick], math.inf, args.tol_rel, os.cpu_count())
        vals.append(done / secs)
        samples.append(done)
    v = statistics.median(vals)
    return {"impl": "reference", "metric": "static solves/s @1e-6 rel residual: served batched FP32+refine (value) "
                                           "vs plain FP64 GPU drop-in",
            "value": round(v, 4), "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded)",
            "config": batch_config(args, args.count, sum(m.m for m in meshes)),
            "cpu_baseline": {"value": round(v, 4), "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": f"{sum(samples)} instances across the size range, LDLT Newton"},
            "e2e": {"value": round(v, 4), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_cantilever(args, world, rank, dist):
    import oracle
    import physim_gb300 as px
    from physim_gb300 import build, mesh as M
    build.build()
    m = M.cantilever()
    ctx = px.Context(args.device, arena_bytes=4 << 30)
    inst = px.Instance(ctx, m)
    x0 = m.X0.ravel().copy()
    o = px.options(precision=px.PREC_FP64, tol_rel=1e-8, tol_max_error=0.0, tol_min_impr=0.0, tol_min_step=0.0,
                   pcg_chunk=args.pcg_chunk, lsearch_type=LSEARCH[args.lsearch])
    for _ in range(args.warmup):
        inst.reset(); inst.solve_static(o)
    ctx.profile(True); ctx.profile_reset()
    clocks = ClockSampler(0); clocks.start()
    ctx.mark(0)
    for _ in range(args.steps):
        inst.reset()
        x, r = inst.solve_static(o)
    ctx.mark(1)
    ms = ctx.elapsed_ms(0, 1)
    clk = clocks.stop()
    out = {"metric": "cantilever static solves/s (FP64 plain GPU Newton, ||g||/||g0|| < 1e-8)",
           "value": round(args.steps / (ms / 1e3), 3), "unit": "solves/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
           "config": {"workload": "cantilever 8x8x32 hexes x 6 tets, 12288 tets", "line_search": args.lsearch},
           "report": r, "clocks": clk}
    if rank == 0 and not args.no_cpu:
        orc = oracle.Oracle(m)
        g0 = float(np.linalg.norm(orc.gradient(x0)))
        t0 = time.perf_counter()
        xr, rr = orc.solve_static(x0, tol_max_error=1e-8 * g0, tol_min_impr=0.0, tol_min_step=0.0,
                                  threads=os.cpu_count())
        secs = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(1 / secs, 4), "unit": "solves/s", "cores": os.cpu_count(),
                               "kind": "port", "sample": "one LDLT Newton solve", "report": rr}
        # the same solve on one thread (OpenMP covers only the element loops, as in the
        # reference; the report's t_* fields are its per-phase timers)
        t1 = time.perf_counter()
        _, r1 = orc.solve_static(x0, tol_max_error=1e-8 * g0, tol_min_impr=0.0, tol_min_step=0.0, threads=1)
        secs1 = time.perf_counter() - t1
        out["cpu_baseline_1thread"] = {"value": round(1 / secs1, 4), "unit": "solves/s", "cores": 1,
                                       "kind": "port", "sample": "one LDLT Newton solve", "report": r1}
        out["rel_displacement_err"] = float(np.linalg.norm(x - xr) / np.linalg.norm(xr - x0))
        out["speedup_vs_cpu"] = round(secs / (ms / 1e3 / args.steps), 1)
    ctx.close()
    return out



# ---------------------------------------------------------------------------
# serving stream: open-loop Poisson arrivals, continuous batching vs plain FIFO
# ---------------------------------------------------------------------------
def serving_requests(count, seed, warm_frac=0.3):
    """Request list: (mesh, base) where base is None for a cold request or the index of an
    earlier request whose instance is re-solved warm with its load perturbed by up to 10%."""
    from physim_gb300 import mesh as M
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        if i > 4 and rng.uniform() < warm_frac:
            base = int(rng.integers(0, i))
            while reqs[base][1] is not None:
                base = reqs[base][1]
            reqs.append((M.perturb_load(reqs[base][0], seed, i), base))
        else:
            reqs.append((M.serving_request(seed, i), None))
    return reqs


def serve_stream(px, ctx, reqs, rate, opts, seed, budget_bytes, slots):
    """Runs the served path live at `rate` req/s (open-loop Poisson arrivals).  A cold request
    hands its host mesh to the server, which builds the instance at admission (inside the
    request's latency); a warm request re-solves the live instance of an earlier request
    under its perturbed load, once that instance's earlier request has finished.  Returns
    per-request latencies (s), the wall time, the arrivals, the reports and server stats."""
    rng = np.random.default_rng(seed + 17)
    n = len(reqs)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
    srv = px.Server(ctx, max_slots=slots, budget_bytes=budget_bytes, opts=opts)
    inst_of = {}  # cold request -> its instance
    busy = set()  # instances (by cold request) with a request in flight
    lat = np.zeros(n)
    reps = [None] * n
    done = 0
    nxt = 0
    waiting = []
    t0 = time.perf_counter()
    while done < n:
        now = time.perf_counter() - t0
        while nxt < n and arrivals[nxt] <= now:
            waiting.append(nxt)
            nxt += 1
        still = []
        for r in waiting:
            mesh, base = reqs[r]
            if base is None:
                inst_of[r] = srv.submit_mesh(mesh, r)
                busy.add(r)
                continue
            if base in busy or base not in inst_of:  # its instance is still busy: wait for it
                still.append(r)
                continue
            inst_of[base].update_load(mesh.force, mesh.gravity)
            srv.submit(inst_of[base], r)
            busy.add(base)
        waiting = still
        active, queued = srv.progress()
        for tag, rep in srv.poll():
            lat[tag] = time.perf_counter() - t0 - arrivals[tag]
            reps[tag] = rep
            busy.discard(reqs[tag][1] if reqs[tag][1] is not None else tag)
            done += 1
        if active == 0 and (queued > 0 or (not waiting and nxt < n)):
            wait_to = arrivals[nxt] if (queued == 0 and nxt < n) else now + 5e-4
            time.sleep(max(0.0, min(0.002, wait_to - (time.perf_counter() - t0))))
    wall = time.perf_counter() - t0
    stats = srv.stats()
    srv.close()
    for inst in inst_of.values():
        inst.close()
    return lat, wall, arrivals, reps, stats


def fifo_latency(arrivals, service):
    """Exact single-server FIFO latencies from arrival times and measured service times."""
    lat = np.zeros(len(arrivals))
    free = 0.0
    for i, (a, s) in enumerate(zip(arrivals, service)):
        start = max(a, free)
        free = start + s
        lat[i] = free - a
    return lat, free


def run_serve(args, world, rank, dist, rates=None, count=None):
    """Open-loop Poisson serving of the 1:1:4 request mix (1e3..2e5 tets, 30 % warm re-solves)
    at each rate of the sweep: the served FP32+refine path with continuous batching and
    admission by the memory budget, against the plain FP64 drop-in as a FIFO queue of one
    solve call per request (a cold request's service time includes creating its instance)."""
    import physim_gb300 as px
    from physim_gb300 import build
    build.build()
    rates = rates or [float(r) for r in args.rates.split(",")]
    count = count or args.requests
    reqs = serving_requests(count, seed=11)
    ctx = px.Context(args.device, arena_bytes=int(args.serve_arena_gb * (1 << 30)))
    if args.pcg_grid >= 0:
        ctx.launch_settings(pcg_grid=args.pcg_grid)
    served = served_options(px, args)
    plain = px.options(precision=px.PREC_FP64, tol_rel=args.tol_rel, tol_max_error=0.0, tol_min_impr=0.0,
                       tol_min_step=0.0, ls_num_max_iters=args.plain_pcg_max)
    budget = int(min(args.serve_budget_gb, 0.94 * args.serve_arena_gb) * (1 << 30))
    # plain drop-in service times: one FP64 call per request, in request order
    svc = np.zeros(count)
    plain_reps = []
    plain_inst = {}
    for i, (mesh, base) in enumerate(reqs):
        t0 = time.perf_counter()
        if base is None:
            plain_inst[i] = px.Instance(ctx, mesh)
            key = i
        else:
            key = base
            plain_inst[key].update_load(mesh.force, mesh.gravity)
        _, r = plain_inst[key].solve_static(plain)
        svc[i] = time.perf_counter() - t0
        plain_reps.append(r["result_name"])
    for inst in plain_inst.values():
        inst.close()
    out = {"source": "1:1:4 boxes, 1e3..2e5 tets log-uniform, Neo-Hookean, gravity + face traction; "
                     "30% warm re-solves of a live instance with its load perturbed by up to 10%",
           "requests_per_rate": count, "tets": [int(min(m.m for m, _ in reqs)), int(max(m.m for m, _ in reqs))],
           "warm_fraction": round(sum(b is not None for _, b in reqs) / count, 3),
           "budget_gb": round(budget / (1 << 30), 1), "arena_gb": args.serve_arena_gb, "slots": args.slots,
           "cold_requests": "instance built at admission (pattern on host workers, device set-up inside the latency)",
           "sweep": []}
    served_res = []
    for rate in rates:
        lat, wall, arrivals, reps, st = serve_stream(px, ctx, reqs, rate, served, 5, budget, args.slots)
        served_res += [r["result_name"] for r in reps]
        flat, fwall = fifo_latency(arrivals, svc)
        out["sweep"].append({
            "rate": rate,
            "served": {"p50_ms": round(1e3 * percentile(list(lat), 50), 2),
                       "p99_ms": round(1e3 * percentile(list(lat), 99), 2),
                       "solves_per_s": round(count / wall, 2),
                       "peak_gb": round(st["peak"] / (1 << 30), 2), "evictions": st["evictions"]},
            "plain_fifo": {"p50_ms": round(1e3 * percentile(list(flat), 50), 2),
                           "p99_ms": round(1e3 * percentile(list(flat), 99), 2),
                           "solves_per_s": round(count / fwall, 2)},
        })
    out["served_results"] = {k: served_res.count(k) for k in sorted(set(served_res))}
    out["plain_results"] = {k: plain_reps.count(k) for k in sorted(set(plain_reps))}
    out["plain_service_ms"] = {"median": round(1e3 * statistics.median(svc), 2), "sum": round(1e3 * svc.sum(), 1)}
    out["plain_fifo_note"] = ("plain latencies: exact FIFO queue over the same arrival times with the measured "
                              "one-call FP64 service time of each request (cold: instance creation + solve)")
    ctx.close()
    return out


def _large_oracle_worker(tol_factor, threads, q):
    """The 48x48x192 cantilever through the oracle (Jacobi-PCG Newton, row-parallel CG), in a
    spawned process that runs on the host cores beside the GPU solves."""
    import oracle
    from physim_gb300 import mesh as M
    t0 = time.perf_counter()
    m = M.cantilever(48, 48, 192, seed=7)
    o = oracle.Oracle(m)
    x0 = o.rest()
    g0 = float(np.linalg.norm(o.gradient(x0)))
    x, r = o.solve_static(x0, tol_max_error=tol_factor * g0, tol_min_impr=0.0, tol_min_step=0.0, ls_solver=1,
                          cg_block_jacobi=1, ls_num_max_iters=12000, cg_parallel=1, threads=threads)
    q.put((x - x0, {k: r[k] for k in ("result_name", "iterations", "lin_iterations", "opt", "opt0")},
           time.perf_counter() - t0))


def run_large(args, world, rank, dist):
    """48x48x192 cantilever with per-element E: plain FP64 vs FP32+refinement at 1e-6."""
    import multiprocessing as mp
    orc_proc = None
    if args.large_oracle:  # started before the first GPU call (a spawned process)
        ctxm = mp.get_context("spawn")
        orc_q = ctxm.Queue()
        orc_proc = ctxm.Process(target=_large_oracle_worker,
                                args=(args.large_oracle_tol, max(1, (os.cpu_count() or 2) - 1), orc_q))
        orc_proc.start()
    import physim_gb300 as px
    from physim_gb300 import build, mesh as M
    build.build()
    m = M.cantilever(48, 48, 192, seed=7)
    ctx = px.Context(args.device, arena_bytes=int(args.arena_gb * (1 << 30)))
    inst = px.Instance(ctx, m)
    res = {}
    # served: PCG in the whole-GPU kernels (launch setting pcg_grid 1) and, for comparison,
    # inside the engine (pcg_grid 0, the same bits); each timed without profiling, then solved
    # again with per-kernel events
    for name, prec, pcg_grid in (("served_fp32_refine", px.PREC_FP32_REFINE, 1),
                                 ("served_engine_pcg", px.PREC_FP32_REFINE, 0),
                                 ("plain_fp64", px.PREC_FP64, 0)):
        o = px.options(precision=prec, tol_rel=args.tol_rel, tol_max_error=0.0, tol_min_impr=0.0, tol_min_step=0.0)
        if prec == px.PREC_FP64:
            o.ls_num_max_iters = args.plain_pcg_max
        else:
            o = served_options(px, args)
        ctx.launch_settings(pcg_grid=pcg_grid)
        inst.reset()
        ctx.mark(0)
        x, r = inst.solve_static(o)
        ctx.mark(1)
        ms = ctx.elapsed_ms(0, 1)
        inst.reset()
        ctx.profile(True)
        ctx.profile_reset()
        ctx.mark(2)
        x2, r2 = inst.solve_static(o)
        ctx.mark(3)
        ms_prof = ctx.elapsed_ms(2, 3)
        eh_n, eh_ms = ctx.profile_read("elem_hess")
        sp_n, sp_ms = ctx.profile_read("spmv")
        up_n, up_ms = ctx.profile_read("pcg_update")
        sp_b = ctx.profile_bytes("spmv")
        ctx.profile(False)
        assert np.array_equal(x, x2)
        res[name] = {"seconds": round(ms / 1e3, 3), "seconds_profiled": round(ms_prof / 1e3, 3), "report": r,
                     "elements_per_s": round(r["hessian_evals"] * m.m / (eh_ms / 1e3), 1) if eh_ms else None,
                     "spmv_gbs": round(sp_b / (sp_ms / 1e3) / 1e9, 1) if sp_ms else None,
                     "pcg_iteration_us": round((sp_ms + up_ms) * 1e3 / max(1, r["pcg_iterations"]), 2)}
        res[name]["x"] = x
    # the whole-GPU PCG kernels and the engine's PCG stages give the same bits
    assert np.array_equal(res["served_fp32_refine"]["x"], res["served_engine_pcg"]["x"])
    res["served_engine_pcg"].pop("x")
    xs, xp = res["served_fp32_refine"].pop("x"), res["plain_fp64"].pop("x")
    x0 = m.X0.ravel()
    out = {"metric": "large single instance static solve (48x48x192, 2.65M tets) @%g rel" % args.tol_rel,
           "value": res["served_fp32_refine"]["seconds"], "unit": "s", "higher_is_better": False,
           "n_gpus": world, "data": "synthetic (seeded per-element E)",
           "config": {"workload": "cantilever 48x48x192 x 6 tets, E log-uniform [1e4,1e6], 2654208 tets",
                      "tets": m.m, "nodes": m.n},
           "served_fp32_refine": res["served_fp32_refine"], "served_engine_pcg": res["served_engine_pcg"],
           "plain_fp64": res["plain_fp64"],
           "served_vs_plain_rel_displacement": float(np.linalg.norm(xs - xp) / np.linalg.norm(xp - x0)),
           "note": ("seconds: unprofiled; spmv_gbs, pcg_iteration_us: from a second, profiled solve (events around "
                    "each kernel, host-driven loop), which gives the same positions")}
    ctx.close()
    if orc_proc is not None:
        du, rep, secs = orc_q.get()
        orc_proc.join()
        nd = float(np.linalg.norm(du))
        out["oracle"] = {"solver": "oracle Newton, Jacobi(3x3)-PCG (row-parallel), ||g|| <= %g ||g0||" % args.large_oracle_tol,
                         "report": rep, "seconds": round(secs, 1),
                         "served_rel_displacement_err": float(np.linalg.norm((xs - x0) - du) / nd),
                         "plain_rel_displacement_err": float(np.linalg.norm((xp - x0) - du) / nd)}
    return out


def _dyn_stats(reps_steps):
    """Per-step statistics of batched implicit steps: Newton iterations, PCG iterations and FP64
    refinement sweeps per linear solve (above 1: the FP32 PCG needed the FP64 residual refinement)."""
    flat = [r for rr in reps_steps for r in rr]
    sweeps = [r["refine_sweeps"] / max(1, r["hessian_evals"]) for r in flat]
    refined = [k for k, rr in enumerate(reps_steps) if any(r["refine_sweeps"] > r["hessian_evals"] for r in rr)]
    return {"non_success": sum(r["result_name"] != "SUCCESS" for r in flat),
            "newton_per_step": round(statistics.mean(r["iterations"] for r in flat), 2),
            "pcg_per_step": round(statistics.mean(r["pcg_iterations"] for r in flat), 1),
            "sweeps_per_linear_solve_mean": round(statistics.mean(sweeps), 3),
            "sweeps_per_linear_solve_max": round(max(sweeps), 3),
            "steps_needing_refinement": refined}


def run_dynamics(args, world, rank, dist):
    """Implicit Euler on near-incompressible blocks (nu = 0.495, 4-cell slabs of 1e4 / 1e8 Pa).
    (1) 16 blocks of 32^3 hexes x 6 tets, batched steps, served FP32+refine vs plain FP64;
    (2) the FP32-vs-FP64 gap over a long run (200 steps) of full-size blocks;
    (3) per-step error against the FP64 oracle on a reduced block of the same material and
        slabs (the oracle's step of a 32^3 block takes over ten minutes on a host core set)."""
    import oracle
    import physim_gb300 as px
    from physim_gb300 import build, mesh as M
    build.build()
    dt = 1e-3
    n_inst = args.dyn_instances
    meshes = [M.slab_block(5, i) for i in range(n_inst)]
    ctx = px.Context(args.device, arena_bytes=int(args.arena_gb * (1 << 30)))
    # homogeneous large blocks: their PCG in the whole-GPU kernels (measured 2.6 % faster per
    # step than inside the engine)
    ctx.launch_settings(pcg_grid=1 if args.pcg_grid != 0 else 0)

    def opts(prec):
        if prec == px.PREC_FP64:
            return px.options(precision=prec, tol_rel=args.tol_rel, tol_max_error=0.0, tol_min_impr=0.0,
                              tol_min_step=0.0, ls_num_max_iters=args.plain_pcg_max)
        return served_options(px, args)

    res = {}
    for name, prec in (("served_fp32_refine", px.PREC_FP32_REFINE), ("plain_fp64", px.PREC_FP64)):
        insts = ctx.create_instances(meshes)
        for it, m in zip(insts, meshes):
            it.reset()
            it.set_velocities(M.slab_initial_velocity(m))
        o = opts(prec)
        ctx.mark(0)
        reps_all = [ctx.batch_dynamic_step(insts, o, dt) for _ in range(args.dyn_steps)]
        ctx.mark(1)
        ms = ctx.elapsed_ms(0, 1)
        res[name] = {"ms_per_step": round(ms / args.dyn_steps, 3), **_dyn_stats(reps_all)}
        for it in insts:
            it.close()

    # (2) long run: FP32+refine and FP64 in lockstep on the first blocks
    long_m = meshes[: args.dyn_long_instances]
    runs = {}
    for name, prec in (("fp32", px.PREC_FP32_REFINE), ("fp64", px.PREC_FP64)):
        insts = ctx.create_instances(long_m)
        for it, m in zip(insts, long_m):
            it.reset()
            it.set_velocities(M.slab_initial_velocity(m))
        runs[name] = (insts, opts(prec), [])
    gaps, t_long = [], time.perf_counter()
    for step in range(args.dyn_long_steps):
        xs = {}
        for name, (insts, o, reps) in runs.items():
            reps.append(ctx.batch_dynamic_step(insts, o, dt))
            xs[name] = [it.positions() for it in insts]
        g = [float(np.linalg.norm(a - b) / max(np.linalg.norm(b - m.X0.ravel()), 1e-300))
             for a, b, m in zip(xs["fp32"], xs["fp64"], long_m)]
        gaps.append(max(g))
    long = {"instances": len(long_m), "steps": args.dyn_long_steps, "seconds": round(time.perf_counter() - t_long, 1),
            "gap_fp32_vs_fp64_max": max(gaps), "gap_last": gaps[-1],
            "gap_by_step_every_10": [round(v, 9) for v in gaps[::10]],
            "fp32": _dyn_stats(runs["fp32"][2]), "fp64": _dyn_stats(runs["fp64"][2])}
    for insts, _, _ in runs.values():
        for it in insts:
            it.close()

    # (3) the oracle: each step from the oracle's own state, on a reduced block
    n = args.dyn_oracle_n
    L = 0.32 * n / 32
    mo = M.slab_block(5, 0, n=n, L=L)
    orc = oracle.Oracle(mo)
    x = orc.rest()
    v = M.slab_initial_velocity(mo, L=L)
    inst = px.Instance(ctx, mo)
    per = {"fp64": [], "fp32": []}
    traj = {"fp64": (x.copy(), v.copy()), "fp32": (x.copy(), v.copy())}
    traj_err = {"fp64": [], "fp32": []}
    oracle_s = 0.0
    ores = []
    for step in range(args.dyn_oracle_steps):
        t0 = time.perf_counter()
        xn, vn, ro = orc.solve_dynamic(x, v, dt, tol_max_error=1e-9, tol_min_impr=0.0, tol_min_step=0.0,
                                       threads=os.cpu_count())
        oracle_s += time.perf_counter() - t0
        ores.append(ro["result_name"])
        move = max(np.linalg.norm(xn - x), 1e-300)
        for name, prec in (("fp64", px.PREC_FP64), ("fp32", px.PREC_FP32_REFINE)):
            o = opts(prec)
            xg, vg, rg = inst.dynamic_step(o, dt, x, v)  # one step from the oracle's state
            per[name].append(float(np.linalg.norm(xg - xn) / move))
            tx, tv = traj[name]
            tx, tv, _ = inst.dynamic_step(o, dt, tx, tv)  # the GPU's own trajectory
            traj[name] = (tx, tv)
            traj_err[name].append(float(np.linalg.norm(tx - xn) / max(np.linalg.norm(xn - mo.X0.ravel()), 1e-300)))
        x, v = xn, vn
    inst.close()
    oracle_part = {"block": f"{n}^3 hexes x 6 tets ({mo.m} tets), same slabs, nu and initial velocity profile",
                   "steps": args.dyn_oracle_steps, "oracle_results": {k: ores.count(k) for k in set(ores)},
                   "oracle_seconds": round(oracle_s, 1),
                   "one_step_rel_err_vs_step_motion": {k: {"max": max(vv), "median": statistics.median(vv)}
                                                       for k, vv in per.items()},
                   "trajectory_rel_err_vs_displacement": {k: {"max": max(vv), "last": vv[-1]}
                                                          for k, vv in traj_err.items()},
                   "note": ("the oracle (LDLT Newton) is run to ||g|| <= 1e-9 and stops at its energy-noise band; "
                            "one-step errors start the GPU from the oracle's state, so they measure one solve")}

    out = {"metric": "implicit-Euler steps/s, 16 blocks 32^3 x 6 tets, nu=0.495, 1e4 contrast",
           "value": round(1e3 / res["served_fp32_refine"]["ms_per_step"], 3), "unit": "batched steps/s",
           "higher_is_better": True, "n_gpus": world, "data": "synthetic (seeded slab orientation)",
           "config": {"workload": "%d instances of a 32^3 block, 196608 tets each, %d steps" % (n_inst, args.dyn_steps),
                      "tol_rel": args.tol_rel},
           "served_fp32_refine": res["served_fp32_refine"], "plain_fp64": res["plain_fp64"],
           "long_run": long, "oracle": oracle_part}
    ctx.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batch", choices=["batch", "cantilever", "large", "serve", "dynamics"])
    ap.add_argument("--rates", default="200,500,1000,2000")
    ap.add_argument("--requests", type=int, default=160)
    ap.add_argument("--slots", type=int, default=256)
    ap.add_argument("--dyn-instances", type=int, default=16)
    ap.add_argument("--dyn-steps", type=int, default=10)
    ap.add_argument("--dyn-long-steps", type=int, default=200)
    ap.add_argument("--dyn-long-instances", type=int, default=2)
    ap.add_argument("--dyn-oracle-steps", type=int, default=20)
    ap.add_argument("--dyn-oracle-n", type=int, default=12)
    ap.add_argument("--served-pcg-max", type=int, default=3000)
    ap.add_argument("--served-sweeps", type=int, default=4)
    ap.add_argument("--plain-pcg-max", type=int, default=12000,
                    help="PCG iterations per Newton step of the plain FP64 path (the served path's budget is "
                         "served_sweeps x served_pcg_max = 4 x 3000)")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-plain-batch", action="store_true",
                    help="skip the plain FP64 solve of the whole batch through the batched engine (about 11 s)")
    ap.add_argument("--serve-budget-gb", type=float, default=150.0, help="serving admission budget (device bytes)")
    ap.add_argument("--serve-arena-gb", type=float, default=160.0, help="device arena of the serving context")
    ap.add_argument("--count", type=int, default=512)
    ap.add_argument("--tol-rel", type=float, default=1e-6)
    ap.add_argument("--inner-tol", type=float, default=1e-4)
    ap.add_argument("--pcg-chunk", type=int, default=32)
    ap.add_argument("--plain-sample", type=int, default=24)
    ap.add_argument("--cpu-sample", type=int, default=12,
                    help="instances of the batch's CPU baseline, spaced evenly over the size range, all solved")
    ap.add_argument("--arena-gb", type=float, default=48.0)
    ap.add_argument("--e2e-sample", action="store_true",
                    help="e2e on the first quarter of the instances instead of the whole workload")
    ap.add_argument("--curvature", type=int, default=0, choices=[0, 1],
                    help="served FP32 PCG at negative curvature: 0 truncate, 1 go on like Eigen's CG")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--pcg-grid", type=int, default=-1, choices=[-1, 0, 1],
                    help="launch setting pcg_grid for FP32 instances above 13,000 nodes: 1 PCG in the whole-GPU "
                         "kernels, 0 in the engine; -1: the workload's default (dynamics 1, the others the "
                         "context's default 0; the large workload times both)")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch settings (no batch tuner)")
    ap.add_argument("--no-graph", action="store_true",
                    help="host-driven solve loop instead of graph launches (a profiler then sees the engine)")
    ap.add_argument("--large-oracle", action="store_true",
                    help="large workload: solve it with the oracle on the host cores too and compare")
    ap.add_argument("--large-oracle-tol", type=float, default=1e-8,
                    help="the oracle's stopping rule, ||g|| <= tol ||g0|| (tighter than the GPU's, as the reference)")
    ap.add_argument("--no-oracle-all", action="store_true",
                    help="skip the comparison of every batch instance with the oracle (about a minute of host time)")
    ap.add_argument("--lsearch", default="simple", choices=sorted(LSEARCH),
                    help="line search of the GPU solves (LSearchType; the CPU baseline keeps Simple)")
    args = ap.parse_args()
    world, rank, local, dist = dist_setup()
    args.device = local  # one replica per GPU: this rank's library context lives on its own device
    if args.impl == "reference":
        out = run_reference(args, world, rank)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    if args.workload == "cantilever":
        out = run_cantilever(args, world, rank, dist)
    elif args.workload == "large":
        out = run_large(args, world, rank, dist)
    elif args.workload == "serve":
        out = run_serve(args, world, rank, dist)
    elif args.workload == "dynamics":
        out = run_dynamics(args, world, rank, dist)
    else:
        out = run_batch(args, world, rank, dist)
        seed, sizes, final_x, final_reps = out.pop("_parity_inputs")
        if not args.no_serve:
            # p50/p99 latency beside solves/s: the serving stream's rate sweep
            out["serving"] = run_serve(args, world, rank, dist)
        if rank == 0 and not args.no_cpu and not args.no_oracle_all:
            # every instance of the batch against the oracle, after all timed regions
            out["accuracy"]["oracle_all"] = oracle_batch_parity(seed, sizes, args.tol_rel, final_x, final_reps,
                                                                max(1, os.cpu_count() or 1))
    if rank == 0:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
