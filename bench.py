#!/usr/bin/env python3
"""Benchmark: site-image gradient evaluations per second of the NLCG step.

Workload (the mixed-precision configuration): two-component GL, a1=-1 b1=1,
a2=-0.6 b2=1, m1=(1,1), m2=(1,2), eta=-0.5, gamma=0.2, H=0.9, 256x256 sites
at dx=0.4, 64 images, seeded synthetic initial string (Meissner to one
fractional vortex per component, noise 1e-3).  One step = one nonlinear
conjugate-gradient iteration of the whole string (every image: update,
gradient, Polak-Ribiere direction, line quartic, line search), i.e.
256*256*64 site-image gradient evaluations.  The string (~0.9 GB of state
streams per step) is larger than L2, so no flush is needed between steps.

``value`` is the FP32 bulk-relaxation throughput (fields in FP32, every
reduction and the beta / step scalars in FP64); the FP64 polish throughput
is reported beside it.  ``e2e`` runs the same steps through the C ABI with
pinned host buffers: each e2e step is one outer iteration of the
reference's loop() in mode S (state copied in, 10 NLCG steps, per-image
energies copied out), with each step's state upload staged on a second
stream while the step before computes (``serial``: one synchronous upload
per step).  ``--impl reference`` times the CPU implementation of
the same step (the C restatement in oracle/, all host threads) on the same
workload.

``time_to_barrier`` times the barrier protocol on the same 256x256 string:
a string phase (IEEE FP64, or FP32 for the mixed schedule) seeds an IEEE
FP64 refinement of the initial minimum and of the index-1 saddle; the time
is until dF = F(saddle) - F(minimum) stays within 1e-6 of the converged FP64
value measured in the same run; ``--ttb-config 1`` runs it on the small
single-component string instead.  ``reference_cuda`` times the reference's
own CUDA NLCG (its unmodified nlcg.cu built for this GPU) beside this
library on configs 2 (FP32) and 1 (FP64).

Multi-GPU: the path does not shard within a string; ``--gpus N`` runs N
independent replicas (one string per GPU) and reports the aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "site·image grad evals/s; time-to-barrier @1e-6 rel, FP32+FP64 vs FP64"
UNIT = "site·image/s"
WORKLOAD = "two-component GL 256x256 dx=0.4, 64 images (mixed-precision config)"
RELAX = 10


def bench_config(world: int) -> dict:
    """The `config` of both arms' JSON lines (the same dict, so that the lines compare)."""
    return {"workload": WORKLOAD, "sites": 256 * 256, "images": 64, "components": 2,
            "line_polynomial": "exact", "line_search": "compat scan",
            "cache": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x: float, world: int, device="cuda") -> float:
    """The largest of each rank's x (the slowest replica's time); identity for one rank."""
    if world == 1:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replicas_value(world: int, units_per_step: int, steps: int, ms_max: float) -> float:
    """Whole-job throughput of `world` replicas: every rank's units over the slowest rank's time."""
    return world * units_per_step * steps / (ms_max / 1e3)


def cpu_oracle_step_rate(prob, st, images: int, steps: int, dtype, budget_s: float = 12.0):
    """Time the C oracle (OpenMP over images) on a sample of `images` images."""
    import numpy as np
    from oracle import cref
    sub = st.__class__(a=st.a[:images], psi_1=st.psi_1[:images],
                       psi_2=None if st.psi_2 is None else st.psi_2[:images])
    orc = cref.Oracle(prob, dtype, fast=True)
    sv = orc.solver(sub, ls_mode=cref.LS_COMPAT, poly_compat=False)
    sv.nlcg_steps(1)                     # warm-up (page-in, thread pool)
    done, t0 = 0, time.perf_counter()
    while done < steps or (time.perf_counter() - t0) < 1.0:
        sv.nlcg_steps(1)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    units = done * images * prob.nx * prob.ny
    return units / dt, dict(steps=done, images=images, seconds=dt, threads=cref.threads(fast=True))


def host_cpu():
    """CPU model and logical core count of this host (for the CPU baseline)."""
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key = line.split(":")[0].strip().lower()
                if key in ("model name", "cpu model", "hardware") and ":" in line:
                    model = line.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    if not model:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
            model = next((l.split(":", 1)[1].strip() for l in out.splitlines() if l.startswith("Model name")), None)
        except (OSError, subprocess.SubprocessError):
            model = None
    if not model:
        import platform
        model = platform.machine()
    return {"model": model, "logical_cores": os.cpu_count()}


def run_reference(args):
    """--impl reference: the CPU implementation (C oracle, all host threads)."""
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    import numpy as np
    from mepgl_gb300 import workloads
    from oracle import cref
    prob, st = workloads.config2()
    sample_images = 16
    orc = cref.Oracle(prob, np.float32, fast=True)
    sub = st.__class__(a=st.a[:sample_images], psi_1=st.psi_1[:sample_images], psi_2=st.psi_2[:sample_images])
    sv = orc.solver(sub, ls_mode=cref.LS_COMPAT, poly_compat=False)
    for _ in range(args.warmup):
        sv.nlcg_steps(1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sv.nlcg_steps(1)
    dt = time.perf_counter() - t0
    units = args.steps * sample_images * prob.nx * prob.ny
    value = units / dt
    sample = (f"{sample_images} of 64 images of the workload per step, {args.steps} steps, "
              f"C restatement (oracle/gl_oracle.c, -O3 -ffp-contract=fast) in FP32 with FP64 reductions, "
              f"OpenMP over images on all host threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(args.gpus),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cref.threads(fast=True), "kind": "port", "sample": sample,
                         "host": host_cpu()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import numpy as np
    import torch

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from mepgl_gb300 import native, workloads

    prob, st = workloads.config2()
    F = st.n_images
    sites = prob.nx * prob.ny
    units_per_step = sites * F
    stream = torch.cuda.Stream()          # a real stream: graph capture and events share it
    torch.cuda.set_stream(stream)
    ctx = native.StringContext(prob, F, "fp32", stream=stream.cuda_stream, line_polynomial=native.POLY_EXACT)
    ctx.set_state(st)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    def maxed(x):
        return max_over_ranks(x, world, "cuda")

    # ---- device-resident timed region (FP32 bulk relaxation) ----------------
    ctx.nlcg_steps(max(args.warmup, 3))
    barrier()
    l0 = ctx.info()["kernel_launches"]
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        ev0.record(stream)
        ctx.nlcg_steps(args.steps)
        ev1.record(stream)
        barrier()
    ms = maxed(ev0.elapsed_time(ev1))
    launches = ctx.info()["kernel_launches"] - l0
    value = replicas_value(world, units_per_step, args.steps, ms)
    fe = ctx.image_scalars()["fenergy"]
    assert np.all(np.isfinite(fe)), "non-finite energies"

    # ---- roofline: the fused persistent launch of the timed region (one launch
    # runs all timed steps; per step), with the separately launched passes timed
    # beside it on the same stream ------------------------------------------------
    ms_grad, ms_dir = ctx.profile_passes(10)
    k_grad, k_dir, k_fused = ctx.pass_kernels()
    S = (2 + 2 * 2) * 4                    # bytes of state per site-image (A, psi_1, psi_2 in FP32)
    bytes_grad = (5 * S + 2) * units_per_step  # read x, d, g_prev; write x, g; masks
    bytes_dir = (4 * S + 2) * units_per_step   # read x, g, d; write d; masks
    peak, peak_kind = peaks()
    kern = {k_grad: {"ms": ms_grad, "bytes": bytes_grad, "gbs": bytes_grad / ms_grad / 1e6},
            k_dir: {"ms": ms_dir, "bytes": bytes_dir, "gbs": bytes_dir / ms_dir / 1e6}}
    if k_fused:
        ms_step = ms / args.steps
        kern[k_fused] = {"ms": ms_step, "bytes": bytes_grad + bytes_dir,
                         "gbs": (bytes_grad + bytes_dir) / ms_step / 1e6, "per": "NLCG step"}
        dom = k_fused
    else:
        dom = max(kern, key=lambda k: kern[k]["ms"])
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic_config2_fp32.json")
    if os.path.exists(tfile):
        with open(tfile) as f:
            traffic = json.load(f).get(dom)
    roofline = {"bound": "hbm", "achieved": kern[dom]["gbs"], "peak": peak, "unit": "GB/s",
                "frac": kern[dom]["gbs"] / peak, "traffic": traffic, "kernel": dom,
                "peak_source": f"{peak_kind} hbm_gbs",
                "step_gbs": (bytes_grad + bytes_dir) / (ms_grad + ms_dir) / 1e6,
                "per": kern[dom].get("per", "launch")}

    # ---- FP64 polish throughput (same string): IEEE double and float-float ----
    def fp64_leg(arith):
        c64 = native.StringContext(prob, F, "fp64", stream=stream.cuda_stream, line_polynomial=native.POLY_EXACT,
                                   fp64_arith=arith)
        c64.set_state(st)
        c64.nlcg_steps(3)
        k64 = max(2, args.steps // 4)
        barrier()
        ev0.record(stream)
        c64.nlcg_steps(k64)
        ev1.record(stream)
        barrier()
        ms64 = maxed(ev0.elapsed_time(ev1))
        g64, d64 = c64.profile_passes(3)
        c64.close()
        return {"value": replicas_value(world, units_per_step, k64, ms64), "ms_per_step": ms64 / k64, "steps": k64,
                "ms_grad": g64, "ms_dir_poly": d64}

    fp64 = fp64_leg(native.FP64_NATIVE)
    fp64["paired"] = fp64_leg(native.FP64_PAIRED)
    # FP64 FLOP roofline of the IEEE-double passes: DADD + DMUL + 2 DFMA per
    # site-image counted by ncu (profiles/fp64_passes_flops_config2.md) over the
    # event-timed passes; no FP64 peak is measured on this machine, so the
    # denominator is GB300's nominal FP64 rate
    fp64_flop = {"k_grad": 480.3, "k_dir_poly": 711.4}
    nominal_fp64_tflops = 1.25
    fp64["flop_roofline"] = {
        k: {"flop_per_site_image": f, "tflops": f * units_per_step / (ms_ / 1e3) / 1e12,
            "frac_of_nominal": f * units_per_step / (ms_ / 1e3) / 1e12 / nominal_fp64_tflops}
        for (k, f), ms_ in zip(fp64_flop.items(), (fp64["ms_grad"], fp64["ms_dir_poly"]))}
    fp64["flop_roofline"]["peak"] = {"tflops": nominal_fp64_tflops, "source": "nominal (not measured)"}

    # ---- the reference's own CUDA build on this GPU ---------------------------
    # its unmodified nlcg.cu / parallel_sum.cu compiled for sm_103a (staged from
    # the reference tree into baseline/_ref by build()), one nlcgSteps call of
    # `steps` steps timed with CUDA events, beside this library on the same
    # workload and precision (compat line search and polynomial, as the
    # reference); config 2 in FP32 and config 1 in FP64
    refcuda = None
    if rank == 0 and not args.no_refcuda:
        from oracle import ref_cuda_build as RC
        if not RC.staged():
            refcuda = {"unavailable": "reference CUDA sources not staged in baseline/_ref (no reference tree "
                                      "where build() ran)"}
        else:
            refcuda = {}
            prob1, st1 = workloads.config1()
            for key, (pr, s0, prec, ours_prec) in {"config2_fp32": (prob, st, "f32", "fp32"),
                                                   "config1_fp64": (prob1, st1, "f64", "fp64")}.items():
                try:
                    k_steps = 20
                    r = RC.run(pr, s0, prec, k_steps, 3)
                    c_o = native.StringContext(pr, s0.n_images, ours_prec, stream=stream.cuda_stream)
                    c_o.set_state(s0)
                    c_o.nlcg_steps(3)
                    barrier()
                    ev0.record(stream)
                    c_o.nlcg_steps(k_steps)
                    ev1.record(stream)
                    barrier()
                    ms_o = ev0.elapsed_time(ev1) / k_steps
                    c_o.close()
                    units = pr.nx * pr.ny * s0.n_images
                    refcuda[key] = {"reference_ms_per_step": r["ms_per_step"],
                                    "reference_site_images_per_s": r["site_images_per_s"],
                                    "ours_ms_per_step": ms_o, "ours_site_images_per_s": units / (ms_o / 1e3),
                                    "speedup": r["ms_per_step"] / ms_o,
                                    "note": "reference: nlcgSteps (12 launches, 4 two-level sums with per-call "
                                            "cudaMalloc/cudaFree, host syncs per step); ours: the library's "
                                            "default NLCG path, same options"}
                except Exception as e:          # a failed reference build must not lose the bench line
                    refcuda[key] = {"unavailable": f"{type(e).__name__}: {str(e)[:200]}"}

    # ---- end to end through the C ABI with pinned host buffers -----------------
    shape = (F, prob.ny, prob.nx, 2)
    host = [torch.from_numpy(np.ascontiguousarray(x, np.float32)).pin_memory()
            for x in (st.a, st.psi_1, st.psi_2)]
    fe_host = torch.zeros(F, dtype=torch.float64).pin_memory()
    L = ctx.L
    import ctypes as C

    ptrs = [C.c_void_p(h.data_ptr()) for h in host]

    def e2e_serial(iters):
        # state in (synchronous copy), steps, energies out
        for _ in range(iters):
            ctx._check(L.mepgl_set_state(ctx.h, *ptrs, native.HOST))
            ctx.nlcg_steps(RELAX)
            ctx._check(L.mepgl_image_scalars(ctx.h, C.c_void_p(fe_host.data_ptr()), None, None))

    def e2e_staged(iters):
        # the same, with each step's inputs uploaded on the context's copy stream while
        # the step before computes (the first step's upload is exposed)
        ctx._check(L.mepgl_stage_state(ctx.h, *ptrs, native.HOST))
        for i in range(iters):
            ctx._check(L.mepgl_set_state(ctx.h, None, None, None, native.STAGED))
            if i + 1 < iters:
                ctx._check(L.mepgl_stage_state(ctx.h, *ptrs, native.HOST))
            ctx.nlcg_steps(RELAX)
            ctx._check(L.mepgl_image_scalars(ctx.h, C.c_void_p(fe_host.data_ptr()), None, None))

    def timed_e2e(fn, iters):
        fn(1)
        barrier()
        t0 = time.perf_counter()
        fn(iters)
        barrier()
        return maxed(time.perf_counter() - t0)

    e2e_iters = max(4, args.steps // 4)

    def rate(sec):
        return world * units_per_step * RELAX * e2e_iters / sec

    serial_s = timed_e2e(e2e_serial, e2e_iters)
    e2e_s = timed_e2e(e2e_staged, e2e_iters)
    h2d = sum(h.numel() * h.element_size() for h in host)
    e2e = {"value": rate(e2e_s), "unit": UNIT,
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": F * 8,
           "step": f"state from pinned host (staged upload of the next step's state overlapping this step) "
                   f"+ {RELAX} NLCG steps + per-image energies to host",
           "serial": {"value": rate(serial_s), "step": "the same with a synchronous state upload per step"}}

    # ---- time to barrier, plain FP64 against FP32 + FP64 ----------------------
    # One run (mepgl_gb300.barrier.time_to_barrier): a string phase in the
    # schedule's precision (mode L, linear reparametrization + `relax` NLCG
    # steps, a fixed budget of outer iterations), then the IEEE FP64
    # refinement of image 0 to its minimum and of the string's energy maximum
    # to the index-1 saddle (preconditioned CG, forcing term 0.1).  dF* = F(saddle) - F(minimum) of a first FP64 run
    # refined to |g| <= 1e-10 (measured here, not hard-coded); each run's time
    # to barrier is when its trace (the string's estimate, then the refined
    # barrier) enters and stays within 1e-6 of dF*.  Schedules: "fp64" IEEE
    # double string, "mixed" FP32 string, "fp64_paired" the string in
    # float-float FP64 (labelled as such); the refinement is IEEE double in all.
    ttb = None
    if rank == 0 and not args.no_ttb:
        from mepgl_gb300 import barrier as B
        # the 64x64 string seeds its saddle at one NLCG step per reparametrization
        # (600 iterations, the oracle golden's protocol); the 256x256 one at 10 (300)
        cfg, reps = args.ttb_config, args.ttb_repeats
        relax = 1 if cfg == 1 else 10
        budget = args.ttb_string if args.ttb_string is not None else (600 if cfg == 1 else 300)
        ref = B.time_to_barrier(cfg, "fp64", relax, max_string=budget, g_tol=1e-10)
        target = ref["barrier"]
        runs = {"fp64": [ref], "mixed": [], "fp64_paired": []}
        for _ in range(reps):
            runs["mixed"].append(B.time_to_barrier(cfg, "mixed", relax, max_string=budget))
            if len(runs["fp64"]) < reps:
                runs["fp64"].append(B.time_to_barrier(cfg, "fp64", relax, max_string=budget))
        runs["fp64_paired"].append(B.time_to_barrier(cfg, "fp64_paired", relax, max_string=budget))

        def leg(rs, rtol):
            ts = [B.time_within([x[0] for x in r["trace"]], [x[1] for x in r["trace"]], target, rtol) for r in rs]
            return {"times_s": ts, "median_s": statistics.median(ts) if all(t is not None for t in ts) else None,
                    "string_s": [r["string_s"] for r in rs], "string_iterations": [r["string_iterations"] for r in rs],
                    "refine_s": [r["total_s"] - r["string_s"] for r in rs],
                    "newton": [r["newton"] for r in rs], "total_s": [r["total_s"] for r in rs],
                    "barrier_rel_err": [abs(r["barrier"] - target) / abs(target) for r in rs],
                    "energy_rel_err": [max(abs(e - e0) / abs(e0) for e, e0 in zip(r["energies"], ref["energies"]))
                                       for r in rs],
                    "is_saddle": [r["is_saddle"] for r in rs], "seed_image": [r["seed_image"] for r in rs]}
        work = {1: "single-component GL 64x64 dx=0.5, 16 images", 2: WORKLOAD}[cfg]
        ttb = {"quantity": "dF = F(saddle) - F(minimum), refined stationary points; time until within 1e-6 of dF*",
               "workload": work, "relax_steps": relax, "string_budget_iterations": budget, "target_dF": target,
               "refinement": "IEEE FP64 Newton with gauge-subspace steps; CG preconditioned by the cosine-basis "
                             "inverse of a constant-coefficient Hessian model, relative tolerance 0.1 per step",
               "target_g_norms": ref["g_norms"], "target_min_curvature": ref["min_curvature"],
               "fp64": leg(runs["fp64"], 1e-6), "mixed": leg(runs["mixed"], 1e-6),
               "fp64_paired_string": leg(runs["fp64_paired"], 1e-6),
               "fp64_to_1e-8": leg(runs["fp64"], 1e-8)}
        if ttb["fp64"]["median_s"] and ttb["mixed"]["median_s"]:
            ttb["speedup_mixed_vs_fp64"] = ttb["fp64"]["median_s"] / ttb["mixed"]["median_s"]

    # ---- CPU baseline (rank 0, N = 1 only) ------------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        rate, info = cpu_oracle_step_rate(prob, st, images=16, steps=2, dtype=np.float32)
        cpu = {"value": rate, "unit": UNIT, "cores": info["threads"], "kind": "port", "host": host_cpu(),
               "sample": f"{info['steps']} NLCG steps on {info['images']} of 64 images of the workload "
                         f"({info['seconds']:.1f} s), C restatement -O3 -ffp-contract=fast in FP32, OpenMP over images"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(world),
            "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "kernels": kern, "fp64": fp64,
            "cpu_baseline": cpu, "clocks": clk.summary(), "time_to_barrier": ttb, "reference_cuda": refcuda,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-ttb", action="store_true", help="skip the time-to-barrier leg")
    ap.add_argument("--no-refcuda", action="store_true", help="skip timing the reference's own CUDA build")
    ap.add_argument("--ttb-config", type=int, choices=(1, 2), default=2,
                    help="workload of that leg: 2 (the 256x256 mixed-precision string) or 1 (64x64, seconds)")
    ap.add_argument("--ttb-repeats", type=int, default=3, help="runs per schedule of the time-to-barrier leg")
    ap.add_argument("--ttb-string", type=int, default=None,
                    help="string-phase budget of the time-to-barrier leg in outer iterations (default 300 of 10 "
                         "NLCG steps on the 256x256 string, 600 of 1 step on the 64x64 one)")
    args = ap.parse_args(argv)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
