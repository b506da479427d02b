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

``time_to_end_state`` times FP64 against FP32-then-FP64 relaxation of the
same 256x256 string to a converged end state (the barrier estimate of the
string method itself does not converge to 1e-6; see barrier.py);
``--ttb-config 1`` runs it on the small single-component string instead.

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

    # ---- time to a converged end state, FP64 vs FP32+FP64 (small string) -------
    # The barrier estimate of the string method does not converge to 1e-6 on
    # these workloads (its value drifts with the reparametrization cadence), so
    # this reports the time until the end-state energy difference F_{F-1} - F_0
    # (which does converge) stays within 1e-6 of the FP64 run's final value.
    # Default (--ttb-config 2): the mixed-precision workload itself, the 256x256
    # two-component string (100 steps per reparametrization; about 2.5 minutes),
    # IEEE FP64 against FP32 then paired-FP64 polish, to the value its long FP64
    # run converges to.  --ttb-config 1: the small single-component string
    # (64x64, 16 images, 50 steps per reparametrization; latency-bound, seconds).
    ttb = None
    if rank == 0 and not args.no_ttb:
        from mepgl_gb300 import barrier as B
        rmx = r64p = None
        if args.ttb_config == 2:
            target = 1.00779044   # F_{F-1} - F_0 after 600 outer iterations of FP64 (IEEE) relaxation
            r64, _ = B.run(2, 100, 160, "fp64")
            rmxp, _ = B.run(2, 100, 250, "mixed", -1, fp64_arith="paired")
            work = "two-component GL 256x256 dx=0.4, 64 images, mode L, 100 NLCG steps per iteration"
        else:
            r64, _ = B.run(1, 50, 150, "fp64")
            target = r64[-1][3]
            rmx, _ = B.run(1, 50, 150, "mixed", -1)
            rmxp, _ = B.run(1, 50, 150, "mixed", -1, fp64_arith="paired")
            r64p, _ = B.run(1, 50, 150, "fp64", fp64_arith="paired")
            work = "single-component GL 64x64 dx=0.5, 16 images, mode L, 50 NLCG steps per iteration"

        def t_to(rec):
            if rec is None:
                return None
            return B.time_within([x[0] for x in rec], [x[3] for x in rec], target, 1e-6)
        ttb = {"quantity": "F_end - F_0 within 1e-6 of the converged FP64 value",
               "workload": work, "target": target,
               "fp64_s": t_to(r64),                 # IEEE double throughout
               "mixed_s": t_to(rmx),                # FP32 until the end states plateau, then IEEE double
               "mixed_paired_s": t_to(rmxp),        # FP32, then paired (float-float) FP64
               "fp64_paired_s": t_to(r64p),         # paired FP64 throughout
               "mixed_fp32_iterations": sum(1 for x in rmxp if x[4] == "fp32"),
               "ends_fp64": r64[-1][3], "ends_mixed": rmxp[-1][3],
               "barrier_fp64": r64[-1][1], "barrier_mixed": rmxp[-1][1]}
        if ttb["fp64_s"] and ttb["mixed_paired_s"]:
            ttb["speedup_mixed_vs_fp64"] = ttb["fp64_s"] / ttb["mixed_paired_s"]
        ttb["ends_rel_err_mixed"] = abs(ttb["ends_mixed"] - target) / abs(target)

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
            "cpu_baseline": cpu, "clocks": clk.summary(), "time_to_end_state": ttb,
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
    ap.add_argument("--no-ttb", action="store_true", help="skip the time-to-converged-end-state leg")
    ap.add_argument("--ttb-config", type=int, choices=(1, 2), default=2,
                    help="workload of that leg: 2 (the 256x256 mixed-precision string, about 2.5 minutes) "
                         "or 1 (64x64, seconds)")
    args = ap.parse_args(argv)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
