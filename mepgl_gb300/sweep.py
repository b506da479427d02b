"""Parameter sweep in one context: many strings of uneven size per launch.

The reference runs a sweep as one process per string (mepgl/batch_run.py:9-21);
here the 64 strings of the batching workload share one context:
single-component GL, N ~ U{96..384}, F ~ U{24..64}, H ~ U[0.5, 1.2],
kappa ~ U[1, 4], dx = 0.5, Meissner to one vortex (seeded per string,
mepgl_gb300.workloads.config4_string).  One step = one NLCG iteration of
every string; the throughput is the aggregate site-image updates per second,
timed with CUDA events on the context's stream (FP32 bulk relaxation).

Schedule (``--bulk B --polish P``): B outer iterations of loop() in mode L
(``--relax`` NLCG steps each) for all strings together in FP32, then the whole
batch converted to FP64 and P more outer iterations.  Per-string barriers
(``--refine K``, the first K strings): each string's image 0 and interior
energy maximum are refined to a minimum and an index-1 saddle in IEEE FP64
(mepgl_gb300.saddle), once from the mixed schedule's string and once from the
same string relaxed in FP64 throughout (B + P iterations); the barrier error
of the mixed schedule is the relative difference of the two refined
barriers.  Each row carries both refinements' final |g| (minimum, saddle)
and Newton counts: a barrier difference means something only where both
converged.  Strings whose energy profile has no interior saddle near the
seed are reported as such.

    python -m mepgl_gb300.sweep [--strings 64] [--steps 20] [--warmup 3] [--bulk 50]
                                [--polish 5] [--refine 8]
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def build_batch(n_strings: int, stream=None, precision="fp32", **options):
    from . import native, workloads
    problems, states = [], []
    for s in range(n_strings):
        p, st = workloads.config4_string(s)
        problems.append(p)
        states.append(st)
    opts = dict(line_polynomial=native.POLY_EXACT)
    opts.update(options)
    b = native.StringBatch(problems, [st.n_images for st in states], precision, stream=stream, **opts)
    for k, st in enumerate(states):
        b.set_string_state(k, st)
    units = sum(p.nx * p.ny * st.n_images for p, st in zip(problems, states))
    return b, problems, states, units


def fp64_reference(prob, state, iterations: int, relax: int):
    """The same string relaxed in IEEE FP64 throughout (exact line search, FMM spline)."""
    from . import native
    c = native.StringContext(prob, state.n_images, "fp64", line_polynomial=native.POLY_EXACT,
                             line_search=native.LS_EXACT, spline=native.SPLINE_FMM)
    c.set_state(state)
    for _ in range(iterations):
        c.loop_iteration("L", relax)
    fe = c.compute_free_energy()
    out = c.get_state()
    c.close()
    return out, fe


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--strings", type=int, default=64)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--bulk", type=int, default=50, help="FP32 outer iterations (mode L)")
    ap.add_argument("--polish", type=int, default=5, help="FP64 outer iterations after the FP32 bulk")
    ap.add_argument("--relax", type=int, default=10)
    ap.add_argument("--refine", type=int, default=0, help="per-string refined barriers of the first K strings")
    ap.add_argument("--g-tol", type=float, default=1e-8)
    a = ap.parse_args(argv)
    import torch
    from . import native, saddle
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    t0 = time.perf_counter()
    b, problems, states, units = build_batch(a.strings, stream=stream.cuda_stream, line_search=native.LS_EXACT,
                                             spline=native.SPLINE_FMM)
    t_build = time.perf_counter() - t0
    b.nlcg_steps(max(a.warmup, 1))
    torch.cuda.synchronize()
    l0 = b.info()["kernel_launches"]
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    b.nlcg_steps(a.steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    launches = b.info()["kernel_launches"] - l0
    out = dict(workload="parameter sweep: %d single-component strings, N 96..384, F 24..64" % a.strings,
               strings=a.strings, site_images_per_step=units, steps=a.steps, ms_per_step=ms / a.steps,
               value=units * a.steps / (ms / 1e3), unit="site·image/s", gpu_launches=launches,
               launches_per_step=launches / a.steps, setup_s=t_build, kernels=b.pass_kernels())
    # mixed schedule: FP32 bulk, FP64 polish, all strings in the same launches
    for s_, st in enumerate(states):
        b.set_string_state(s_, st)
    t1 = time.perf_counter()
    for _ in range(a.bulk):
        b.loop_iteration("L", a.relax)
    b.synchronize()
    t_bulk = time.perf_counter() - t1
    b.set_precision("fp64")
    t2 = time.perf_counter()
    for _ in range(a.polish):
        b.loop_iteration("L", a.relax)
    b.synchronize()
    out["schedule"] = dict(bulk_fp32_iterations=a.bulk, polish_fp64_iterations=a.polish, relax=a.relax,
                           bulk_s=t_bulk, polish_s=time.perf_counter() - t2)
    if a.refine:
        rows = []
        for k in range(min(a.refine, a.strings)):
            fe = b.string_free_energy(k)
            st_mixed = b.get_string_state(k)
            row = dict(string=k, n=problems[k].nx, images=states[k].n_images)
            try:
                r_mixed = saddle.refine_barrier(problems[k], st_mixed, fe, g_tol=a.g_tol, adjoint=False,
                                                stream=stream.cuda_stream)
                st64, fe64 = fp64_reference(problems[k], states[k], a.bulk + a.polish, a.relax)
                r_64 = saddle.refine_barrier(problems[k], st64, fe64, g_tol=a.g_tol, adjoint=False,
                                             stream=stream.cuda_stream)
                row.update(barrier_mixed=r_mixed.barrier, barrier_fp64=r_64.barrier,
                           string_barrier_mixed=r_mixed.string_barrier, string_barrier_fp64=r_64.string_barrier,
                           saddle=bool(r_mixed.is_saddle and r_64.is_saddle),
                           converged=bool(r_mixed.converged and r_64.converged),
                           g_mixed=[x["g_norm"] for x in r_mixed.reports],
                           g_fp64=[x["g_norm"] for x in r_64.reports],
                           newton=[len(r_mixed.trace) - 1, len(r_64.trace) - 1],
                           refine_s=r_mixed.trace[-1][0])
                if row["saddle"]:
                    row["rel_err"] = abs(r_mixed.barrier - r_64.barrier) / abs(r_64.barrier)
            except ValueError as e:
                row["error"] = str(e)
            rows.append(row)
            print(json.dumps(row), flush=True)
        errs = [r["rel_err"] for r in rows if "rel_err" in r]
        conv = [r["rel_err"] for r in rows if "rel_err" in r and r["converged"]]
        out["per_string_barrier"] = dict(strings=len(rows), with_saddle=len(errs),
                                         max_rel_err=max(errs) if errs else None,
                                         median_rel_err=float(np.median(errs)) if errs else None,
                                         converged=len(conv), max_rel_err_converged=max(conv) if conv else None,
                                         rows=rows)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
