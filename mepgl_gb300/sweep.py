"""Parameter sweep in one context: many strings of uneven size per launch.

The reference runs a sweep as one process per string (mepgl/batch_run.py);
here the 64 strings of the batching workload share one context:
single-component GL, N ~ U{96..384}, F ~ U{24..64}, H ~ U[0.5, 1.2],
kappa ~ U[1, 4], dx = 0.5, Meissner to one vortex (seeded per string,
mepgl_gb300.workloads.config4_string).  One step = one NLCG iteration of
every string; the throughput is the aggregate site·image updates per second,
timed with CUDA events on the context's stream (FP32 bulk relaxation).

After the timed steps the per-string barrier error of the FP32 fields is
reported: the barrier max_n F_n - F_0 of the same state evaluated with the
FP32 and with the FP64 energy kernel; ``--polish P`` then runs P FP64 outer
iterations (mode L, ``--relax`` steps each).

    python -m mepgl_gb300.sweep [--strings 64] [--steps 20] [--warmup 3] [--polish 0]
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
    b = native.StringBatch(problems, [st.n_images for st in states], precision, stream=stream,
                           line_polynomial=native.POLY_EXACT, **options)
    for k, st in enumerate(states):
        b.set_string_state(k, st)
    units = sum(p.nx * p.ny * st.n_images for p, st in zip(problems, states))
    return b, problems, states, units


def barrier_errors(b, n_strings: int):
    """Per-string barrier of the current fields, FP32 vs FP64 evaluation (switches b to FP64)."""
    d32 = [float(np.max(e) - e[0]) for e in (b.string_free_energy(k) for k in range(n_strings))]
    b.set_precision("fp64")
    d64 = [float(np.max(e) - e[0]) for e in (b.string_free_energy(k) for k in range(n_strings))]
    return [abs(x - y) / max(abs(y), 1e-300) for x, y in zip(d32, d64)], d64


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--strings", type=int, default=64)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--polish", type=int, default=0)
    ap.add_argument("--relax", type=int, default=10)
    a = ap.parse_args(argv)
    import torch
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    t0 = time.perf_counter()
    b, problems, states, units = build_batch(a.strings, stream=stream.cuda_stream)
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
    errs, d64 = barrier_errors(b, a.strings)
    out = dict(workload="parameter sweep: %d single-component strings, N 96..384, F 24..64" % a.strings,
               strings=a.strings, site_images_per_step=units, steps=a.steps, ms_per_step=ms / a.steps,
               value=units * a.steps / (ms / 1e3), unit="site·image/s", gpu_launches=launches,
               launches_per_step=launches / a.steps, setup_s=t_build,
               barrier_fp32_vs_fp64_rel_err=dict(max=max(errs), median=float(np.median(errs))))
    if a.polish:
        t1 = time.perf_counter()
        for _ in range(a.polish):
            b.loop_iteration("L", a.relax)
        b.synchronize()
        out["polish"] = dict(iterations=a.polish, relax=a.relax, wall_s=time.perf_counter() - t1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
