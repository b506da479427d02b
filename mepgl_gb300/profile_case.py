"""Small, self-contained NLCG run for profiler captures.

    python -m mepgl_gb300.profile_case [--precision fp32|fp64] [--n 256] [--images 64] [--steps 4] [--fused]

Builds the two-component benchmark string (default: the full 256x256, 64
image workload, ~0.6 GB of device state in FP32 -- larger than L2, small for
a profiler), then runs ``--steps`` NLCG steps launched pass by pass (no CUDA
graph), so a capture with ``-k regex:k_grad -s <n> -c 1`` sees few launches
before the one it records.  Prints the per-pass CUDA-event times.

``--fused``: instead, two ``mepgl_nlcg_steps`` calls of ``--steps`` steps
each, which a build with fused FP32 steps runs as two persistent launches
(a capture with ``-k regex:k_nlcg_s -s 1 -c 1`` records the second); prints
the second call's milliseconds per step.

``--reparam linear|cubic``: instead, ``--steps`` reparametrization events
(``mepgl_redistribute`` with the image count kept: arc lengths of the fields
and of B, J, the plan, one resample launch per field, the status check), one
warm-up event first; prints milliseconds per event and the HBM rate over its
algorithmic bytes: x read three times (two arc lengths' sources and the
resample) and written once, B and J written and read once, the masks once.
"""
from __future__ import annotations

import argparse
import json


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--precision", default="fp32", choices=("fp32", "fp64"))
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--images", type=int, default=64)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--fp64-arith", choices=("native", "paired"), default="native",
                    help="FP64 NLCG passes in double or in float-float pairs")
    ap.add_argument("--fused", action="store_true", help="whole nlcg_steps calls (one launch each when fused)")
    ap.add_argument("--reparam", choices=("linear", "cubic"), help="time reparametrization events instead")
    a = ap.parse_args(argv)
    from . import native, workloads
    prob, st = workloads.config2(n=a.n, images=a.images)
    ctx = native.StringContext(prob, st.n_images, a.precision, use_graphs=0, line_polynomial=native.POLY_EXACT,
                               fp64_arith=native.FP64_PAIRED if a.fp64_arith == "paired" else native.FP64_NATIVE)
    ctx.set_state(st)
    if a.reparam:
        import torch
        kind = native.REDIST_LINEAR if a.reparam == "linear" else native.REDIST_CUBIC
        ctx.nlcg_steps(2)
        ctx.redistribute(kind)
        ctx.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(a.steps):
            ctx.redistribute(kind)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / a.steps
        rs = 4 if a.precision == "fp32" else 8
        units = a.n * a.n * a.images
        per_unit = 4 * 6 * rs + 2 * 5 * rs + 2   # 4S + B, J (5 reals) out and in + masks
        print(json.dumps({"precision": a.precision, "reparam": a.reparam, "n": a.n, "images": a.images,
                          "events": a.steps, "ms_per_event": ms, "bytes_per_event": units * per_unit,
                          "gbs": units * per_unit / ms / 1e6}))
        return
    if a.fused:
        import time
        ctx.nlcg_steps(a.steps)
        ctx.synchronize()
        t0 = time.perf_counter()
        ctx.nlcg_steps(a.steps)
        ctx.synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / a.steps
        print(json.dumps({"precision": a.precision, "n": a.n, "images": a.images, "steps": a.steps,
                          "kernels": ctx.pass_kernels(), "ms_per_step_host_clock": ms}))
        return
    ms_grad, ms_dir = ctx.profile_passes(a.steps)
    fe = ctx.image_scalars()["fenergy"]
    print(json.dumps({"precision": a.precision, "fp64_arith": a.fp64_arith, "n": a.n, "images": a.images,
                      "steps": a.steps,
                      "ms_grad": ms_grad, "ms_dir_poly": ms_dir, "energy0": float(fe[0])}))


if __name__ == "__main__":
    main()
