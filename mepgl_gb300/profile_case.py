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
    a = ap.parse_args(argv)
    from . import native, workloads
    prob, st = workloads.config2(n=a.n, images=a.images)
    ctx = native.StringContext(prob, st.n_images, a.precision, use_graphs=0, line_polynomial=native.POLY_EXACT,
                               fp64_arith=native.FP64_PAIRED if a.fp64_arith == "paired" else native.FP64_NATIVE)
    ctx.set_state(st)
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
