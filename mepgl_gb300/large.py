"""The large workload: a 2048x2048 two-component string of 128 images.

q1 = 1, q2 = 0.5, delta = 0.1, eta = 0, gamma = 0.3, H = 1.1, dx = 0.25,
superconducting domain a disk of radius 1000 lattice units, Meissner to one
composite vortex 20 units inside the rim (built on the device,
mepgl_gb300.workloads.config5_device).  The FP32 state (x, g, d, two
buffers each) takes 77 GB, the FP64 state 155 GB, inside 180 GB.

Reports, per precision, the NLCG step time (CUDA events on the context's
stream), the site·image throughput and the HBM rate of each pass in
algorithmic bytes (k_grad 5S + M, k_dir_poly 4S + M per site·image).

``--barrier B``: time to barrier in the mixed pipeline.  A string phase of B
outer iterations (mode L: linear reparametrization + ``--relax`` NLCG steps,
exact line polynomial and search) in FP32, then image 0 refined to its
minimum and the interior energy maximum to an index-1 saddle in IEEE FP64
(mepgl_gb300.saddle.refine_barrier).  Only images 0, k - 1, k, k + 1 leave the
device string (a device-to-device copy); the FP32 string is freed before the
refinement.  Reports the string-phase time, the refinement trace, the
barrier, |g| at both points and the lowest curvature at the saddle, and the
string phase an IEEE FP64 string would take at the measured FP64 step time.

    python -m mepgl_gb300.large [--n 2048] [--images 128] [--steps 6] [--fp64-steps 2]
                                [--barrier 300 --relax 10]
"""
from __future__ import annotations

import argparse
import json


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--images", type=int, default=128)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--no-paired", action="store_true", help="skip the paired (float-float) FP64 leg")
    ap.add_argument("--barrier", type=int, default=0, help="string-phase outer iterations of the barrier leg (0: off)")
    ap.add_argument("--relax", type=int, default=10)
    ap.add_argument("--g-tol", type=float, default=1e-8)
    ap.add_argument("--max-newton", type=int, default=40)
    a = ap.parse_args(argv)
    import torch
    from . import native, workloads
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    units = a.n * a.n * a.images
    out = dict(workload="two-component GL %dx%d dx=0.25, %d images, disk domain" % (a.n, a.n, a.images),
               site_images=units)
    legs = [("fp32", "fp32", a.steps, torch.float32, native.FP64_NATIVE),
            ("fp64", "fp64", a.fp64_steps, torch.float64, native.FP64_NATIVE)]
    if not a.no_paired:
        legs.append(("fp64_paired", "fp64", a.fp64_steps, torch.float64, native.FP64_PAIRED))
    for key, prec, steps, tdt, arith in legs:
        if steps <= 0:
            continue
        prob, (fa, f1, f2) = workloads.config5_device(a.n, a.images, dtype=tdt)
        ctx = native.StringContext(prob, a.images, prec, stream=stream.cuda_stream, line_polynomial=native.POLY_EXACT,
                                   fp64_arith=arith)
        torch.cuda.synchronize()
        ctx.set_state_device(fa.data_ptr(), f1.data_ptr(), f2.data_ptr())
        ctx.synchronize()
        del fa, f1, f2
        torch.cuda.empty_cache()
        ctx.nlcg_steps(2)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.nlcg_steps(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        mg, md = ctx.profile_passes(2)
        S = 6 * (4 if prec == "fp32" else 8)
        bg, bd = (5 * S + 2) * units, (4 * S + 2) * units
        out[key] = dict(ms_per_step=ms, value=units / (ms / 1e3), unit="site·image/s",
                         k_grad=dict(ms=mg, gbs=bg / mg / 1e6), k_dir_poly=dict(ms=md, gbs=bd / md / 1e6),
                         step_gbs=(bg + bd) / ms / 1e6, device_gb=torch.cuda.mem_get_info()[1] / 1e9 -
                         torch.cuda.mem_get_info()[0] / 1e9)
        ctx.close()
        torch.cuda.empty_cache()
    if a.barrier > 0:
        out["time_to_barrier"] = barrier_leg(a, stream)
        if "fp64" in out:
            out["time_to_barrier"]["fp64_string_phase_estimate_s"] = \
                a.barrier * a.relax * out["fp64"]["ms_per_step"] / 1e3
    print(json.dumps(out))


def barrier_leg(a, stream) -> dict:
    import time

    import torch

    from . import native, saddle, workloads
    from .problem import StringState
    prob, (fa, f1, f2) = workloads.config5_device(a.n, a.images, dtype=torch.float32)
    ctx = native.StringContext(prob, a.images, "fp32", stream=stream.cuda_stream, line_polynomial=native.POLY_EXACT,
                               line_search=native.LS_EXACT, spline=native.SPLINE_FMM)
    ctx.set_state_device(fa.data_ptr(), f1.data_ptr(), f2.data_ptr())
    ctx.synchronize()
    t0 = time.perf_counter()
    trace = []
    for it in range(a.barrier):
        ctx.loop_iteration("L", a.relax)
        if (it + 1) % 10 == 0 or it + 1 == a.barrier:
            fe = ctx.compute_free_energy()
            trace.append((time.perf_counter() - t0, float(fe.max() - fe[0]), "string"))
    fe = ctx.compute_free_energy()
    k = saddle.seed_image(fe)
    ctx.get_state_device(fa.data_ptr(), f1.data_ptr(), f2.data_ptr())
    ctx.synchronize()
    idx = [0, k - 1, k, k + 1]
    sub = StringState(a=fa[idx].double().cpu().numpy(), psi_1=f1[idx].double().cpu().numpy(),
                      psi_2=f2[idx].double().cpu().numpy())
    ctx.close()
    del fa, f1, f2
    torch.cuda.empty_cache()
    t_string = time.perf_counter() - t0
    r = saddle.refine_barrier(prob, sub, fe[idx], g_tol=a.g_tol, max_newton=a.max_newton, t0=t0, adjoint=False,
                              stream=stream.cuda_stream)
    trace += [(t, b, "refine") for t, b, _, _ in r.trace]
    return dict(schedule="FP32 string, IEEE FP64 refinement", string_iterations=a.barrier, relax=a.relax,
                seed_image=k, string_barrier=float(fe.max() - fe[0]), string_s=t_string,
                refine_s=trace[-1][0] - t_string, total_s=trace[-1][0], barrier=r.barrier,
                energies=list(r.energies), g_norms=[x["g_norm"] for x in r.reports],
                min_curvature=r.reports[1]["min_curvature"], is_saddle=r.is_saddle, converged=r.converged,
                newton=len(r.trace) - 1, cg_iterations=list(r.cg_iterations),
                preconditioned=bool(r.reports[1]["preconditioned"]),
                trace=[(round(t, 3), b, ph) for t, b, ph in trace])


if __name__ == "__main__":
    main()
