"""Barrier and end-state convergence of the string method on the GPU.

One run = ``iterations`` outer iterations of loop() in mode L or C (one
reparametrization + ``relax`` NLCG steps, mepgl/src/mepgl.cu:148-303) on a
seeded workload, recording after each iteration the wall time, the barrier
estimate dF = max_n F_n - F_0 (mepgl/post.py:188), its argmax image and the
end-state difference F_{F-1} - F_0.  Schedules:

* ``fp64`` / ``fp32``: one precision throughout;
* ``mixed``: FP32 for ``--fp32-iterations`` outer iterations, then FP64.

The summary gives the final values, the spread (max - min) of each quantity
over the final tenth of the run and, when ``--target-ends`` is given, the
time after which F_{F-1} - F_0 stays within ``--rtol`` of it.

    python -m mepgl_gb300.barrier --config 2 --relax 100 --iterations 250 \
        --schedule fp64 --out barrier_c2_fp64.json
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import native, workloads


def _workload(cfg: int):
    if cfg == 1:
        return workloads.config1()
    if cfg == 2:
        return workloads.config2()
    raise SystemExit("--config must be 1 or 2")


def time_within(t, v, target, rtol):
    """First time after which |v - target| <= rtol |target| for the rest of the run."""
    ok = np.abs(np.asarray(v) - target) <= rtol * abs(target)
    bad = np.nonzero(~ok)[0]
    k = 0 if bad.size == 0 else bad[-1] + 1
    return None if k >= len(t) else float(t[k])


def run(cfg: int, relax: int, iterations: int, schedule: str = "fp64", fp32_iterations: int = -1,
        mode: str = "L", switch_window: int = 10, switch_tol: float = 1e-5, fp64_arith: str = "native"):
    """fp32_iterations < 0 (mixed): switch to FP64 once F_{F-1} - F_0 has
    changed by at most switch_tol (relative) over switch_window iterations,
    i.e. when FP32 has reached its resolution."""
    prob, st = _workload(cfg)
    prec = "fp32" if schedule in ("fp32", "mixed") else "fp64"
    c = native.StringContext(prob, st.n_images, prec, line_polynomial=native.POLY_EXACT,
                             line_search=native.LS_EXACT, spline=native.SPLINE_FMM,
                             fp64_arith=native.FP64_PAIRED if fp64_arith == "paired" else native.FP64_NATIVE)
    c.set_state(st)
    c.synchronize()
    rec = []
    t0 = time.perf_counter()
    switched = schedule != "mixed"
    for it in range(iterations):
        if not switched:
            if fp32_iterations >= 0:
                switched = it == fp32_iterations
            elif len(rec) > switch_window:
                e_now, e_old = rec[-1][3], rec[-1 - switch_window][3]
                switched = abs(e_now - e_old) <= switch_tol * abs(e_now)
            if switched:
                c.set_precision("fp64")
        c.loop_iteration(mode, relax)
        fe = c.compute_free_energy()
        rec.append((time.perf_counter() - t0, float(fe.max() - fe[0]), int(fe.argmax()), float(fe[-1] - fe[0]),
                    c.info()["precision"]))
    # envelope-theorem sensitivities of the final string: dF/dH of the max
    # image and of the last image, minus that of image 0 (exact where the
    # images are stationary; the max image of a discrete string is not)
    adj = c.param_adjoint()
    k = int(np.argmax(c.compute_free_energy()))
    sens = dict(dbarrier_dH=float(adj[k, 0] - adj[0, 0]), dends_dH=float(adj[-1, 0] - adj[0, 0]))
    c.close()
    return rec, sens


def time_to_barrier(cfg: int, schedule: str = "fp64", relax: int = 10, max_string: int = 300, window: int = 5,
                    plateau: float | None = None, g_tol: float = 1e-8, max_newton: int = 40, **refine_options):
    """One timed run of the barrier protocol on a workload.

    String phase: outer iterations of loop() in mode L (one linear
    reparametrization + ``relax`` NLCG steps, exact line polynomial and
    search) in the schedule's precision -- ``fp64`` IEEE double, ``fp64_paired``
    float-float NLCG passes, ``mixed`` FP32 -- for ``max_string`` iterations,
    or, with ``plateau`` given, until the string's interior energy maximum stays
    on the same image for ``window`` iterations and its estimate
    max_n F_n - F_0 changes by at most ``plateau`` (relative) over them (on the
    256x256 string the estimate wanders by about 5 % for hundreds of
    iterations, so the bench uses the fixed budget).  Refinement: image 0 to
    its minimum and that image to an index-1 saddle in IEEE double
    (saddle.refine_barrier) to |g| <= g_tol.

    Returns a dict with the trace [(seconds, barrier estimate, phase)] --
    the string's estimate during the string phase, F(saddle) - F(minimum)
    during the refinement -- and the final refined barrier."""
    from . import saddle
    prob, st = _workload(cfg)
    prec = "fp32" if schedule == "mixed" else "fp64"
    arith = native.FP64_PAIRED if schedule == "fp64_paired" else native.FP64_NATIVE
    c = native.StringContext(prob, st.n_images, prec, line_polynomial=native.POLY_EXACT,
                             line_search=native.LS_EXACT, spline=native.SPLINE_FMM, fp64_arith=arith)
    c.set_state(st)
    c.synchronize()
    t0 = time.perf_counter()
    trace, hist = [], []
    for it in range(max_string):
        c.loop_iteration("L", relax)
        fe = c.compute_free_energy()
        k = saddle.seed_image(fe)
        est = float(fe.max() - fe[0])
        trace.append((time.perf_counter() - t0, est, "string"))
        hist.append((k, est))
        if plateau is not None and len(hist) > window:
            ks = {h[0] for h in hist[-window - 1:]}
            if len(ks) == 1 and abs(est - hist[-window - 1][1]) <= plateau * abs(est):
                break
    state = c.get_state()
    fe = c.compute_free_energy()
    c.close()
    t_string = time.perf_counter() - t0
    r = saddle.refine_barrier(prob, state, fe, g_tol=g_tol, max_newton=max_newton, t0=t0, adjoint=False,
                              **refine_options)
    trace += [(t, b, "refine") for t, b, _, _ in r.trace]
    return dict(schedule=schedule, trace=trace, barrier=r.barrier, string_iterations=len(hist),
                string_s=t_string, total_s=trace[-1][0], seed_image=r.seed_image, is_saddle=r.is_saddle,
                converged=r.converged, newton=len(r.trace) - 1, min_curvature=r.reports[1]["min_curvature"],
                g_norms=(r.reports[0]["g_norm"], r.reports[1]["g_norm"]), energies=r.energies)


def summarise(rec, target_ends=None, rtol=1e-6):
    t = np.array([r[0] for r in rec])
    dF = np.array([r[1] for r in rec])
    ends = np.array([r[3] for r in rec])
    k = max(3, len(rec) // 10)
    out = dict(iterations=len(rec), wall_s=float(t[-1]), barrier=float(dF[-1]), argmax=int(rec[-1][2]),
               barrier_spread=float(np.ptp(dF[-k:])), ends=float(ends[-1]), ends_spread=float(np.ptp(ends[-k:])))
    if target_ends is not None:
        out["target_ends"] = target_ends
        out["rtol"] = rtol
        out["time_to_ends_s"] = time_within(t, ends, target_ends, rtol)
    return out


def compare(paths, rtol=1e-6):
    """Time for each saved run to bring F_{F-1} - F_0 within rtol of the first
    run's final value (the first run is the long FP64 reference)."""
    runs = [json.load(open(p)) for p in paths]
    target = runs[0]["trace"][-1][3]
    out = []
    for p, r in zip(paths, runs):
        tr = r["trace"]
        out.append(dict(run=p, schedule=r["summary"]["schedule"], target_ends=target, rtol=rtol,
                        time_to_ends_s=time_within([x[0] for x in tr], [x[3] for x in tr], target, rtol),
                        wall_s=tr[-1][0], final_barrier=tr[-1][1]))
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--compare", nargs="+", default=None,
                    help="saved runs (first = reference); print each run's time to its end-state value")
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--relax", type=int, default=10)
    ap.add_argument("--iterations", type=int, default=1000)
    ap.add_argument("--schedule", choices=("fp64", "fp32", "mixed"), default="fp64")
    ap.add_argument("--fp32-iterations", type=int, default=-1,
                    help="mixed: outer iterations in FP32 (< 0: until F_end - F_0 plateaus)")
    ap.add_argument("--switch-window", type=int, default=10)
    ap.add_argument("--switch-tol", type=float, default=1e-5)
    ap.add_argument("--fp64-arith", choices=("native", "paired"), default="native",
                    help="FP64 NLCG passes in double or in float-float pairs")
    ap.add_argument("--mode", choices=("L", "C"), default="L")
    ap.add_argument("--target-ends", type=float, default=None)
    ap.add_argument("--rtol", type=float, default=1e-6)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    if a.compare:
        for row in compare(a.compare, a.rtol):
            print(json.dumps(row))
        return
    rec, sens = run(a.config, a.relax, a.iterations, a.schedule, a.fp32_iterations, a.mode, a.switch_window,
                    a.switch_tol, a.fp64_arith)
    s = summarise(rec, a.target_ends, a.rtol)
    s.update(sens)
    fp32_its = sum(1 for r in rec if r[4] == "fp32")
    s.update(config=a.config, relax=a.relax, schedule=a.schedule, fp32_iterations=fp32_its, mode=a.mode,
             fp64_arith=a.fp64_arith)
    print(json.dumps(s))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(dict(summary=s, trace=rec), f)


if __name__ == "__main__":
    main()
