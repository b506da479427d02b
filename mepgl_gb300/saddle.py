"""Barrier of a relaxed string from refined stationary points.

The reference reports the barrier of a string as dF = max_n F_n - F_0
(mepgl/post.py:188): the largest image energy of the relaxed string.  That
value depends on the image count and on how many NLCG steps run between
reparametrizations, and it does not converge to 1e-6.  Here the relaxed
string only seeds a refinement (mepgl_refine_stationary, IEEE double):

* image 0, the initial end state, is refined to its minimum;
* the interior image of largest energy is refined to an index-1 saddle,
  starting its min-mode search from the chord tangent x_{k+1} - x_{k-1};

and the barrier is dF* = F(saddle) - F(minimum), a property of the energy
landscape that converges quadratically with the refinement.

    python -m mepgl_gb300.saddle --config 1 --relax 1 --iterations 600
"""
from __future__ import annotations

import argparse
import json
import time
from dataclasses import dataclass, field

import numpy as np

from . import native
from .problem import StringState


@dataclass
class BarrierResult:
    barrier: float                       # F(saddle) - F(minimum)
    energies: tuple                      # (F(minimum), F(saddle))
    seed_image: int                      # string image the saddle search started from
    string_barrier: float                # max_n F_n - F_0 of the seeding string
    reports: list
    trace: list = field(default_factory=list)   # (seconds, barrier, |g| min, |g| saddle) per Newton iteration
    state: StringState | None = None     # refined [minimum, saddle] fields
    dbarrier_dH: float | None = None     # envelope theorem: dF/dH(saddle) - dF/dH(minimum)
    cg_iterations: tuple = (0, 0)        # CG iterations over all calls (minimum, saddle)

    @property
    def converged(self) -> bool:
        return all(r["converged"] for r in self.reports)

    @property
    def is_saddle(self) -> bool:
        """The refined point has a negative curvature (else the search fell into a minimum)."""
        return self.reports[1]["min_curvature"] < 0


def seed_image(fenergy) -> int:
    """Interior image of largest energy (the string's saddle estimate)."""
    fe = np.asarray(fenergy, float)
    if fe.size < 3:
        raise ValueError("need at least 3 images to seed a saddle")
    return 1 + int(np.argmax(fe[1:-1]))


def seed_state(state: StringState, k: int):
    """Fields of [image 0, image k] in float64 and the chord tangent of image k."""
    def pick(f):
        return None if f is None else np.ascontiguousarray(f[[0, k]], np.float64)

    def chord(f):
        if f is None:
            return None
        t = np.zeros((2,) + f.shape[1:])
        t[1] = np.asarray(f[k + 1], np.float64) - np.asarray(f[k - 1], np.float64)
        return t
    sub = StringState(a=pick(state.a), psi_1=pick(state.psi_1), psi_2=pick(state.psi_2))
    mode = StringState(a=chord(state.a), psi_1=chord(state.psi_1), psi_2=chord(state.psi_2))
    return sub, mode


def refine_barrier(prob, state: StringState, fenergy, g_tol: float = 1e-8, max_newton: int = 40,
                   stream=None, keep_state: bool = False, adjoint: bool = True, t0: float | None = None,
                   **options) -> BarrierResult:
    """Refine the string's image 0 to a minimum and its interior maximum to a
    saddle; one library call per Newton iteration, so that the barrier is
    traced (``t0``: perf_counter origin of the trace times)."""
    fe = np.asarray(fenergy, float)
    k = seed_image(fe)
    sub, mode = seed_state(state, k)
    kinds = [native.STATIONARY_MINIMUM, native.STATIONARY_SADDLE]
    t0 = time.perf_counter() if t0 is None else t0
    with native.StringContext(prob, 2, "fp64", stream=stream) as ctx:
        ctx.set_state(sub)
        reps = ctx.refine_stationary(kinds, mode, max_newton=0, g_tol=g_tol, **options)
        trace = [(time.perf_counter() - t0, reps[1]["energy"] - reps[0]["energy"], reps[0]["g_norm"],
                  reps[1]["g_norm"])]
        cg = [0, 0]
        for _ in range(max_newton):
            if all(r["converged"] for r in reps):
                break
            reps = ctx.refine_stationary(kinds, None, max_newton=1, g_tol=g_tol, **options)
            cg = [c + r["cg_iterations"] for c, r in zip(cg, reps)]
            trace.append((time.perf_counter() - t0, reps[1]["energy"] - reps[0]["energy"], reps[0]["g_norm"],
                          reps[1]["g_norm"]))
        res = BarrierResult(barrier=reps[1]["energy"] - reps[0]["energy"],
                            energies=(reps[0]["energy"], reps[1]["energy"]), seed_image=k,
                            string_barrier=float(fe.max() - fe[0]), reports=reps, trace=trace,
                            cg_iterations=tuple(cg))
        if adjoint:
            adj = ctx.param_adjoint()
            res.dbarrier_dH = float(adj[1, 0] - adj[0, 0])
        if keep_state:
            res.state = ctx.get_state()
    return res


def relax_string(cfg: int, relax: int, iterations: int, precision: str = "fp64", mode: str = "L", **wl):
    """Relaxed string of a workload (exact line polynomial and search, FMM spline)."""
    from . import workloads
    prob, st = {1: workloads.config1, 2: workloads.config2}[cfg](**wl)
    c = native.StringContext(prob, st.n_images, precision, line_polynomial=native.POLY_EXACT,
                             line_search=native.LS_EXACT, spline=native.SPLINE_FMM)
    c.set_state(st)
    for _ in range(iterations):
        c.loop_iteration(mode, relax)
    fe = c.compute_free_energy()
    out = c.get_state()
    c.close()
    return prob, out, fe


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--relax", type=int, default=1)
    ap.add_argument("--iterations", type=int, default=600)
    ap.add_argument("--precision", choices=("fp32", "fp64"), default="fp64")
    ap.add_argument("--g-tol", type=float, default=1e-8)
    ap.add_argument("--max-newton", type=int, default=40)
    ap.add_argument("--gauge-degree", type=int, default=-1)
    a = ap.parse_args(argv)
    t = time.perf_counter()
    prob, st, fe = relax_string(a.config, a.relax, a.iterations, a.precision)
    t_string = time.perf_counter() - t
    r = refine_barrier(prob, st, fe, g_tol=a.g_tol, max_newton=a.max_newton, gauge_degree=a.gauge_degree)
    print(json.dumps(dict(config=a.config, string_s=t_string, refine_s=r.trace[-1][0], barrier=r.barrier,
                          string_barrier=r.string_barrier, seed_image=r.seed_image, converged=r.converged,
                          is_saddle=r.is_saddle, dbarrier_dH=r.dbarrier_dH, reports=r.reports, trace=r.trace)))


if __name__ == "__main__":
    main()
