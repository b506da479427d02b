"""Precision schedules and barrier convergence.

The barrier of a string is ``dF = max_n F_n - F_0`` (mepgl/post.py:188).
:func:`relax_string` runs outer iterations of the reference's loop() (one
reparametrization + ``relax`` NLCG steps per iteration) and records dF after
each, evaluated with the free-energy kernel on the current state.

Mixed precision (FP32 bulk, FP64 polish): the fields start in FP32 -- every
reduction and the beta / step scalars are FP64 anyway -- and switch to FP64
when the FP32 barrier has stopped improving (relative change below
``switch_tol`` over ``window`` iterations); after the switch the NLCG history
restarts and the run continues in FP64.  On GB300 an FP32 iteration costs a
fifteenth of an FP64 one, so the bulk of the descent is nearly free.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import native


def barrier(fenergy) -> float:
    fe = np.asarray(fenergy, float)
    return float(np.max(fe) - fe[0])


@dataclass
class Trace:
    t: list = field(default_factory=list)          # seconds since start
    dF: list = field(default_factory=list)
    iteration: list = field(default_factory=list)
    precision: list = field(default_factory=list)
    switched_at: int | None = None

    def time_to(self, target: float, rtol: float) -> float | None:
        """First time after which |dF - target| <= rtol |target| holds for good."""
        ok = [abs(d - target) <= rtol * abs(target) for d in self.dF]
        for k in range(len(ok)):
            if all(ok[k:]):
                return self.t[k]
        return None


def relax_string(ctx: native.StringContext, iterations: int, mode: str = "L", relax: int = 10,
                 schedule: str = "fp64", switch_tol: float = 1e-6, window: int = 5, target: float | None = None,
                 rtol: float = 1e-6, stable_tol: float | None = None, trace: Trace | None = None) -> Trace:
    """Run up to ``iterations`` outer iterations.

    schedule: "fp64" / "fp32" keep the context precision; "mixed" starts in
    whatever precision the context has (FP32) and switches to FP64 on the
    plateau.  Stops early when ``target`` is given and dF is within ``rtol``
    of it (FP64 only), or when ``stable_tol`` is given and dF changed by less
    than that (relative) over ``window`` FP64 iterations.
    """
    tr = trace or Trace()
    t0 = time.perf_counter() - (tr.t[-1] if tr.t else 0.0)
    for it in range(iterations):
        ctx.loop_iteration(mode, relax)
        dF = barrier(ctx.compute_free_energy())
        tr.t.append(time.perf_counter() - t0)
        tr.dF.append(dF)
        tr.iteration.append(len(tr.iteration))
        tr.precision.append(ctx.info()["precision"])
        fp64 = tr.precision[-1] == "fp64"
        if schedule == "mixed" and not fp64 and len(tr.dF) > window:
            old = tr.dF[-1 - window]
            if abs(dF - old) <= switch_tol * max(abs(dF), 1e-300):
                ctx.set_precision("fp64")
                tr.switched_at = len(tr.dF)
        if fp64 and target is not None and abs(dF - target) <= rtol * abs(target):
            break
        if fp64 and stable_tol is not None and len(tr.dF) > window:
            ref = tr.dF[-1 - window]
            if tr.precision[-1 - window] == "fp64" and abs(dF - ref) <= stable_tol * max(abs(dF), 1e-300):
                break
    return tr
