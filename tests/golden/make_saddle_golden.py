"""Write tests/golden/saddle_cfg1.json: the converged barrier of the plain-method
string (64x64, dx = 0.5, 16 images, single component, H = 0.8), computed on
the CPU with the C oracle only.

1. The seeded initial string (mepgl_gb300.workloads.config1) is relaxed by
   the oracle's loop() in mode L with one NLCG step per reparametrization
   (exact line polynomial and search, FMM spline), 600 iterations.
2. Image 0 is refined to its minimum and the interior image of largest
   energy to an index-1 saddle by oracle/saddle_ref.py (gauge-subspace
   steps, Lanczos min mode, shifted CG), to |g| <= 1e-9.

The record holds the two energies, the barrier, the lowest curvature at the
saddle and dF/dH at both points (oracle parameter adjoint).  It takes several
minutes:  python tests/golden/make_saddle_golden.py
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from mepgl_gb300 import workloads as W  # noqa: E402
from oracle import cref, saddle_ref as SR  # noqa: E402


def main():
    t0 = time.time()
    prob, st = W.config1()
    o = cref.Oracle(prob)
    sv = o.solver(st, ls_mode=cref.LS_EXACT, poly_compat=False)
    for _ in range(600):
        sv.iteration("L", 1, spline=cref.SPLINE_FMM)
    r = sv.get()
    fe = o.energy(r["a"], r["psi_1"])
    k = 1 + int(np.argmax(fe[1:-1]))
    R = SR.Refiner(o)
    x0 = R.pack(r["a"][0:1], r["psi_1"][0:1])
    xk = R.pack(r["a"][k:k + 1], r["psi_1"][k:k + 1])
    tau = R.pack(r["a"][k + 1:k + 2] - r["a"][k - 1:k], r["psi_1"][k + 1:k + 2] - r["psi_1"][k - 1:k])
    xm, rm = R.refine(x0, SR.MINIMUM, g_tol=1e-9)
    xs, rs = R.refine(xk, SR.SADDLE, mode=tau, g_tol=1e-9)
    adj_m = o.param_adjoint(*R.unpack(xm))[0]
    adj_s = o.param_adjoint(*R.unpack(xs))[0]
    neg = R.morse_negatives(xs, tau, 40)
    out = dict(workload="config1 64x64 dx=0.5 16 images, mode L, 1 NLCG step per reparametrization, 600 iterations",
               seed_image=k, string_barrier=float(fe[k] - fe[0]), e_min=rm["energy"], e_saddle=rs["energy"],
               barrier=rs["energy"] - rm["energy"], g_min=rm["g_norm"], g_saddle=rs["g_norm"],
               min_curvature=float(rs["min_curvature"]), negative_ritz=[float(v) for v in neg],
               dF_dH_min=float(adj_m[0]), dF_dH_saddle=float(adj_s[0]),
               dbarrier_dH=float(adj_s[0] - adj_m[0]), seconds=time.time() - t0)
    with open(os.path.join(HERE, "saddle_cfg1.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
