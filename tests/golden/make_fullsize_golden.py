#!/usr/bin/env python3
"""Write tests/golden/ref_cfg1_full.json: the reference's own kernels
(host-compiled from the reference tree by oracle/ref_build.py, driven by
oracle/ref_driver.cpp) on the plain-method string at its full size:
64x64, dx = 0.5, 16 images, single component, FP64, seeded input
mepgl_gb300.workloads.config1() (regenerated by the tests from its seed, so
only outputs are stored):

* the per-image free energies of the input (computeFreeEnergy);
* loop() in mode L, 5 outer iterations of 10 NLCG steps (reference line
  search and polynomial): per-iteration energies, final energies, steps;
* loop() in mode C (cubic reparametrization every 10 steps, the method the
  workload names; the reference compiles its cubic only in FP32 builds, the
  host variant keeps it in double), 3 outer iterations of 10 steps.

Requires the reference sources ($MEPGL_REFERENCE or ../reference).  Run from
the repository root:  python tests/golden/make_fullsize_golden.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from mepgl_gb300 import workloads as W  # noqa: E402
from oracle import refkernels  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def main():
    prob, st = W.config1()
    R = refkernels.load_ref(prob.nx, prob.dx, 1, "f64", False)
    p2 = np.zeros_like(st.psi_1)
    out = dict(workload="config1 64x64 dx=0.5 16 images FP64 (workloads.config1 seed 1001)",
               fenergy=[float(v) for v in R.free_energy(prob, st.a, st.psi_1, p2)])
    for mode, iters, relax in (("L", 5, 10), ("C", 3, 10)):
        r = R.loop(prob, st.a.copy(), st.psi_1.copy(), p2.copy(), mode, iters, relax, history=True)
        fe = np.asarray(r["fenergy"], float)
        out[f"loop_{mode}"] = dict(iterations=iters, relax=relax, history=np.asarray(r["history"]).tolist(),
                                   alpha=np.asarray(r["alpha"]).tolist(),
                                   final_energy=[float(v) for v in R.free_energy(prob, r["a"], r["psi_1"], p2)],
                                   barrier=float(fe.max() - fe[0]))
    path = os.path.join(OUT, "ref_cfg1_full.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
