#!/usr/bin/env python3
"""Generate the golden vectors in tests/golden/ from the reference's own kernels.

The reference (maiani/mepgl) ships no tests and no fixtures, so its parity
vectors are produced here by running its own ``__global__`` kernels on the
CPU (``oracle/_ref``, host-compiled from the reference tree by
``oracle/ref_build.py``; requires the reference sources, which are only
present where the fixtures are generated).  Each ``.npz`` holds the seeded
inputs and the reference outputs, so the tests that read them need neither
the reference nor this script.

Run from the repository root:  ``python tests/golden/make_golden.py``
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from mepgl_gb300 import workloads as W  # noqa: E402
from mepgl_gb300.problem import PARAM_NAMES  # noqa: E402
from oracle import refkernels  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def _problem_arrays(prob):
    d = {name: getattr(prob, name) for name in PARAM_NAMES}
    d.update(comp_domain=prob.comp_domain, sc_domain=prob.sc_domain,
             scalars=np.array([prob.dx, prob.q_1, prob.q_2, prob.eta, prob.gamma, prob.delta]),
             flags=np.array([prob.nx, prob.ny, int(prob.multicomponent), int(prob.thin_film)]))
    return d


def make_case(name, prob, st, images_new=(None,), loops=(("S", 3, 3), ("L", 3, 3), ("C", 3, 3), ("M", 2, 3)),
              seed=0):
    comps = prob.ncomp
    R = refkernels.load_ref(prob.nx, prob.dx, comps, "f64", prob.thin_film)
    rng = np.random.default_rng(seed)
    out = _problem_arrays(prob)
    p2 = st.psi_2 if comps == 2 else np.zeros_like(st.psi_1)
    out.update(a=st.a, psi_1=st.psi_1, psi_2=p2)
    out["fenergy"] = R.free_energy(prob, st.a, st.psi_1, p2)
    ga, g1, g2 = R.gradient(prob, st.a, st.psi_1, p2)
    out.update(grad_a=ga, grad_psi_1=g1, grad_psi_2=g2)
    # a descent-ish direction: -gradient plus a little noise
    da = -ga + 0.01 * rng.standard_normal(ga.shape)
    d1 = -g1 + 0.01 * rng.standard_normal(g1.shape)
    d2 = (-g2 + 0.01 * rng.standard_normal(g2.shape)) if comps == 2 else np.zeros_like(g2)
    out.update(dir_a=da, dir_psi_1=d1, dir_psi_2=d2)
    fe, poly = R.polynomial(prob, st.a, st.psi_1, p2, da, d1, d2)
    out.update(poly_energy=fe, poly=poly, alpha=R.line_search(fe, poly))
    b, j1, j2 = R.jb(prob, st.a, st.psi_1, p2)
    out.update(b=b, j_1=j1, j_2=j2)
    out["s"] = R.arc_length(st.a, st.psi_1, p2)
    out["s_jb"] = R.arc_length_jb(b, j1, j2)
    F = st.a.shape[0]
    for fnew in (F, F + 3):
        out[f"linear_{fnew}"] = R.redistribute(out["s_jb"], st.psi_1, fnew)
        out[f"cubic_{fnew}"] = R.redistribute(out["s_jb"], st.psi_1, fnew, cubic=True)
    for mode, iters, relax in loops:
        r = R.loop(prob, st.a, st.psi_1, p2, mode, iters, relax, history=True)
        for k in ("a", "psi_1", "psi_2", "fenergy", "alpha", "g_norm2", "s", "s_jb", "history"):
            out[f"loop_{mode}_{k}"] = r[k]
        out[f"loop_{mode}_cfg"] = np.array([iters, relax])
    path = os.path.join(OUT, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) // 1024} KiB)")


def main():
    rng = np.random.default_rng(20261203)
    p = W.random_problem(rng, n=16, multicomponent=False)
    make_case("ref_c1_masked", p, W.random_state(rng, p, images=5), seed=1)
    p = W.random_problem(rng, n=16, multicomponent=True)
    make_case("ref_c2_couplings", p, W.random_state(rng, p, images=5), seed=2)
    p = W.random_problem(rng, n=16, multicomponent=True, thin_film=True)
    make_case("ref_c2_thinfilm", p, W.random_state(rng, p, images=4), seed=3)
    p = W.random_problem(rng, n=16, multicomponent=True, uniform=False)
    make_case("ref_c2_persite", p, W.random_state(rng, p, images=4), seed=4)
    # configuration-1 physics at 32x32, 8 images, several L/C iterations
    prob, st = W.config1(n=32, images=8)
    make_case("ref_cfg1_n32", prob, st, loops=(("L", 3, 10), ("C", 2, 10), ("S", 2, 10)), seed=5)
    # two-component configuration-2 physics at 24x24, 6 images
    prob, st = W.config2(n=24, images=6)
    make_case("ref_cfg2_n24", prob, st, loops=(("L", 2, 6), ("S", 2, 6)), seed=6)


if __name__ == "__main__":
    main()
