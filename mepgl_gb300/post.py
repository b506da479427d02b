"""Post-processing of a finished simulation: the data part of the
reference's post.py (mepgl/post.py:50-151), computed on the GPU, without the
plots (matplotlib is not a dependency).

    python -m mepgl_gb300.post -s SIMULATION [--inset K]

Reads ``simulations/S/output_data`` (the files the ``mepgl`` executable
writes), loads the string into a context, and writes
``simulations/S/S.npz`` with the reference's keys -- ``fenergy``, ``s_gd``,
``s_ph`` (arc lengths in the field and in the (B, J) metric), ``w_1``,
``w_2`` (winding sums) and ``phi`` (flux) -- plus the energy profile
``dF = F_n - F_0``, the barrier ``max dF`` and the end-state difference.

``--inset K`` moves the winding loop K sites inside the lattice edge; the
reference walks the edge itself (K = 0), where |psi| = 0 outside the
superconductor gives NaN.
"""
from __future__ import annotations

import argparse
import os

import numpy as np

from . import native, npyio


def observables(simulation_dir: str, inset: int = 0, precision: str = "fp64") -> dict:
    prob, st = npyio.load_directory(os.path.join(simulation_dir, "output_data"))
    c = native.StringContext(prob, st.n_images, precision)
    try:
        c.set_state(st)
        fe = c.compute_free_energy()
        obs = c.observables(inset)
        s_gd, s_ph = c.arc_length(), c.arc_length_jb()
    finally:
        c.close()
    dF = fe - fe[0]
    return dict(fenergy=fe, s_gd=s_gd, s_ph=s_ph, w_1=obs["w_1"], w_2=obs["w_2"], phi=obs["phi"], dF=dF,
                barrier=float(np.max(dF)), end_difference=float(dF[-1]))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("-s", "--simulation", required=True)
    ap.add_argument("--root", default="simulations")
    ap.add_argument("--inset", type=int, default=0)
    a = ap.parse_args(argv)
    d = os.path.join(a.root, a.simulation)
    out = observables(d, a.inset)
    np.savez(os.path.join(d, f"{a.simulation}.npz"), **{k: (np.nan if v is None else v) for k, v in out.items()})
    print(f"barrier {out['barrier']:.10g}, end-state difference {out['end_difference']:.10g}, "
          f"flux {out['phi'][0]:.6g} .. {out['phi'][-1]:.6g}")


if __name__ == "__main__":
    main()
