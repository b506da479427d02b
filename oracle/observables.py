"""CPU restatement of the per-image observables (TEST INFRASTRUCTURE).

Only tests use this module, as the checker of the device observables
(mepgl_observables).  Arrays follow the library layout (F, ny, nx[, 2]),
x fastest.

* flux: Phi_n = dx^2 * sum of B over image n (mepgl/post.py:131-133), with B
  from the oracle's computeJB restatement;
* winding: compute_winding (mepgl/mepgl_lib/gl_utils.py:10-41): around the
  rectangle `inset` sites inside the lattice edge, counter-clockwise from
  the lower-left corner, the sum of (u dv - v du) / (u^2 + v^2) over the
  steps, each taken at its start site.  inset = 0 is the reference's loop.
"""
from __future__ import annotations

import numpy as np


def flux(b, dx):
    b = np.asarray(b, np.float64)
    return b.reshape(b.shape[0], -1).sum(axis=1) * dx * dx


def loop_sites(nx, ny, inset=0):
    """Start and end sites (i, j) of every step of the loop, in order."""
    i0 = j0 = inset
    i1, j1 = nx - 1 - inset, ny - 1 - inset
    steps = [((i, j0), (i + 1, j0)) for i in range(i0, i1)]
    steps += [((i1, j), (i1, j + 1)) for j in range(j0, j1)]
    steps += [((i, j1), (i - 1, j1)) for i in range(i1, i0, -1)]
    steps += [((i0, j), (i0, j - 1)) for j in range(j1, j0, -1)]
    return steps


def winding(psi, inset=0):
    psi = np.asarray(psi, np.float64)
    F, ny, nx, _ = psi.shape
    steps = loop_sites(nx, ny, inset)
    a = np.array([s[0] for s in steps])
    b = np.array([s[1] for s in steps])
    u, v = psi[:, a[:, 1], a[:, 0], 0], psi[:, a[:, 1], a[:, 0], 1]
    du, dv = psi[:, b[:, 1], b[:, 0], 0] - u, psi[:, b[:, 1], b[:, 0], 1] - v
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.sum((u * dv - v * du) / (u * u + v * v), axis=1)
