"""Reading and writing the reference's simulation directories.

Layout (mepgl/mepgl_lib/launcher_utils.py:195-266, mepgl/src/io.cu): a
simulation ``S`` has ``simulations/S/input_data/`` holding ``x, y,
comp_domain, sc_domain, a_1, b_1, m_xx_1, m_yy_1, a_2, b_2, m_xx_2, m_yy_2, h``
((N, N) arrays indexed [i, j], axis 0 = x), ``q.npy`` = [q_1, q_2, eta,
gamma, delta], and one sub-directory per image with ``ax, ay, u_1, v_1[, u_2,
v_2]``.  ``output_data/`` has the same files plus ``fenergy, s, s_jb`` and per
image ``jx_1, jy_1, b[, jx_2, jy_2]``.

The library's layout is the transpose (x fastest, ``[j, i]``); these helpers
convert, like the reference's loader does (io.cu:69-88).
"""
from __future__ import annotations

import os

import numpy as np

from .problem import PARAM_NAMES, Problem, StringState


def _t(a):
    return np.ascontiguousarray(np.asarray(a).T)


def read_config(path: str) -> dict:
    """``key = value`` lines of a mepgl.cfg file (missing file -> {})."""
    out = {}
    if not os.path.exists(path):
        return out
    with open(path) as f:
        for line in f:
            line = line.split("#", 1)[0]
            if "=" in line:
                k, v = line.split("=", 1)
                out[k.strip()] = v.strip()
    return out


def load_directory(d: str, n_images: int | None = None, cfg: dict | None = None):
    """(Problem, StringState) from an input_data or output_data directory."""
    cfg = dict(cfg or {})
    cfg.update(read_config(os.path.join(d, "mepgl.cfg")))
    x = np.load(os.path.join(d, "x.npy"))
    nx, ny = x.shape
    dx = float(cfg.get("dx", x[1, 0] - x[0, 0]))
    mc = bool(int(cfg["multicomponent"])) if "multicomponent" in cfg else os.path.exists(os.path.join(d, "0", "u_2.npy"))
    q = np.load(os.path.join(d, "q.npy")).astype(np.float64)
    kw = {n: _t(np.load(os.path.join(d, f"{n}.npy")).astype(np.float64)) for n in PARAM_NAMES}
    prob = Problem(nx=nx, ny=ny, dx=dx, comp_domain=_t(np.load(os.path.join(d, "comp_domain.npy")).astype(np.int32)),
                   sc_domain=_t(np.load(os.path.join(d, "sc_domain.npy")).astype(np.int32)), **kw,
                   q_1=float(q[0]), q_2=float(q[1]), eta=float(q[2]), gamma=float(q[3]), delta=float(q[4]),
                   multicomponent=mc, thin_film=bool(int(cfg.get("thin_film", 0))))
    if n_images is None:
        n_images = 0
        while os.path.exists(os.path.join(d, str(n_images), "u_1.npy")):
            n_images += 1

    def field(nre, nim):
        out = np.zeros((n_images, ny, nx, 2))
        for n in range(n_images):
            out[n, ..., 0] = _t(np.load(os.path.join(d, str(n), nre)))
            out[n, ..., 1] = _t(np.load(os.path.join(d, str(n), nim)))
        return out

    st = StringState(a=field("ax.npy", "ay.npy"), psi_1=field("u_1.npy", "v_1.npy"),
                     psi_2=field("u_2.npy", "v_2.npy") if mc else None)
    for extra in ("fenergy", "s", "s_jb"):
        p = os.path.join(d, f"{extra}.npy")
        if os.path.exists(p):
            st.extra[extra] = np.load(p)
    return prob, st


def write_input(d: str, prob: Problem, st: StringState, x=None, y=None, dtype=np.float32):
    """Write an input_data directory in the reference's layout."""
    os.makedirs(d, exist_ok=True)
    if x is None:
        ii = np.arange(prob.nx)[:, None] * prob.dx + 0 * np.arange(prob.ny)[None, :]
        x = ii
    if y is None:
        y = 0 * np.arange(prob.nx)[:, None] + np.arange(prob.ny)[None, :] * prob.dx
    np.save(os.path.join(d, "x.npy"), np.asarray(x, dtype))
    np.save(os.path.join(d, "y.npy"), np.asarray(y, dtype))
    np.save(os.path.join(d, "comp_domain.npy"), _t(prob.comp_domain).astype(np.int32))
    np.save(os.path.join(d, "sc_domain.npy"), _t(prob.sc_domain).astype(np.int32))
    for n in PARAM_NAMES:
        np.save(os.path.join(d, f"{n}.npy"), _t(getattr(prob, n)).astype(dtype))
    np.save(os.path.join(d, "q.npy"), np.array([prob.q_1, prob.q_2, prob.eta, prob.gamma, prob.delta], dtype))
    for n in range(st.n_images):
        dd = os.path.join(d, str(n))
        os.makedirs(dd, exist_ok=True)
        np.save(os.path.join(dd, "ax.npy"), _t(st.a[n, ..., 0]).astype(dtype))
        np.save(os.path.join(dd, "ay.npy"), _t(st.a[n, ..., 1]).astype(dtype))
        np.save(os.path.join(dd, "u_1.npy"), _t(st.psi_1[n, ..., 0]).astype(dtype))
        np.save(os.path.join(dd, "v_1.npy"), _t(st.psi_1[n, ..., 1]).astype(dtype))
        if prob.multicomponent:
            np.save(os.path.join(dd, "u_2.npy"), _t(st.psi_2[n, ..., 0]).astype(dtype))
            np.save(os.path.join(dd, "v_2.npy"), _t(st.psi_2[n, ..., 1]).astype(dtype))


def write_config(path: str, **kw):
    with open(path, "w") as f:
        f.write("# runtime settings of the mepgl executable (replace the generated headers)\n")
        for k, v in kw.items():
            f.write(f"{k} = {v}\n")
