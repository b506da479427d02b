"""Launcher functions with the reference's interface (mepgl/mepgl_lib/launcher_utils.py).

* ``generate_init`` writes ``simulations/<name>/input_data/`` exactly as the
  reference does (float32 by default, float64 on request -- the executable
  reads either, by dtype).
* ``generate_headers`` keeps its signature but writes the runtime settings to
  ``./mepgl.cfg`` instead of generating C headers: nothing is recompiled,
  so it returns False.
* ``launch_simulation`` runs the stages with the ``mepgl`` executable of this
  package, copying output_data to input_data between stages as
  ``reload.py`` does (launcher_utils.py:151-189).
"""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np

from .npyio import write_config

PKG = os.path.dirname(os.path.abspath(__file__))
EXE = os.path.join(PKG, "_lib", "mepgl")


def executable() -> str:
    if not os.path.exists(EXE):
        from . import build
        build.build()
    return EXE


def generate_headers(N, dx, default_relaxation_step_number, multicomponent, thin_film=False, double_precision=False,
                     dev_number=0, path="./mepgl.cfg", **extra):
    settings = dict(N=N, dx=repr(float(dx)), multicomponent=int(bool(multicomponent)), thin_film=int(bool(thin_film)),
                    precision="fp64" if double_precision else "fp32",
                    relaxation_steps=int(default_relaxation_step_number), dev_number=int(dev_number))
    settings.update(extra)
    write_config(path, **settings)
    return False


def generate_init(F, a_1, a_2, ax, ay, b_1, b_2, comp_domain, delta, eta, gamma, h, m_xx_1, m_xx_2, m_yy_1, m_yy_2,
                  multicomponent, q_1, q_2, sc_domain, simulation_name, u_1, u_2, v_1, v_2, x, y,
                  double_precision=False):
    dt = np.float64 if double_precision else np.float32
    d = f"./simulations/{simulation_name}/input_data/"
    if os.path.exists(d):
        shutil.rmtree(d)
    os.makedirs(d, exist_ok=True)
    save = lambda name, arr, t=dt: np.save(d + name, np.asarray(arr).astype(t))
    save("x.npy", x)
    save("y.npy", y)
    save("comp_domain.npy", comp_domain, np.int32)
    save("sc_domain.npy", sc_domain, np.int32)
    for name, arr in (("a_1", a_1), ("b_1", b_1), ("m_xx_1", m_xx_1), ("m_yy_1", m_yy_1), ("a_2", a_2),
                      ("b_2", b_2), ("m_xx_2", m_xx_2), ("m_yy_2", m_yy_2), ("h", h)):
        save(f"{name}.npy", np.broadcast_to(np.asarray(arr, dtype=np.float64), np.shape(x)))
    save("q.npy", np.array([q_1, q_2, eta, gamma, delta], dtype=np.float64))
    F0 = int(np.atleast_1d(F)[0])
    for n in range(F0):
        os.makedirs(d + f"{n}/", exist_ok=True)
        save(f"{n}/ax.npy", ax[n])
        save(f"{n}/ay.npy", ay[n])
        save(f"{n}/u_1.npy", u_1[n])
        save(f"{n}/v_1.npy", v_1[n])
        if multicomponent:
            save(f"{n}/u_2.npy", u_2[n])
            save(f"{n}/v_2.npy", v_2[n])


def reload(simulation_name):
    """Copy output_data to input_data (the reference's reload.py)."""
    base = f"./simulations/{simulation_name}/"
    shutil.rmtree(base + "input_data", ignore_errors=True)
    shutil.copytree(base + "output_data", base + "input_data")


def launch_simulation(simulation_name, F, iterations, modes, extra_args=(), check=True):
    """Run every stage; stage i resamples F[i] -> F[i+1] images at its end."""
    F = np.atleast_1d(F)
    iterations = np.atleast_1d(iterations)
    modes = np.atleast_1d(modes)
    exe = executable()
    P = F.shape[0]
    for i in range(P):
        f_out = F[i + 1] if i + 1 < P else F[i]
        cmd = [exe, "--simname", str(simulation_name), "--mode", str(modes[i]), "--Fin", str(int(F[i])),
               "--Fout", str(int(f_out)), "--iterations", str(int(iterations[i]))] + list(extra_args)
        r = subprocess.run(cmd)
        if check and r.returncode != 0:
            raise RuntimeError(f"mepgl stage {i} failed with exit code {r.returncode}")
        if i + 1 < P:
            reload(simulation_name)
