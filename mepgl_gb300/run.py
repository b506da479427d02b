"""``python -m mepgl_gb300.run [-ni] [-rc] [-- extra mepgl flags]``

Drop-in for the reference's ``run.py`` (mepgl/run.py): run from a directory
holding a reference-style ``config.py``.  Without ``-ni`` / ``-rc`` it copies
config.py into ``simulations/<name>/``, writes the initial string and the
runtime settings; ``-rc`` reloads output_data as input_data; then every stage
runs through the ``mepgl`` executable.  Unlike the reference nothing is
recompiled: the lattice size, spacing, component count and precision are
runtime settings.  ``mepgl_lib.builder`` imports in config.py resolve to
:mod:`mepgl_gb300.builder`.  Post-processing (post.py, matplotlib) is not
part of this package; it runs if a ``post.py`` sits next to config.py.
"""
from __future__ import annotations

import argparse
import importlib
import os
import shutil
import subprocess
import sys
import types

from . import builder as _builder
from . import launcher


def _alias_reference_modules():
    pkg = types.ModuleType("mepgl_lib")
    pkg.builder = _builder
    sys.modules.setdefault("mepgl_lib", pkg)
    sys.modules.setdefault("mepgl_lib.builder", _builder)


def main(argv=None):
    ap = argparse.ArgumentParser(description="Initialization and run of a string-method simulation.")
    ap.add_argument("-d", "--debug", action="store_true", help="accepted for compatibility (no build step)")
    ap.add_argument("-ni", "--no-init", action="store_true", dest="no_init")
    ap.add_argument("-rc", "--reload-continue", action="store_true", dest="rel_cont")
    ap.add_argument("extra", nargs="*", help="extra flags passed to mepgl (after --)")
    args = ap.parse_args(argv)

    sys.path.insert(0, os.getcwd())
    _alias_reference_modules()
    config = importlib.import_module("config")
    name = config.simulation_name
    print(f"Simulation name: {name}")
    sim = f"./simulations/{name}/"
    if not (args.no_init or args.rel_cont):
        os.makedirs(sim, exist_ok=True)
        shutil.copy("./config.py", sim + "config.py")
        print("[*] Generating init files. ")
        launcher.generate_init(
            config.F, config.a_1, config.a_2, config.ax, config.ay, config.b_1, config.b_2, config.comp_domain,
            config.delta, config.eta, config.gamma, config.h, config.m_xx_1, config.m_xx_2, config.m_yy_1,
            config.m_yy_2, config.multicomponent, config.q_1, config.q_2, config.sc_domain, name, config.u_1,
            config.u_2, config.v_1, config.v_2, config.x, config.y)
        launcher.generate_headers(
            N=config.N, dx=config.dx, default_relaxation_step_number=config.default_relaxation_step_number,
            multicomponent=config.multicomponent, thin_film=getattr(config, "thin_film", False),
            double_precision=getattr(config, "double_precision", False), dev_number=getattr(config, "dev_number", 0),
            path=sim + "input_data/mepgl.cfg")
        print("==> Initialization finished.\n")
    if args.rel_cont:
        print("Reloading simulation data...   ", end="")
        launcher.reload(name)
        print("done.\n")
    print("[*] Running simulation.")
    launcher.launch_simulation(name, config.F, config.iterations, config.modes, extra_args=args.extra)
    if os.path.exists("./post.py"):
        print("[*] Post processing.")
        subprocess.run([sys.executable, "./post.py"])
    return 0


if __name__ == "__main__":
    sys.exit(main())
