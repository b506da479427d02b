"""Shared pytest configuration: markers, repository on sys.path, golden loader."""
import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")
    config.addinivalue_line("markers", "slow: longer CPU test")


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def load_golden(name):
    """Return (Problem, StringState, dict of arrays) for a golden case."""
    from mepgl_gb300.problem import PARAM_NAMES, Problem, StringState
    z = dict(np.load(os.path.join(GOLDEN_DIR, name + ".npz")))
    nx, ny, mc, film = (int(v) for v in z["flags"])
    dx, q1, q2, eta, gamma, delta = (float(v) for v in z["scalars"])
    prob = Problem(nx=nx, ny=ny, dx=dx, comp_domain=z["comp_domain"], sc_domain=z["sc_domain"],
                   **{k: z[k] for k in PARAM_NAMES}, q_1=q1, q_2=q2, eta=eta, gamma=gamma, delta=delta,
                   multicomponent=bool(mc), thin_film=bool(film))
    st = StringState(a=z["a"], psi_1=z["psi_1"], psi_2=z["psi_2"] if mc else None)
    return prob, st, z


@pytest.fixture(params=golden_names())
def golden(request):
    return load_golden(request.param)
