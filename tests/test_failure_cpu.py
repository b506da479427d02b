"""Failure detection on the host side of the `mepgl` executable (no GPU).

The reference reads its inputs unchecked (mepgl/src/io.cu:18-125) and would
index past its arrays in the arc-length resample with too few images
(mepgl/src/interpolation.cu:252-322).  The executable here rejects both
before it creates a context, with the library status as exit code:
3 (MEPGL_ERR_NAN) for a non-finite input value, 1 (MEPGL_ERR_INVALID_ARG)
for too few images.  These checks run before any CUDA call, so they are
tested here without a GPU.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from mepgl_gb300 import npyio, workloads as W


@pytest.fixture(scope="module")
def exe():
    from mepgl_gb300 import build
    build.build()
    return os.path.join(ROOT, "mepgl_gb300", "_lib", "mepgl")


def _sim(tmp_path, images=4):
    prob, st = W.config1(n=12, images=images)
    d = tmp_path / "simulations" / "t" / "input_data"
    npyio.write_input(str(d), prob, st, dtype=np.float64)
    npyio.write_config(str(d / "mepgl.cfg"), dx=repr(prob.dx), multicomponent=0, precision="fp64")
    return d


def _run(exe, cwd, *args):
    return subprocess.run([exe, "--simname", "t", *args], cwd=cwd, stdin=subprocess.DEVNULL, capture_output=True,
                          text=True, timeout=120)


@pytest.mark.parametrize("name", ["1/u_1.npy", "h.npy", "3/ay.npy"])
def test_nan_in_an_input_file_exits_with_the_nan_status(exe, tmp_path, name):
    d = _sim(tmp_path)
    path = d / name
    arr = np.load(path)
    arr[3, 5] = np.nan if name != "3/ay.npy" else np.inf
    np.save(path, arr)
    r = _run(exe, tmp_path, "--mode", "S", "--iterations", "1")
    assert r.returncode == 3, r.stdout + r.stderr
    assert "non-finite value" in r.stderr and name.split("/")[-1] in r.stderr


def test_nan_coupling_exits_with_the_nan_status(exe, tmp_path):
    d = _sim(tmp_path)
    np.save(d / "q.npy", np.array([1.0, 1.0, np.nan, 0.0, 0.0]))
    r = _run(exe, tmp_path, "--mode", "S", "--iterations", "1")
    assert r.returncode == 3 and "non-finite coupling" in r.stderr, r.stdout + r.stderr


def test_cubic_mode_needs_four_images(exe, tmp_path):
    _sim(tmp_path, images=3)
    r = _run(exe, tmp_path, "--mode", "C", "--iterations", "1")
    assert r.returncode == 1 and "needs at least 4 images" in r.stderr, r.stdout + r.stderr


def test_linear_mode_needs_two_images(exe, tmp_path):
    _sim(tmp_path, images=1)
    r = _run(exe, tmp_path, "--mode", "L", "--iterations", "1")
    assert r.returncode == 1 and "needs at least 2 images" in r.stderr, r.stdout + r.stderr


def test_missing_images_is_an_argument_error(exe, tmp_path):
    d = tmp_path / "simulations" / "t" / "input_data"
    prob, st = W.config1(n=12, images=2)
    npyio.write_input(str(d), prob, st, dtype=np.float64)
    os.rename(d / "0", d / "zero")
    r = _run(exe, tmp_path, "--mode", "S", "--iterations", "1")
    assert r.returncode == 1 and "no images" in r.stderr, r.stdout + r.stderr
