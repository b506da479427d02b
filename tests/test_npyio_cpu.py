"""Simulation-directory I/O (Python) and the executable's .npy reader/writer (C++)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from mepgl_gb300 import npyio, workloads as W


def test_directory_roundtrip(tmp_path):
    prob, st = W.config2(n=12, images=3)
    d = str(tmp_path / "input_data")
    npyio.write_input(d, prob, st, dtype=np.float64)
    npyio.write_config(os.path.join(d, "mepgl.cfg"), dx=repr(prob.dx), multicomponent=1)
    p2, s2 = npyio.load_directory(d)
    assert (p2.nx, p2.ny, p2.multicomponent) == (prob.nx, prob.ny, True)
    assert p2.dx == prob.dx
    np.testing.assert_array_equal(p2.sc_domain, prob.sc_domain)
    np.testing.assert_array_equal(p2.h, prob.h)
    np.testing.assert_array_equal(s2.psi_2, st.psi_2)
    np.testing.assert_array_equal(s2.a, st.a)


@pytest.fixture(scope="module")
def roundtrip_exe(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("npy") / "npy_roundtrip")
    src = os.path.join(ROOT, "mepgl_gb300", "csrc")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", src, os.path.join(ROOT, "tests", "npy_roundtrip.cpp"),
                    os.path.join(src, "npy.cpp"), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32, np.int64, np.bool_])
@pytest.mark.parametrize("shape", [(5,), (3, 4), (2, 3, 4)])
def test_cpp_reader_writer(roundtrip_exe, tmp_path, dtype, shape):
    a = (np.arange(np.prod(shape)).reshape(shape) % 7 - 3).astype(dtype)
    src, dst = str(tmp_path / "a.npy"), str(tmp_path / "b.npy")
    np.save(src, a)
    subprocess.run([roundtrip_exe, src, dst], check=True)
    b = np.load(dst)
    assert b.dtype == np.float64 and b.shape == shape
    np.testing.assert_array_equal(b, a.astype(np.float64))


def test_cpp_reader_rejects_garbage(roundtrip_exe, tmp_path):
    bad = tmp_path / "bad.npy"
    bad.write_bytes(b"not numpy at all")
    r = subprocess.run([roundtrip_exe, str(bad), str(tmp_path / "o.npy")], capture_output=True, text=True)
    assert r.returncode == 1 and "not an .npy" in r.stderr
