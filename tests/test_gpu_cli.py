"""The `mepgl` executable and the run.py-compatible launcher, end to end on the GPU.

A simulation directory is written in the reference's layout, the executable
runs with the reference's flags (mode L, a resample to more images at the
end), and the saved output_data is compared with the C oracle running the
same loop() iterations, arc length and linear resample.
"""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from conftest import ROOT
from mepgl_gb300 import npyio, workloads as W
from oracle import cref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def exe():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mepgl_gb300 import build
    build.build()
    return os.path.join(ROOT, "mepgl_gb300", "_lib", "mepgl")


def _run(exe, cwd, *args):
    r = subprocess.run([exe, *args], cwd=cwd, stdin=subprocess.DEVNULL, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return r.stdout


def test_cli_mode_l_with_final_resample_matches_oracle(exe, tmp_path):
    prob, st = W.config2(n=20, images=5)
    d = tmp_path / "simulations" / "t" / "input_data"
    npyio.write_input(str(d), prob, st, dtype=np.float64)
    npyio.write_config(str(d / "mepgl.cfg"), dx=repr(prob.dx), multicomponent=1, precision="fp64",
                       relaxation_steps=4)
    out = _run(exe, tmp_path, "--simname", "t", "--mode", "L", "--Fin", "5", "--Fout", "7", "--iterations", "3")
    assert "Finished" in out
    assert (tmp_path / "energy.csv").exists()
    p_out, s_out = npyio.load_directory(str(tmp_path / "simulations" / "t" / "output_data"))
    assert s_out.n_images == 7 and s_out.a.dtype == np.float64

    o = cref.Oracle(prob)
    sv = o.solver(st)
    for _ in range(3):
        sv.iteration("L", 4)
    r = sv.get()
    b, j1, j2 = o.jb(r["a"], r["psi_1"], r["psi_2"])
    s_jb = o.arc_length(b, j1, j2)
    fields = [o.redistribute(s_jb, r[k], 7) for k in ("a", "psi_1", "psi_2")]
    e_ref = o.energy(*fields)
    np.testing.assert_allclose(s_out.extra["fenergy"], e_ref, rtol=1e-9)
    assert np.max(np.abs(s_out.psi_1 - fields[1])) < 1e-8
    assert np.max(np.abs(s_out.a - fields[0])) < 1e-8
    # B and J of the output images
    b_out = np.load(tmp_path / "simulations" / "t" / "output_data" / "3" / "b.npy").T
    bo, _, _ = o.jb(*fields)
    np.testing.assert_allclose(b_out, bo[3], atol=1e-9)


def test_cli_reads_float32_inputs_in_fp64(exe, tmp_path):
    """The reference's FP64 build misreads float32 .npy inputs; this one converts."""
    prob, st = W.config1(n=16, images=3)
    d = tmp_path / "simulations" / "f" / "input_data"
    npyio.write_input(str(d), prob, st, dtype=np.float32)
    npyio.write_config(str(d / "mepgl.cfg"), dx=repr(prob.dx), multicomponent=0, precision="fp64")
    _run(exe, tmp_path, "--simname", "f", "--mode", "S", "--Fin", "3", "--Fout", "3", "--iterations", "1",
         "--relaxation-steps", "2")
    _, s_out = npyio.load_directory(str(tmp_path / "simulations" / "f" / "output_data"))
    st32 = st.astype(np.float32).astype(np.float64)
    sv = cref.Oracle(prob).solver(st32)
    sv.nlcg_steps(2)
    np.testing.assert_allclose(s_out.psi_1, sv.get()["psi_1"], atol=1e-9)


CONFIG = """
import numpy as np
from mepgl_lib.builder import StringBuilder

dev_number = 0
double_precision = False
simulation_name = "tiny"
F = np.array([4, 6])
iterations = np.array([2, 2])
modes = np.array(["S", "L"])
default_relaxation_step_number = 5
multicomponent = False
thin_film = False
N = 24
L = 6
builder = StringBuilder(F[0], Nx=N, Ny=N, x_lim=[-L / 2, L / 2], y_lim=[-L / 2, L / 2],
                        multicomponent=multicomponent, seed=3)
x, y = builder.x, builder.y
dx = builder.x_ax[1] - builder.x_ax[0]
comp_domain, sc_domain = builder.get_domain_matrices()
q_1 = -1.0; a_1 = -1.0; b_1 = 1.0; m_xx_1 = 1.0; m_yy_1 = 1.0
q_2 = -1.0; a_2 = -1.0; b_2 = 1.0; m_xx_2 = 1.0; m_yy_2 = 1.0
eta = 0.0; gamma = 0.0; delta = 0.0
ones = np.ones((N, N))
a_1 *= ones; b_1 *= ones; m_xx_1 *= ones; m_yy_1 *= ones
a_2 *= ones; b_2 *= ones; m_xx_2 *= ones; m_yy_2 *= ones
h = 0.5 * comp_domain
builder.add_vortex(np.linspace(4, 0, F[0]), np.zeros(F[0]), -np.ones(F[0]), 1)
u_1, v_1, u_2, v_2 = builder.generate_matter_fields(psi_abs_1=1.0, noise=0.05)
ax = np.zeros_like(u_1)
ay = np.zeros_like(u_1)
"""


def test_run_module_with_reference_style_config(exe, tmp_path):
    (tmp_path / "config.py").write_text(textwrap.dedent(CONFIG))
    env = dict(os.environ, PYTHONPATH=ROOT + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, "-m", "mepgl_gb300.run"], cwd=tmp_path, env=env, capture_output=True,
                       text=True, stdin=subprocess.DEVNULL, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    out = tmp_path / "simulations" / "tiny" / "output_data"
    fe = np.load(out / "fenergy.npy")
    assert fe.shape == (6,) and np.all(np.isfinite(fe))
    assert (out / "5" / "u_1.npy").exists() and (out / "mepgl.cfg").exists()
