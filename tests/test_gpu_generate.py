"""Initial strings built on the device (mepgl_generate_string): without
noise they equal the reference-interface builder (mepgl_gb300.builder, the
reference's StringBuilder envelope and phases) to 1e-12; the Philox noise
is reproducible per seed, independent between seeds, N(0, sigma^2) and
masked to the superconducting domain; the gauges give the builder's A."""
import numpy as np
import pytest

from mepgl_gb300.builder import StringBuilder
from mepgl_gb300.problem import Problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def native():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mepgl_gb300 import build
    build.build()
    from mepgl_gb300 import native as N
    return N


def _setup(mc=True, F=5, Nx=40, Ny=33):
    dx = 20.0 / (Nx - 1)                     # one lattice spacing on both axes
    sb = StringBuilder(F, Nx, Ny, (-10.0, 10.0), (-8.0, -8.0 + dx * (Ny - 1)), mc, B_z=0.6)
    sb.set_sc_domain(lambda x, y: x * x / 81 + y * y / 49 <= 1.0)
    xv = np.linspace(-9.0, 2.0, F)
    wv = np.array([0] + [1] * (F - 1))
    sb.add_vortex(xv, 0.3 + 0 * xv, wv, 1)
    if mc:
        sb.add_vortex(xv + 0.5, -0.2 + 0 * xv, wv, 2)
        sb.add_vortex(3.0 + 0 * xv, 2.0 + 0 * xv, -wv, 2)
    comp, sc = sb.get_domain_matrices()
    prob = Problem.uniform(Nx, Ny, dx, multicomponent=mc, comp_domain=comp.T.copy(), sc_domain=sc.T.copy())
    tracks = [(c, np.asarray(x), np.asarray(y), np.asarray(w)) for c, vs in ((1, sb.vortices_1), (2, sb.vortices_2))
              for x, y, w in vs]
    return sb, prob, tracks


@pytest.mark.parametrize("mc", [True, False])
def test_noiseless_string_matches_builder(native, mc):
    sb, prob, tracks = _setup(mc)
    c = native.StringContext(prob, sb.F, "fp64")
    c.generate_string(tracks, x0=-10.0, y0=-8.0, psi_abs_1=1.0, psi_abs_2=0.8, gauge="symmetric", b_z=0.6)
    st = c.get_state()
    u1, v1, u2, v2 = sb.generate_matter_fields(psi_abs_1=1.0, psi_abs_2=0.8, noise=0.0)
    ax, ay = sb.generate_vector_potential("symmetric")
    tr = lambda f: np.transpose(f, (0, 2, 1))
    np.testing.assert_allclose(st.psi_1[..., 0], tr(u1), atol=1e-12)
    np.testing.assert_allclose(st.psi_1[..., 1], tr(v1), atol=1e-12)
    if mc:
        np.testing.assert_allclose(st.psi_2[..., 0], tr(u2), atol=1e-12)
        np.testing.assert_allclose(st.psi_2[..., 1], tr(v2), atol=1e-12)
    np.testing.assert_allclose(st.a[..., 0], tr(ax), atol=1e-12)
    np.testing.assert_allclose(st.a[..., 1], tr(ay), atol=1e-12)


def test_noise_is_seeded_gaussian_and_masked(native):
    sb, prob, tracks = _setup(True, F=4, Nx=160, Ny=130)
    c = native.StringContext(prob, sb.F, "fp64")
    c.generate_string(tracks, x0=-10.0, y0=-8.0)
    base = c.get_state()
    runs = []
    for seed in (7, 7, 8):
        c.generate_string(tracks, x0=-10.0, y0=-8.0, noise=0.05, seed=seed)
        runs.append(c.get_state())
    np.testing.assert_array_equal(runs[0].psi_1, runs[1].psi_1)
    sc = prob.sc_domain.astype(bool)
    z = (runs[0].psi_1 - base.psi_1)[:, sc, :] / 0.05
    z2 = (runs[2].psi_1 - base.psi_1)[:, sc, :] / 0.05
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01
    assert abs(np.corrcoef(z.ravel(), z2.ravel())[0, 1]) < 0.01
    w = (runs[0].psi_2 - base.psi_2)[:, sc, :].ravel() / 0.05
    assert abs(np.corrcoef(z.ravel(), w)[0, 1]) < 0.01
    assert np.all(runs[0].psi_1[:, ~sc, :] == 0)
    f32 = native.StringContext(prob, sb.F, "fp32")
    f32.generate_string(tracks, x0=-10.0, y0=-8.0, noise=0.05, seed=7)
    np.testing.assert_allclose(f32.get_state().psi_1, runs[0].psi_1, atol=1e-6)
