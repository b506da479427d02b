"""Device observables (mepgl_observables) against the oracle restatement:
flux dx^2 sum B and the winding sums of compute_winding, on the lattice edge
(the reference's loop) and on an inset rectangle; tolerance 1e-12 relative
in FP64 (NaN where the reference's loop divides by |psi|^2 = 0), 2e-5 in
FP32.  The post-processing module writes the reference's summary keys."""
import numpy as np
import pytest

from mepgl_gb300 import workloads as W
from mepgl_gb300.problem import PARAM_NAMES
from oracle import cref
from oracle import observables as O

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


def _case(seed, mc, nx=29, ny=21):
    rng = np.random.default_rng(seed)
    prob = W.random_problem(rng, n=max(nx, ny), multicomponent=mc, uniform=False)
    kw = {k: getattr(prob, k)[:ny, :nx].copy() for k in PARAM_NAMES + ("comp_domain", "sc_domain")}
    prob = prob.with_(nx=nx, ny=ny, **kw)
    return prob, W.random_state(rng, prob, images=3)


@pytest.mark.parametrize("mc", [True, False])
@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-12), ("fp32", 2e-5)])
def test_flux_and_winding_vs_oracle(native, mc, precision, rtol):
    prob, st = _case(51, mc)
    c = native.StringContext(prob, st.n_images, precision)
    c.set_state(st)
    dt = np.float64 if precision == "fp64" else np.float32
    b, _, _ = cref.Oracle(prob, dt).jb(st.a, st.psi_1, st.psi_2)
    for inset in (0, 3):
        obs = c.observables(inset)
        np.testing.assert_allclose(obs["phi"], O.flux(b, prob.dx), rtol=rtol, atol=rtol * np.abs(b).sum() * prob.dx ** 2)
        fields = [st.psi_1] + ([st.psi_2] if mc else [])
        for k, f in enumerate(fields):
            want = O.winding(np.asarray(f, dt), inset)
            np.testing.assert_allclose(obs[f"w_{k + 1}"], want, rtol=rtol, atol=rtol * np.nanmax(np.abs(want)),
                                       equal_nan=True)
        if not mc:
            assert obs["w_2"] is None


def test_vortex_string_winds_once(native):
    """Config 1: Meissner state to one vortex at lattice (8, 32); the loop 5
    sites inside the edge encloses the vortex (2 pi) and nothing in image 0."""
    prob, st = W.config1()
    c = native.StringContext(prob, st.n_images, "fp64")
    c.set_state(st)
    w = c.observables(5)["w_1"]
    assert abs(w[0]) < 0.05 and abs(w[-1] - 2 * np.pi) < 0.2
    assert np.all(np.isnan(c.observables(0)["w_1"]))     # the edge lies in the vacuum margin


def test_post_module_writes_reference_keys(native, tmp_path):
    from mepgl_gb300 import npyio, post
    prob, st = W.config2(n=24, images=4)
    out = tmp_path / "sim" / "output_data"
    npyio.write_input(str(out), prob, st, dtype=np.float64)
    r = post.observables(str(tmp_path / "sim"), inset=5)
    for key in ("fenergy", "s_gd", "s_ph", "w_1", "w_2", "phi", "dF"):
        assert len(r[key]) == 4
    c = native.StringContext(prob, 4, "fp64")
    c.set_state(st)
    np.testing.assert_allclose(r["fenergy"], c.compute_free_energy(), rtol=1e-12)
    np.testing.assert_allclose(r["phi"], c.observables(5)["phi"], rtol=1e-12)
    assert r["barrier"] == pytest.approx(np.max(r["fenergy"] - r["fenergy"][0]))
    post.main(["-s", "sim", "--root", str(tmp_path), "--inset", "5"])
    z = np.load(tmp_path / "sim" / "sim.npz")
    assert set(("fenergy", "s_gd", "s_ph", "w_1", "w_2", "phi")) <= set(z.files)
