"""Gauge links on the GPU (discretization = MEPGL_DISC_LINK): energy,
gradient and adjoints against the oracle's link functional, exact invariance
under a random lattice gauge transform, and, for the reference
discretisation, gauge covariance that improves as dx -> 0.

Tolerances: FP64 energies 1e-12 relative, gradients 1e-12 of the max-norm
(sin / cos of the link phases may differ from the host's by an ulp); FP32
2e-5; gauge invariance 1e-12 (FP64)."""
import numpy as np
import pytest

from mepgl_gb300 import workloads as W
from mepgl_gb300.problem import PARAM_NAMES, Problem, StringState
from oracle import cref
from test_oracle_link import lattice_gauge

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


def _case(seed, mc=True, film=False, uniform=False, nx=37, ny=22):
    rng = np.random.default_rng(seed)
    prob = W.random_problem(rng, n=max(nx, ny), multicomponent=mc, thin_film=film, uniform=uniform)
    kw = {k: getattr(prob, k)[:ny, :nx].copy() for k in PARAM_NAMES + ("comp_domain", "sc_domain")}
    prob = prob.with_(nx=nx, ny=ny, q_2=prob.q_1, **kw)
    return rng, prob, W.random_state(rng, prob, images=3)


def relmax(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _ctx(native, prob, st, precision="fp64"):
    c = native.StringContext(prob, st.n_images, precision, discretization=native.DISC_LINK)
    c.set_state(st)
    return c


@pytest.mark.parametrize("mc,film,uniform", [(True, False, False), (True, False, True), (False, False, True),
                                             (True, True, False)])
def test_link_energy_gradient_vs_oracle(native, mc, film, uniform):
    rng, prob, st = _case(31, mc, film, uniform)
    o = cref.Oracle(prob)
    c = _ctx(native, prob, st)
    e, g = c.energy_grad()
    np.testing.assert_allclose(e, o.energy_link(st.a, st.psi_1, st.psi_2), rtol=1e-12)
    go = o.gradient_link(st.a, st.psi_1, st.psi_2)
    for k in range(1 + prob.ncomp):
        if film and k == 0:
            assert np.all(g[0] == 0)
            continue
        assert relmax(g[k], go[k]) < 1e-12, k
    c32 = _ctx(native, prob, st, "fp32")
    o32 = cref.Oracle(prob, np.float32)
    e32, g32 = c32.energy_grad()
    np.testing.assert_allclose(e32, o32.energy_link(st.a, st.psi_1, st.psi_2), rtol=2e-5)
    go32 = o32.gradient_link(st.a, st.psi_1, st.psi_2)
    assert relmax(g32[1], go32[1]) < 2e-5


def test_link_energy_is_gauge_invariant_on_gpu(native):
    rng, prob, st = _case(32, True, False, False)
    chi = rng.uniform(-5, 5, (st.n_images, prob.ny, prob.nx))
    e0 = _ctx(native, prob, st).compute_free_energy()
    e1 = _ctx(native, prob, lattice_gauge(prob, st, chi)).compute_free_energy()
    np.testing.assert_allclose(e1, e0, rtol=1e-12)
    # the gradient transforms covariantly: |dF/dpsi| is invariant site by site
    _, g0 = _ctx(native, prob, st).energy_grad()
    _, g1 = _ctx(native, prob, lattice_gauge(prob, st, chi)).energy_grad()
    for k in (1, 2):
        n0 = np.hypot(g0[k][..., 0], g0[k][..., 1])
        n1 = np.hypot(g1[k][..., 0], g1[k][..., 1])
        assert relmax(n1, n0) < 1e-11


def test_link_adjoints_match_central_differences(native):
    rng, prob, st = _case(33, True, False, True)
    adj = _ctx(native, prob, st).param_adjoint()
    h = 1e-6
    for k, shift in enumerate((lambda p, e: p.with_(h=p.h + e), lambda p, e: p.with_(eta=p.eta + e),
                               lambda p, e: p.with_(gamma=p.gamma + e))):
        fd = (_ctx(native, shift(prob, h), st).compute_free_energy()
              - _ctx(native, shift(prob, -h), st).compute_free_energy()) / (2 * h)
        np.testing.assert_allclose(adj[:, k], fd, rtol=1e-6, atol=1e-6 * np.abs(fd).max())


def test_link_mode_refuses_nlcg(native):
    _, prob, st = _case(34)
    c = _ctx(native, prob, st)
    with pytest.raises(native.MepglError):
        c.nlcg_steps(2)
    with pytest.raises(native.MepglError):
        c.loop_iteration("L", 2)


def test_link_autograd_backward(native):
    import torch
    from mepgl_gb300.autograd import GLEnergy
    _, prob, st = _case(35, True, False, False)
    g = GLEnergy(prob, st.n_images, discretization=native.DISC_LINK)
    t = [torch.tensor(x, device="cuda").requires_grad_() for x in (st.a, st.psi_1, st.psi_2)]
    e = g(*t)
    e.sum().backward()
    go = cref.Oracle(prob).gradient_link(st.a, st.psi_1, st.psi_2)
    for k in range(3):
        assert relmax(t[k].grad.cpu().numpy(), go[k]) < 1e-12
    g.close()


def test_reference_discretisation_gauge_covariance_improves_with_dx(native):
    """Smooth chi on a fixed physical square: the reference's linearised
    differences change the energy by O(dx^2) under the continuum transform
    (measured on the oracle: 1.1e-2, 2.7e-3, 6.6e-4 at n = 24, 48, 96)."""
    L = 6.0
    errs = []
    for n in (24, 48, 96):
        dx = L / n
        x = (np.arange(n) + 0.5) * dx
        X, Y = np.meshgrid(x, x, indexing="xy")
        psi = (0.8 + 0.1 * np.sin(2 * np.pi * X / L)) * np.exp(1j * 2 * np.pi * Y / L)
        a = np.stack([0.2 * np.cos(2 * np.pi * Y / L), 0.1 * np.sin(2 * np.pi * X / L)], axis=-1)
        chi = 0.7 * np.sin(2 * np.pi * X / L) * np.cos(2 * np.pi * Y / L)
        dchi = np.stack([0.7 * 2 * np.pi / L * np.cos(2 * np.pi * X / L) * np.cos(2 * np.pi * Y / L),
                         -0.7 * 2 * np.pi / L * np.sin(2 * np.pi * X / L) * np.sin(2 * np.pi * Y / L)], axis=-1)
        prob = Problem.uniform(n, n, dx, h=0.5)
        s0 = StringState(a=a[None], psi_1=np.stack([psi.real, psi.imag], axis=-1)[None])
        pg = psi * np.exp(1j * chi)
        s1 = StringState(a=(a + dchi)[None], psi_1=np.stack([pg.real, pg.imag], axis=-1)[None])
        e = []
        for s in (s0, s1):
            c = native.StringContext(prob, 1, "fp64")
            c.set_state(s)
            e.append(c.compute_free_energy()[0])
        errs.append(abs(e[1] - e[0]) / abs(e[0]))
    assert errs[0] > errs[1] > errs[2]
    assert errs[1] / errs[2] > 3.0
