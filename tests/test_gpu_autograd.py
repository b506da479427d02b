"""GLEnergy (torch.autograd.Function over the CUDA kernels) and the parameter
adjoints dF/dH, dF/deta, dF/dgamma.

Tolerances: forward energies 1e-12 relative to the oracle; backward 1e-12 of
the max-norm against the oracle gradient; adjoints 1e-12 against the oracle
adjoint; central finite differences with h = 1e-6 agree to 1e-6 relative
(truncation ~h^2, rounding ~1e-16 |F| / h)."""
import numpy as np
import pytest

from mepgl_gb300 import workloads as W
from mepgl_gb300.problem import PARAM_NAMES
from oracle import cref

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def native():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mepgl_gb300 import build
    build.build()
    from mepgl_gb300 import native as N
    return N


def _case(seed, mc=True, film=False, uniform=False, nx=26, ny=19, images=3):
    rng = np.random.default_rng(seed)
    prob = W.random_problem(rng, n=max(nx, ny), multicomponent=mc, thin_film=film, uniform=uniform)
    kw = {k: getattr(prob, k)[:ny, :nx].copy() for k in PARAM_NAMES + ("comp_domain", "sc_domain")}
    prob = prob.with_(nx=nx, ny=ny, **kw)
    return prob, W.random_state(rng, prob, images=images)


def _cuda(x, dtype=torch.float64):
    return None if x is None else torch.tensor(np.ascontiguousarray(x), dtype=dtype, device="cuda")


def relmax(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("mc,film,uniform", [(True, False, False), (True, False, True), (False, False, False),
                                             (True, True, False)])
def test_forward_backward_and_adjoint_vs_oracle(mc, film, uniform):
    from mepgl_gb300.autograd import GLEnergy
    prob, st = _case(11, mc, film, uniform)
    g = GLEnergy(prob, st.n_images)
    a = _cuda(st.a).requires_grad_()
    p1 = _cuda(st.psi_1).requires_grad_()
    p2 = _cuda(st.psi_2).requires_grad_() if mc else None
    theta = torch.tensor([0.0, prob.eta, prob.gamma], dtype=torch.float64, requires_grad=True)
    e = g(a, p1, p2, theta)
    o = cref.Oracle(prob)
    np.testing.assert_allclose(e.detach().cpu().numpy(), o.energy(st.a, st.psi_1, st.psi_2), rtol=1e-12)
    w = torch.tensor(np.random.default_rng(5).uniform(-2, 2, st.n_images), dtype=torch.float64, device="cuda")
    (e * w).sum().backward()
    go = o.gradient(st.a, st.psi_1, st.psi_2)
    wn = w.cpu().numpy()[:, None, None, None]
    assert relmax(a.grad.cpu().numpy(), go[0] * wn) < 1e-12
    assert relmax(p1.grad.cpu().numpy(), go[1] * wn) < 1e-12
    if mc:
        assert relmax(p2.grad.cpu().numpy(), go[2] * wn) < 1e-12
    adj = o.param_adjoint(st.a, st.psi_1, st.psi_2)
    want = (w.cpu().numpy()[:, None] * adj).sum(0)
    np.testing.assert_allclose(theta.grad.numpy(), want, rtol=1e-12, atol=1e-12 * np.abs(adj).max())
    g.close()


def test_adjoints_match_central_differences():
    from mepgl_gb300.autograd import GLEnergy
    prob, st = _case(12, True, False, False)
    g = GLEnergy(prob, st.n_images)
    a, p1, p2 = _cuda(st.a), _cuda(st.psi_1), _cuda(st.psi_2)
    th0 = np.array([0.0, prob.eta, prob.gamma])
    theta = torch.tensor(th0, requires_grad=True)
    e = g(a, p1, p2, theta)
    grads = []
    for n in range(st.n_images):
        gr, = torch.autograd.grad(e[n], theta, retain_graph=True)
        grads.append(gr.numpy())
    grads = np.array(grads)
    h = 1e-6
    for k in range(3):
        tp, tm = th0.copy(), th0.copy()
        tp[k] += h
        tm[k] -= h
        ep = g(a, p1, p2, torch.tensor(tp)).cpu().numpy()
        em = g(a, p1, p2, torch.tensor(tm)).cpu().numpy()
        fd = (ep - em) / (2 * h)
        np.testing.assert_allclose(grads[:, k], fd, rtol=1e-6, atol=1e-6 * np.abs(fd).max())
    g.close()


def test_field_gradient_matches_directional_difference():
    from mepgl_gb300.autograd import GLEnergy
    prob, st = _case(13, True, False, True)
    g = GLEnergy(prob, st.n_images)
    rng = np.random.default_rng(3)
    x = [_cuda(st.a), _cuda(st.psi_1), _cuda(st.psi_2)]
    v = [torch.tensor(rng.standard_normal(st.a.shape), device="cuda") for _ in range(3)]
    xs = [t.clone().requires_grad_() for t in x]
    e = g(*xs)
    e.sum().backward()
    dirn = sum(float((t.grad * vv).sum()) for t, vv in zip(xs, v))
    h = 1e-6
    ep = g(*[t + h * vv for t, vv in zip(x, v)]).sum().item()
    em = g(*[t - h * vv for t, vv in zip(x, v)]).sum().item()
    assert abs((ep - em) / (2 * h) - dirn) <= 1e-6 * abs(dirn)
    g.close()


def test_config3_full_size_adjoints_and_gradient():
    """512 x 512, 32 images, two components, FP64 (the differentiation
    workload): adjoints against central differences (h = 1e-6) on every image,
    the backward pass against the oracle gradient on two images."""
    from mepgl_gb300.autograd import GLEnergy
    prob, st = W.config3()
    g = GLEnergy(prob, st.n_images)
    a, p1, p2 = _cuda(st.a), _cuda(st.psi_1), _cuda(st.psi_2)
    th0 = np.array([0.0, prob.eta, prob.gamma])
    a_req = a.clone().requires_grad_()
    theta = torch.tensor(th0, requires_grad=True)
    e = g(a_req, p1, p2, theta)
    w = torch.zeros(st.n_images, dtype=torch.float64, device="cuda")
    w[0], w[17] = 1.0, -0.5
    (e * w).sum().backward()
    sub = [0, 17]
    go = cref.Oracle(prob).gradient(st.a[sub], st.psi_1[sub], st.psi_2[sub])
    ga = a_req.grad.cpu().numpy()
    assert relmax(ga[0], go[0][0]) < 1e-12
    assert relmax(ga[17], -0.5 * go[0][1]) < 1e-12
    adj = g.context(th0).param_adjoint()
    h = 1e-6
    for k in range(3):
        tp, tm = th0.copy(), th0.copy()
        tp[k] += h
        tm[k] -= h
        fd = (g(a, p1, p2, torch.tensor(tp)).cpu().numpy() - g(a, p1, p2, torch.tensor(tm)).cpu().numpy()) / (2 * h)
        np.testing.assert_allclose(adj[:, k], fd, rtol=1e-6, atol=1e-6 * np.abs(fd).max())
    np.testing.assert_allclose(theta.grad.numpy(), (w.cpu().numpy()[:, None] * adj).sum(0), rtol=1e-12)
    g.close()


def test_envelope_theorem_on_relaxed_end_states(native):
    """Config 1's end states (Meissner and one vortex) relaxed to stationarity:
    the adjoint difference dF_end/dH - dF_0/dH equals the central difference
    of the re-relaxed energy difference at H +- 1e-4."""
    prob, st = W.config1()
    ends = st.__class__(a=st.a[[0, -1]], psi_1=st.psi_1[[0, -1]])

    def relax(p):
        c = native.StringContext(p, 2, "fp64", line_polynomial=1, line_search=1)
        c.set_state(ends)
        for _ in range(100):
            c.nlcg_steps(100)
        return c

    c0 = relax(prob)
    adj = c0.param_adjoint()[:, 0]
    fe = c0.compute_free_energy()
    _, gr = c0.energy_grad()
    assert max(np.abs(x).max() for x in gr if x is not None) < 1e-4
    eps = 1e-4
    dp = np.diff(relax(prob.with_(h=prob.h + eps)).compute_free_energy())[0]
    dm = np.diff(relax(prob.with_(h=prob.h - eps)).compute_free_energy())[0]
    fd = (dp - dm) / (2 * eps)
    assert abs((adj[1] - adj[0]) - fd) <= 1e-5 * abs(fd), (adj, fd, fe)
