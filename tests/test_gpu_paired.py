"""Paired FP64 arithmetic (fp64_arith = MEPGL_FP64_PAIRED): the two NLCG
passes compute in float-float pairs on double fields.  Their per-image
scalars and trajectories agree with IEEE double (the native passes and the
oracle) to the precision of the pairs: energies 1e-11 relative, |g|^2 1e-10,
steps within one grid point of the reference's scan (exact step: 1e-7)."""
import numpy as np
import pytest

from mepgl_gb300 import workloads as W
from mepgl_gb300.problem import PARAM_NAMES
from oracle import cref

pytestmark = pytest.mark.gpu

GRID_STEP = np.log(1.025) * 1.0001


@pytest.fixture(scope="module", autouse=True)
def native():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mepgl_gb300 import build
    build.build()
    from mepgl_gb300 import native as N
    return N


def _case(seed, mc=True, uniform=True, nx=45, ny=30, images=4):
    rng = np.random.default_rng(seed)
    prob = W.random_problem(rng, n=max(nx, ny), multicomponent=mc, uniform=uniform)
    kw = {k: getattr(prob, k)[:ny, :nx].copy() for k in PARAM_NAMES + ("comp_domain", "sc_domain")}
    prob = prob.with_(nx=nx, ny=ny, **kw)
    return prob, W.random_state(rng, prob, images=images)


def _ctx(native, prob, st, paired, **opt):
    c = native.StringContext(prob, st.n_images, "fp64",
                             fp64_arith=native.FP64_PAIRED if paired else native.FP64_NATIVE, **opt)
    c.set_state(st)
    return c


@pytest.mark.parametrize("mc,uniform", [(True, True), (True, False), (False, True)])
def test_first_step_scalars_match_double(native, mc, uniform):
    prob, st = _case(41, mc, uniform)
    o = cref.Oracle(prob)
    e0 = o.energy(st.a, st.psi_1, st.psi_2)
    go = o.gradient(st.a, st.psi_1, st.psi_2)
    g2 = sum(np.sum(g.reshape(st.n_images, -1) ** 2, axis=1) for g in go[: 1 + prob.ncomp])
    # exact steps: a continuous alpha keeps both runs on the same x1
    c = _ctx(native, prob, st, True, line_search=1, line_polynomial=1)
    c.nlcg_steps(2)
    sc = c.image_scalars()
    cn = _ctx(native, prob, st, False, line_search=1, line_polynomial=1)
    cn.nlcg_steps(2)
    sn = cn.image_scalars()
    np.testing.assert_allclose(sc["g_norm2"], sn["g_norm2"], rtol=1e-10)
    np.testing.assert_allclose(sc["fenergy"], sn["fenergy"], rtol=1e-11)
    np.testing.assert_allclose(sc["alpha"], sn["alpha"], rtol=1e-7)
    c1 = _ctx(native, prob, st, True, line_polynomial=1)
    c1.nlcg_steps(1)
    np.testing.assert_allclose(c1.image_scalars()["fenergy"], e0, rtol=1e-11)
    assert np.all(np.isfinite(g2))


def test_paired_trajectory_vs_oracle(native):
    prob, st = _case(42, True, True)
    sv = cref.Oracle(prob).solver(st, ls_mode=1, poly_compat=False)
    c = _ctx(native, prob, st, True, line_search=1, line_polynomial=1)
    for _ in range(3):
        sv.nlcg_steps(2)
        c.nlcg_steps(2)
        r = sv.get()
        sc = c.image_scalars()
        np.testing.assert_allclose(sc["fenergy"], r["fenergy"], rtol=1e-10)
        np.testing.assert_allclose(sc["alpha"], r["alpha"], rtol=1e-7)
    fin = c.get_state()
    assert np.max(np.abs(fin.psi_1 - r["psi_1"])) / np.max(np.abs(r["psi_1"])) < 1e-8


def test_paired_loop_and_batches(native):
    """Mode L iterations on two strings in one context, paired against double."""
    cases = [_case(43, True, True, 40, 28, 5), _case(44, True, True, 33, 36, 4)]
    out = []
    for paired in (True, False):
        b = native.StringBatch([p for p, _ in cases], [s.n_images for _, s in cases], "fp64",
                               fp64_arith=native.FP64_PAIRED if paired else native.FP64_NATIVE, line_search=1,
                               line_polynomial=1)
        for k, (_, s) in enumerate(cases):
            b.set_string_state(k, s)
        for _ in range(3):
            b.loop_iteration("L", 4)
        out.append([b.string_free_energy(k) for k in range(2)])
    for a, d in zip(*out):
        np.testing.assert_allclose(a, d, rtol=1e-9)


@pytest.mark.parametrize("mc", [True, False])
def test_energy_grad_of_a_paired_context_is_ieee_double(native, mc):
    """mepgl_energy_grad returns the IEEE double gradient in every FP64 mode:
    a paired context's gradient equals a native context's bit for bit (the
    float-float gradient-only form serves the refinement's internal gauge
    Hessian only)."""
    prob, st = _case(21 + int(mc), mc=mc)
    out = []
    for paired in (False, True):
        with _ctx(native, prob, st, paired) as c:
            out.append(c.energy_grad())
    (e0, g0), (e1, g1) = out
    np.testing.assert_array_equal(e0, e1)
    for a, b in zip(g0, g1):
        if a is not None:
            np.testing.assert_array_equal(a, b)
