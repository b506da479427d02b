"""Batched strings: one context advancing several strings with the same
launches gives, string by string, bit-identical results to one context per
string (every per-image reduction runs in a fixed order that does not depend
on where the image sits in the batch), and matches the oracle."""
import numpy as np
import pytest

from mepgl_gb300 import workloads as W
from mepgl_gb300.problem import PARAM_NAMES
from oracle import cref

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


def _rect(rng, nx, ny, images, uniform=True, mc=True):
    prob = W.random_problem(rng, n=max(nx, ny), multicomponent=mc, uniform=uniform)
    kw = {k: getattr(prob, k)[:ny, :nx].copy() for k in PARAM_NAMES + ("comp_domain", "sc_domain")}
    prob = prob.with_(nx=nx, ny=ny, **kw)
    return prob, W.random_state(rng, prob, images=images)


def _singles(native, cases, precision, **opt):
    out = []
    for prob, st in cases:
        c = native.StringContext(prob, st.n_images, precision, **opt)
        c.set_state(st)
        out.append(c)
    return out


def _batch(native, cases, precision, **opt):
    b = native.StringBatch([p for p, _ in cases], [s.n_images for _, s in cases], precision, **opt)
    for k, (_, st) in enumerate(cases):
        b.set_string_state(k, st)
    return b


def _assert_same(b, singles):
    for k, c in enumerate(singles):
        np.testing.assert_array_equal(b.string_free_energy(k), c.compute_free_energy())
        sb, sc = b.get_string_state(k), c.get_state()
        np.testing.assert_array_equal(sb.a, sc.a)
        np.testing.assert_array_equal(sb.psi_1, sc.psi_1)
        if sc.psi_2 is not None:
            np.testing.assert_array_equal(sb.psi_2, sc.psi_2)


@pytest.mark.parametrize("opts", [dict(), dict(line_search=1, line_polynomial=1, spline=1)])
def test_ragged_batch_equals_single_strings(native, opts):
    rng = np.random.default_rng(77)
    cases = [_rect(rng, 37, 21, 5), _rect(rng, 64, 40, 7, uniform=False), _rect(rng, 18, 33, 4)]
    b = _batch(native, cases, "fp64", **opts)
    singles = _singles(native, cases, "fp64", **opts)
    assert len(b) == 3 and b.string_info(1) == dict(nx=64, ny=40, n_images=7)
    b.nlcg_steps(5)
    for c in singles:
        c.nlcg_steps(5)
    _assert_same(b, singles)
    for mode in "LC":
        b.loop_iteration(mode, 4)
        for c in singles:
            c.loop_iteration(mode, 4)
        _assert_same(b, singles)
    for k, c in enumerate(singles):
        sb, sc = b.string_scalars(k), c.image_scalars()
        for key in sb:
            np.testing.assert_array_equal(sb[key], sc[key])
        np.testing.assert_array_equal(b.string_arc_length(k), c.arc_length())


def test_batch_against_oracle(native):
    rng = np.random.default_rng(78)
    cases = [_rect(rng, 24, 24, 4), _rect(rng, 30, 17, 3)]
    b = _batch(native, cases, "fp64", line_search=1, line_polynomial=1)
    b.nlcg_steps(6)
    for k, (prob, st) in enumerate(cases):
        sv = cref.Oracle(prob).solver(st, ls_mode=1, poly_compat=False)
        sv.nlcg_steps(6)
        np.testing.assert_allclose(b.string_scalars(k)["fenergy"], sv.get()["fenergy"], rtol=1e-11)


def test_more_strings_than_one_launch_holds(native):
    """20 single-component FP32 strings (sweep strings shrunk to 24..40 sites
    and 3..6 images): two launch groups, each string as if alone."""
    cases = []
    for s in range(20):
        rng = np.random.default_rng(s)
        cases.append(W.config4_string(s, n=int(rng.integers(24, 41)), images=int(rng.integers(3, 7))))
    b = _batch(native, cases, "fp32", line_polynomial=1)
    singles = _singles(native, cases, "fp32", line_polynomial=1)
    for it in (4, 3):
        b.nlcg_steps(it)
        for c in singles:
            c.nlcg_steps(it)
    _assert_same(b, singles)
    b.loop_iteration("L", 3)
    for c in singles:
        c.loop_iteration("L", 3)
    _assert_same(b, singles)


def test_batch_rejects_mixed_component_counts(native):
    rng = np.random.default_rng(79)
    cases = [_rect(rng, 16, 16, 3), _rect(rng, 16, 16, 3, mc=False)]
    with pytest.raises(native.MepglError):
        native.StringBatch([p for p, _ in cases], [3, 3], "fp64")
    b = _batch(native, [cases[0], cases[0]], "fp64")
    with pytest.raises(native.MepglError):
        b.string_info(2)
    with pytest.raises(ValueError):
        b.redistribute_linear(5)
