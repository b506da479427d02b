"""Known-answer and property tests of the C oracle (CPU only)."""
import numpy as np
import pytest

from mepgl_gb300 import workloads as W
from mepgl_gb300.problem import Problem
from oracle import cref


def test_meissner_energy_analytic():
    """psi = sqrt(-a/b), A = 0, uniform H on a full domain: F = H^2 (N-1)^2 dx^2 / 2
    (only the curl term survives); a second component at psi_2 = 0 adds
    (a^2 / 2b)(N-1)^2 dx^2."""
    n, dx, H = 24, 0.5, 0.8
    for mc in (False, True):
        prob = Problem.uniform(n, n, dx, a=(-1.0, -0.6), b=(1.0, 1.0), h=H, multicomponent=mc)
        F = 2
        a = np.zeros((F, n, n, 2))
        p1 = np.zeros((F, n, n, 2)); p1[..., 0] = 1.0
        p2 = np.zeros((F, n, n, 2)) if mc else None
        e = cref.Oracle(prob).energy(a, p1, p2)
        expect = 0.5 * H ** 2 * (n - 1) ** 2 * dx ** 2
        if mc:
            expect += 0.5 * 0.6 ** 2 * (n - 1) ** 2 * dx ** 2
        np.testing.assert_allclose(e, expect, rtol=1e-13)


def test_gradient_is_derivative_of_energy():
    """Central differences (h = 1e-6) of the energy against the gradient, uniform parameters."""
    rng = np.random.default_rng(3)
    prob = W.random_problem(rng, n=8, multicomponent=True)
    st = W.random_state(rng, prob, images=1, amp=0.2)
    o = cref.Oracle(prob)
    g = o.gradient(st.a, st.psi_1, st.psi_2)
    fields = [st.a, st.psi_1, st.psi_2]
    for f in range(3):
        for _ in range(12):
            j, i, c = rng.integers(prob.ny), rng.integers(prob.nx), rng.integers(2)
            hh = 1e-6
            plus = [x.copy() for x in fields]; minus = [x.copy() for x in fields]
            plus[f][0, j, i, c] += hh; minus[f][0, j, i, c] -= hh
            fd = (o.energy(*plus)[0] - o.energy(*minus)[0]) / (2 * hh)
            assert abs(fd - g[f][0, j, i, c]) < 1e-6 * max(1.0, abs(fd)), (f, j, i, c)


def test_global_phase_invariance():
    """A constant U(1) phase on every component leaves the energy unchanged."""
    rng = np.random.default_rng(4)
    prob = W.random_problem(rng, n=10, multicomponent=True)
    st = W.random_state(rng, prob, images=2)
    o = cref.Oracle(prob)
    th = 0.7321
    rot = lambda p: np.stack([p[..., 0] * np.cos(th) - p[..., 1] * np.sin(th),
                              p[..., 0] * np.sin(th) + p[..., 1] * np.cos(th)], axis=-1)
    e0 = o.energy(st.a, st.psi_1, st.psi_2)
    e1 = o.energy(st.a, rot(st.psi_1), rot(st.psi_2))
    np.testing.assert_allclose(e1, e0, rtol=1e-13)


def test_exact_polynomial_first_coefficient_is_directional_derivative():
    """With the exact expansion, B = g . d and F(x + a d) equals the quartic."""
    rng = np.random.default_rng(5)
    prob = W.random_problem(rng, n=10, multicomponent=True)
    st = W.random_state(rng, prob, images=3, amp=0.2)
    d = W.random_state(rng, prob, images=3, amp=0.1)
    o = cref.Oracle(prob)
    g = o.gradient(st.a, st.psi_1, st.psi_2)
    e, poly = o.polynomial(st.a, st.psi_1, st.psi_2, d.a, d.psi_1, d.psi_2, compat=False)
    gd = sum(np.sum(gg * dd, axis=(1, 2, 3)) for gg, dd in zip(g, (d.a, d.psi_1, d.psi_2)))
    np.testing.assert_allclose(poly[:, 0], gd, rtol=1e-11)
    for al in (0.3, 1.1):
        ex = o.energy(st.a + al * d.a, st.psi_1 + al * d.psi_1, st.psi_2 + al * d.psi_2)
        quart = e + poly[:, 0] * al + poly[:, 1] * al ** 2 + poly[:, 2] * al ** 3 + poly[:, 3] * al ** 4
        np.testing.assert_allclose(quart, ex, rtol=1e-12)


def test_compat_polynomial_equals_exact_for_q_minus_one_except_cubic_y():
    """The reference's x-link slip vanishes for q = -1 (the charge its shipped
    configurations use); only the halved y-link cubic coefficient remains."""
    rng = np.random.default_rng(6)
    prob = W.random_problem(rng, n=10, multicomponent=False).with_(q_1=-1.0)
    st = W.random_state(rng, prob, images=2)
    d = W.random_state(rng, prob, images=2, amp=0.1)
    o = cref.Oracle(prob)
    e1, pc = o.polynomial(st.a, st.psi_1, None, d.a, d.psi_1, None, compat=True)
    e2, pe = o.polynomial(st.a, st.psi_1, None, d.a, d.psi_1, None, compat=False)
    np.testing.assert_allclose(pc[:, [0, 1, 3]], pe[:, [0, 1, 3]], rtol=1e-13)
    assert np.all(np.abs(pc[:, 2] - pe[:, 2]) > 0)


def test_exact_line_search_is_first_minimum_of_the_scan():
    """LS_EXACT returns the first local minimum downhill from 0 (a stationary
    point with positive curvature, the quartic non-increasing before it), and
    the reference's 2.5 % scan lands within one grid step of it."""
    o = cref.Oracle(Problem.uniform(4, 4, 0.5))
    rng = np.random.default_rng(7)
    for _ in range(40):
        c = np.array([rng.uniform(1, 10), -rng.uniform(0.1, 5), rng.uniform(-1, 5), rng.uniform(-2, 2),
                      rng.uniform(0.01, 2)])
        a = o.line_search(c[None, :1], c[None, 1:], mode=cref.LS_EXACT)[0]
        a_scan = o.line_search(c[None, :1], c[None, 1:], mode=cref.LS_COMPAT)[0]
        dp = c[1] + 2 * c[2] * a + 3 * c[3] * a ** 2 + 4 * c[4] * a ** 3
        ddp = 2 * c[2] + 6 * c[3] * a + 12 * c[4] * a ** 2
        assert abs(dp) <= 1e-9 * (abs(c[1]) + 1) and ddp > 0
        xs = np.linspace(0, a, 20001)
        f = c[0] + c[1] * xs + c[2] * xs ** 2 + c[3] * xs ** 3 + c[4] * xs ** 4
        assert np.all(np.diff(f) <= 1e-12 * abs(c[0]))
        assert abs(np.log(a / a_scan)) < np.log(1.025) * 1.0001


def test_linear_spline_reproduces_linear_data():
    prob = Problem.uniform(6, 5, 0.5)
    o = cref.Oracle(prob)
    F = 7
    s = np.sort(np.concatenate([[0.0, 1.0], np.random.default_rng(1).uniform(0, 1, F - 2)]))
    base = np.random.default_rng(2).standard_normal((1, 5, 6, 2))
    slope = np.random.default_rng(3).standard_normal((1, 5, 6, 2))
    f = base + slope * s[:, None, None, None]
    out = o.redistribute(s, f, 11)
    sn = np.linspace(0, 1, 11)[:, None, None, None]
    np.testing.assert_allclose(out, base + slope * sn, atol=1e-13)


def test_fmm_cubic_reproduces_cubic_data_and_compat_does_not():
    prob = Problem.uniform(4, 3, 0.5)
    o = cref.Oracle(prob)
    F = 9
    s = np.sort(np.concatenate([[0.0, 1.0], np.random.default_rng(4).uniform(0.05, 0.95, F - 2)]))
    cf = np.random.default_rng(5).standard_normal((4, 1, 3, 4, 2))
    poly = lambda t: cf[0] + cf[1] * t + cf[2] * t ** 2 + cf[3] * t ** 3
    f = np.concatenate([poly(x) for x in s])
    sn = np.linspace(0, 1, 13)
    want = np.concatenate([poly(x) for x in sn])
    fmm = o.redistribute(s, f, 13, cubic=True, spline=cref.SPLINE_FMM)
    np.testing.assert_allclose(fmm, want, atol=1e-11)
    compat = o.redistribute(s, f, 13, cubic=True, spline=cref.SPLINE_COMPAT)
    assert np.max(np.abs(compat - want)) > 1e-4
    # both agree at the nodes' end points
    np.testing.assert_allclose(compat[0], f[0], atol=1e-15)


def test_endpoints_survive_reparametrization():
    prob, st = W.config1(n=16, images=6)
    o = cref.Oracle(prob)
    sv = o.solver(st)
    sv.iteration("L", 0)
    r = sv.get()
    np.testing.assert_array_equal(r["psi_1"][0], st.psi_1[0])
    np.testing.assert_array_equal(r["psi_1"][-1], st.psi_1[-1])


def test_float32_oracle_tracks_float64():
    prob, st = W.config2(n=16, images=4)
    o64 = cref.Oracle(prob)
    o32 = cref.Oracle(prob, np.float32)
    e64 = o64.energy(st.a, st.psi_1, st.psi_2)
    e32 = o32.energy(st.a, st.psi_1, st.psi_2)
    np.testing.assert_allclose(e32, e64, rtol=2e-5)
