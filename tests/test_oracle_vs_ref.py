"""The C oracle against the reference's own kernels on fresh random problems.

Needs the reference tree (the kernels are host-compiled from it by
oracle/ref_build.py); skipped elsewhere.  The golden-vector tests cover the
same ground without the reference.
"""
import numpy as np
import pytest

from mepgl_gb300 import workloads as W
from oracle import cref, ref_build

pytestmark = pytest.mark.skipif(not ref_build.reference_available(), reason="reference sources absent")


@pytest.mark.parametrize("seed", range(4))
@pytest.mark.parametrize("comps,film,uniform", [(1, False, True), (2, False, True), (2, True, True),
                                                (2, False, False), (1, True, False)])
def test_kernels_match_reference(seed, comps, film, uniform):
    from oracle import refkernels
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(9, 20))
    prob = W.random_problem(rng, n=n, multicomponent=comps == 2, thin_film=film, uniform=uniform)
    st = W.random_state(rng, prob, images=3)
    R = refkernels.load_ref(n, prob.dx, comps, "f64", film)
    o = cref.Oracle(prob)
    p2 = st.psi_2 if comps == 2 else np.zeros_like(st.psi_1)
    np.testing.assert_allclose(o.energy(st.a, st.psi_1, p2), R.free_energy(prob, st.a, st.psi_1, p2), rtol=1e-13)
    for mine, ref in zip(o.gradient(st.a, st.psi_1, p2), R.gradient(prob, st.a, st.psi_1, p2)):
        assert np.max(np.abs(mine - ref)) <= 1e-13 * max(np.max(np.abs(ref)), 1e-300)
    d = W.random_state(rng, prob, images=3, amp=0.05)
    d2 = d.psi_2 if comps == 2 else np.zeros_like(d.psi_1)
    e1, p1 = o.polynomial(st.a, st.psi_1, p2, d.a, d.psi_1, d2, compat=True)
    e2, pr = R.polynomial(prob, st.a, st.psi_1, p2, d.a, d.psi_1, d2)
    np.testing.assert_allclose(e1, e2, rtol=1e-13)
    np.testing.assert_allclose(p1, pr, rtol=1e-11, atol=1e-13 * np.max(np.abs(pr)))
    for mine, ref in zip(o.jb(st.a, st.psi_1, p2), R.jb(prob, st.a, st.psi_1, p2)):
        np.testing.assert_allclose(mine, ref, rtol=1e-13, atol=1e-14)


@pytest.mark.parametrize("mode", "SMLC")
def test_loop_matches_reference(mode):
    from oracle import refkernels
    prob, st = W.config1(n=20, images=6, seed=7)
    R = refkernels.load_ref(20, prob.dx, 1, "f64", False)
    r = R.loop(prob, st.a, st.psi_1, None, mode, 3, 4, history=True)
    sv = cref.Oracle(prob).solver(st)
    for _ in range(3):
        sv.iteration(mode, 4)
    o = sv.get()
    np.testing.assert_allclose(o["fenergy"], r["fenergy"], rtol=1e-12)
    np.testing.assert_allclose(o["psi_1"], r["psi_1"], atol=1e-11)
