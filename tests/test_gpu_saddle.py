"""Stationary-point refinement on the GPU (mepgl_refine_stationary).

The plain-method string (64x64, 16 images, FP64) is relaxed on the GPU and
its image 0 and interior energy maximum are refined to a minimum and an
index-1 saddle.  Checks:

* the barrier and both energies against tests/golden/saddle_cfg1.json,
  which the C oracle alone computed on the CPU (string relaxation and the
  numpy restatement of the refinement, oracle/saddle_ref.py): FP64 barrier
  tolerance 1e-8 relative, energies 1e-10;
* at the GPU's saddle, the oracle's own energy (1e-12) and gradient norm
  (a stationary point of the reference functional), and its Morse index by
  an oracle-side Lanczos (exactly one negative curvature);
* dF/dH by the envelope theorem at the refined points against a central
  difference of the re-converged barrier at H +- h;
* minima of a two-component string against the oracle refiner;
* the preconditioned and the plain conjugate gradients (and the two forcing
  terms) reach the same stationary points, the preconditioned one in fewer
  CG iterations.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR
from mepgl_gb300 import workloads as W
from mepgl_gb300.problem import StringState
from oracle import cref, saddle_ref as SR

pytestmark = pytest.mark.gpu

BARRIER_RTOL = 1e-8      # FP64 barrier tolerance
ENERGY_RTOL = 1e-10      # FP64 per-image energy tolerance


@pytest.fixture(scope="module", autouse=True)
def native():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mepgl_gb300 import build
    build.build()
    from mepgl_gb300 import native as N
    return N


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(GOLDEN_DIR, "saddle_cfg1.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def config1_barrier(native):
    from mepgl_gb300 import saddle
    prob, st, fe = saddle.relax_string(1, 1, 600, "fp64")
    res = saddle.refine_barrier(prob, st, fe, g_tol=1e-9, max_newton=40, keep_state=True)
    return prob, st, fe, res


def test_config1_barrier_matches_the_oracle_golden(config1_barrier, golden):
    prob, st, fe, r = config1_barrier
    assert r.converged and r.is_saddle, r.reports
    assert r.seed_image == golden["seed_image"]
    np.testing.assert_allclose(r.barrier, golden["barrier"], rtol=BARRIER_RTOL)
    np.testing.assert_allclose(r.energies[0], golden["e_min"], rtol=ENERGY_RTOL)
    np.testing.assert_allclose(r.energies[1], golden["e_saddle"], rtol=ENERGY_RTOL)
    # the string's own estimate is below the saddle (images on the path sit under it)
    assert r.string_barrier < r.barrier


def test_gpu_saddle_is_an_index1_stationary_point_of_the_oracle(config1_barrier):
    prob, st, fe, r = config1_barrier
    o = cref.Oracle(prob)
    s = r.state
    e = o.energy(s.a, s.psi_1)
    np.testing.assert_allclose(e, r.energies, rtol=1e-12)
    ga, g1, _ = o.gradient(s.a, s.psi_1)
    gn = np.sqrt(np.sum(ga ** 2, axis=(1, 2, 3)) + np.sum(g1 ** 2, axis=(1, 2, 3)))
    assert np.all(gn < 1e-8), gn
    R = SR.Refiner(o)
    xs = R.pack(s.a[1:2], s.psi_1[1:2])
    k = r.seed_image
    tau = R.pack(st.a[k + 1:k + 2] - st.a[k - 1:k], st.psi_1[k + 1:k + 2] - st.psi_1[k - 1:k])
    neg = R.morse_negatives(xs, tau, 40)
    assert len(neg) == 1, neg
    np.testing.assert_allclose(neg[0], r.reports[1]["min_curvature"], rtol=1e-4)


def test_envelope_theorem_dbarrier_dH_at_the_config1_saddle(native, config1_barrier, golden):
    from mepgl_gb300 import saddle
    prob, st, fe, r = config1_barrier
    _, mode = saddle.seed_state(st, r.seed_image)
    h = 1e-3

    def barrier_at(dh):
        p = prob.with_(h=prob.h + dh)
        with native.StringContext(p, 2, "fp64") as c:
            c.set_state(r.state)
            kinds = [native.STATIONARY_MINIMUM, native.STATIONARY_SADDLE]
            rep = c.refine_stationary(kinds, mode, g_tol=1e-10, max_newton=40)
            assert all(x["converged"] for x in rep) and rep[1]["min_curvature"] < 0, rep
            return rep[1]["energy"] - rep[0]["energy"]

    fd = (barrier_at(h) - barrier_at(-h)) / (2 * h)
    np.testing.assert_allclose(r.dbarrier_dH, fd, rtol=1e-5)
    np.testing.assert_allclose(r.dbarrier_dH, golden["dbarrier_dH"], rtol=1e-6)


def test_minima_of_a_two_component_string_match_the_oracle_refiner(native):
    prob, st = W.config2(n=24, images=3)
    sub = StringState(a=st.a[[0, 2]], psi_1=st.psi_1[[0, 2]], psi_2=st.psi_2[[0, 2]])
    with native.StringContext(prob, 2, "fp64") as c:
        c.set_state(sub)
        rep = c.refine_stationary([native.STATIONARY_MINIMUM] * 2, g_tol=1e-9, max_newton=40)
    assert all(x["converged"] for x in rep), rep
    o = cref.Oracle(prob)
    R = SR.Refiner(o)
    for k in range(2):
        x = R.pack(sub.a[k:k + 1], sub.psi_1[k:k + 1], sub.psi_2[k:k + 1])
        _, ref = R.refine(x, SR.MINIMUM, g_tol=1e-9)
        np.testing.assert_allclose(rep[k]["energy"], ref["energy"], rtol=ENERGY_RTOL)


@pytest.mark.parametrize("case", ["thin_film", "tiny"])
def test_minimum_refinement_edge_cases_match_the_oracle_refiner(native, case):
    """A thin film (A fixed: no gauge basis, the A dofs masked out of the
    preconditioner) and a 4 x 4 lattice (too small for the preconditioner's
    probe comb: plain CG) refine image 0 to the oracle refiner's minimum.  On
    16 sites the automatic gauge basis (14 functions) is degenerate, so the
    4 x 4 case runs both refiners without gauge steps."""
    deg = -1
    if case == "thin_film":
        prob, st = W.config1(n=16, images=3)
        prob = prob.with_(thin_film=True)
    else:
        prob, st = W.config1(n=4, images=3, margin=0)
        deg = 0
    sub = StringState(a=st.a[0:1], psi_1=st.psi_1[0:1])
    with native.StringContext(prob, 1, "fp64") as c:
        c.set_state(sub)
        rep = c.refine_stationary([native.STATIONARY_MINIMUM], g_tol=1e-9, max_newton=40, gauge_degree=deg)
    assert rep[0]["converged"], rep
    assert rep[0]["preconditioned"] == (1 if case == "thin_film" else 0), rep
    o = cref.Oracle(prob)
    R = SR.Refiner(o, deg=None if deg < 0 else deg)
    _, ref = R.refine(R.pack(sub.a, sub.psi_1), SR.MINIMUM, g_tol=1e-9)
    np.testing.assert_allclose(rep[0]["energy"], ref["energy"], rtol=ENERGY_RTOL, atol=1e-12)


def test_preconditioned_and_plain_cg_reach_the_same_stationary_points(config1_barrier):
    from mepgl_gb300 import saddle
    prob, st, fe, r = config1_barrier
    runs = {}
    for pc, forcing in ((1, 0), (0, 0), (1, 1)):
        runs[pc, forcing] = saddle.refine_barrier(prob, st, fe, g_tol=1e-9, max_newton=40, adjoint=False,
                                                  precondition=pc, forcing=forcing)
    for key, q in runs.items():
        assert q.converged and q.is_saddle, (key, q.reports)
        assert all(rep["preconditioned"] == key[0] for rep in q.reports), (key, q.reports)
        np.testing.assert_allclose(q.barrier, r.barrier, rtol=1e-10)
        np.testing.assert_allclose(q.energies, r.energies, rtol=1e-12)
    cg = {k: sum(q.cg_iterations) for k, q in runs.items()}
    assert cg[1, 0] < cg[0, 0], cg


def test_refinement_arguments_are_checked(native):
    prob, st = W.config1(n=16, images=3)
    with native.StringContext(prob, 3, "fp32") as c:
        c.set_state(st)
        with pytest.raises(native.MepglError) as e:
            c.refine_stationary([0, 1, 0])
        assert e.value.status == 5          # FP64 contexts only
    with native.StringContext(prob, 3, "fp64") as c:
        c.set_state(st)
        with pytest.raises(native.MepglError) as e:
            c.refine_stationary([0, 1, 0])  # a saddle needs a starting direction
        assert e.value.status == 1
        with pytest.raises(native.MepglError) as e:
            c.refine_stationary([0, 7, 0])
        assert e.value.status == 1
        for bad in (dict(precondition=2), dict(forcing=-1)):
            with pytest.raises(native.MepglError) as e:
                c.refine_stationary([0, 0, 0], **bad)
            assert e.value.status == 1
        rep = c.refine_stationary([2, 2, 2])   # all skipped: nothing changes
        assert all(x["converged"] for x in rep)
        np.testing.assert_array_equal(c.get_state().psi_1, st.psi_1)
