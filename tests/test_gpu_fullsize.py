"""Parity at the benchmark configurations' full sizes.

* Plain-method string (64x64, dx = 0.5, 16 images, FP64): the library runs
  the reference's loop() in mode L (5 x 10 NLCG steps) and mode C (3 x 10)
  with the reference's options, against tests/golden/ref_cfg1_full.json,
  written by the reference's own kernels host-compiled
  (tests/golden/make_fullsize_golden.py): per-image energy 1e-10, barrier
  max_n F_n - F_0 1e-8 relative, the per-iteration energies 1e-10.
* Large string (2048x2048, dx = 0.25, disk of radius 1000, two components
  with unequal charges): energy and gradient of two images against the C
  oracle in FP64 (1e-12), and four FP32 NLCG steps of a four-image string
  against the FP32 oracle (energies 2e-5, the tolerance of the FP32 tests).
* Sweep strings 0..3 (N ~ U{96..384}, F ~ U{24..64}) at full size in one
  batched context: FP64 energies against the oracle (1e-12) and two FP32
  steps per string against the FP32 oracle.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR
from mepgl_gb300 import workloads as W
from oracle import cref

pytestmark = pytest.mark.gpu

ENERGY_RTOL = 1e-10      # FP64 per-image energy tolerance
BARRIER_RTOL = 1e-8      # FP64 barrier tolerance
FP32_RTOL = 2e-5


@pytest.fixture(scope="module", autouse=True)
def native():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mepgl_gb300 import build
    build.build()
    from mepgl_gb300 import native as N
    return N


def _rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.abs(b)))


@pytest.mark.parametrize("mode", ["L", "C"])
def test_config1_full_size_loop_against_the_reference_kernels(native, mode):
    with open(os.path.join(GOLDEN_DIR, "ref_cfg1_full.json")) as f:
        z = json.load(f)
    prob, st = W.config1()
    c = native.StringContext(prob, st.n_images, "fp64")
    c.set_state(st)
    assert _rel(c.compute_free_energy(), z["fenergy"]) < 1e-12
    ref = z[f"loop_{mode}"]
    hist = []
    for _ in range(ref["iterations"]):
        c.loop_iteration(mode, ref["relax"])
        hist.append(c.image_scalars()["fenergy"])
    assert _rel(hist, ref["history"]) < ENERGY_RTOL
    fe = c.compute_free_energy()
    assert _rel(fe, ref["final_energy"]) < ENERGY_RTOL
    want = np.asarray(ref["final_energy"])
    barrier, want_barrier = fe.max() - fe[0], want.max() - want[0]
    assert abs(barrier - want_barrier) <= BARRIER_RTOL * abs(want_barrier)
    c.close()


def test_config5_full_lattice_against_the_oracle(native):
    prob, st = W.config5(images=4)
    o64 = cref.Oracle(prob)
    two = st.__class__(a=st.a[[0, 3]], psi_1=st.psi_1[[0, 3]], psi_2=st.psi_2[[0, 3]])
    c = native.StringContext(prob, 2, "fp64")
    c.set_state(two)
    e, g = c.energy_grad()
    np.testing.assert_allclose(e, o64.energy(two.a, two.psi_1, two.psi_2), rtol=1e-12)
    want = o64.gradient(two.a, two.psi_1, two.psi_2)
    for got, ref in zip(g, want):
        assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
    c.close()
    o32 = cref.Oracle(prob, np.float32)
    c = native.StringContext(prob, 4, "fp32", line_search=1, line_polynomial=1)
    c.set_state(st)
    sv = o32.solver(st, ls_mode=1, poly_compat=False)
    for _ in range(4):
        c.nlcg_steps(1)
        sv.nlcg_steps(1)
        got, ref = c.image_scalars()["fenergy"], sv.get()["fenergy"]
        np.testing.assert_allclose(got, ref, rtol=FP32_RTOL)
    c.close()


def test_config4_full_size_strings_against_the_oracle(native):
    cases = [W.config4_string(s) for s in range(4)]
    b = native.StringBatch([p for p, _ in cases], [s.n_images for _, s in cases], "fp64")
    for k, (p, s) in enumerate(cases):
        b.set_string_state(k, s)
    for k, (p, s) in enumerate(cases):
        np.testing.assert_allclose(b.string_free_energy(k), cref.Oracle(p).energy(s.a, s.psi_1), rtol=1e-12)
    b.close()
    b = native.StringBatch([p for p, _ in cases], [s.n_images for _, s in cases], "fp32", line_search=1,
                           line_polynomial=1)
    for k, (p, s) in enumerate(cases):
        b.set_string_state(k, s)
    b.nlcg_steps(2)
    for k, (p, s) in enumerate(cases):
        sv = cref.Oracle(p, np.float32).solver(s, ls_mode=1, poly_compat=False)
        sv.nlcg_steps(2)
        np.testing.assert_allclose(b.string_scalars(k)["fenergy"], sv.get()["fenergy"], rtol=FP32_RTOL)
    b.close()


def test_large_string_barrier_leg_extracts_the_seed_images(native):
    """mepgl_gb300.large's time-to-barrier leg on a small disk string: the
    four images copied out of the FP32 device string reach the FP64
    refinement intact (its first barrier, before any Newton step, is the FP32
    string's F_k - F_0 re-evaluated in FP64), and the leg reports a finite
    refinement."""
    import argparse

    import torch
    from mepgl_gb300 import large
    a = argparse.Namespace(n=128, images=8, barrier=4, relax=2, g_tol=1e-8, max_newton=2)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    r = large.barrier_leg(a, stream)
    assert 1 <= r["seed_image"] <= a.images - 2
    assert [p for _, _, p in r["trace"]].count("string") == 1
    first = [b for _, b, p in r["trace"] if p == "refine"][0]
    e0 = abs(r["energies"][0])
    assert abs(first - r["string_barrier"]) <= 1e-3 * abs(r["string_barrier"]) + 1e-5 * e0, (first, r)
    assert r["newton"] <= a.max_newton and np.all(np.isfinite(r["g_norms"])) and np.isfinite(r["barrier"])
