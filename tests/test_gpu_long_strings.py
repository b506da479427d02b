"""GPU: reparametrization of strings with many images on a small lattice.

Past a few hundred images the reparametrization kernels switch to their
long-string forms: the plan works on its global arrays instead of shared
memory (more than about 500 images), the FP64 cubic resample keeps its
columns in the global scratch (more than about 750 images) and the FP32 one
needs more than 48 KB of shared memory, and the arc-length cumulation runs in
one thread (more than 4096 images).  Each form is checked against the C
oracle: arc lengths 1e-13 absolute, FP64 resamples 1e-11 relative, FP32 ones
2e-5.
"""
import numpy as np
import pytest

from mepgl_gb300 import workloads as W
from mepgl_gb300.problem import StringState
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


def long_string(F, n=12, seed=11):
    """F images on a smooth path between the Meissner state and a vortex
    state, with a seeded wiggle so that the images are unevenly spaced."""
    prob, st0 = W.config2(n=n, images=2, margin=2)
    rng = np.random.default_rng(seed)
    t = np.linspace(0.0, 1.0, F)[:, None, None, None]
    wig = np.sin(3 * np.pi * t)

    def path(x):
        return (1 - t) * x[0] + t * x[-1] + 0.05 * wig * rng.standard_normal(x[0].shape)

    return prob, StringState(a=path(st0.a), psi_1=path(st0.psi_1), psi_2=path(st0.psi_2))


def relmax(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def oracle_resample(prob, st, s, cubic):
    o = cref.Oracle(prob)
    F = st.n_images
    return [o.redistribute(s, x, F, cubic=cubic, spline=cref.SPLINE_COMPAT) for x in (st.a, st.psi_1, st.psi_2)]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_cubic_resample_of_800_images(native, precision):
    prob, st = long_string(800)
    c = native.StringContext(prob, st.n_images, precision)
    c.set_state(st)
    s = c.arc_length_jb()
    got0 = c.get_state()   # the fields the context holds (rounded to FP32 in FP32)
    c.redistribute_cubic()
    got = c.get_state()
    want = oracle_resample(prob, got0, s, cubic=True)
    tol = 1e-11 if precision == "fp64" else 2e-5
    for g, w in zip((got.a, got.psi_1, got.psi_2), want):
        assert relmax(g, w) < tol


def test_linear_resample_and_arc_length_of_4200_images(native):
    prob, st = long_string(4200, n=8)
    c = native.StringContext(prob, st.n_images, "fp64")
    c.set_state(st)
    o = cref.Oracle(prob)
    b, j1, j2 = o.jb(st.a, st.psi_1, st.psi_2)
    s_ref = o.arc_length(b, j1, j2)
    s = c.arc_length_jb()
    np.testing.assert_allclose(s, s_ref, atol=1e-13)
    np.testing.assert_allclose(c.arc_length(), o.arc_length(st.a, st.psi_1, st.psi_2), atol=1e-13)
    c.redistribute_linear()
    got = c.get_state()
    want = oracle_resample(prob, st, s, cubic=False)
    for g, w in zip((got.a, got.psi_1, got.psi_2), want):
        assert relmax(g, w) < 1e-12
