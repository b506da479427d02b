"""GPU: staged state uploads (mepgl_stage_state + mepgl_set_state with
MEPGL_STAGED) give exactly the context that a plain mepgl_set_state gives,
also when NLCG steps run while the staged copy is in flight, and a stage
that was not installed is replaced by the next one."""
import numpy as np
import pytest

from mepgl_gb300 import workloads as W

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


def pinned(st, dtype):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(x, dtype)).pin_memory() for x in (st.a, st.psi_1, st.psi_2)]


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_staged_state_equals_set_state(native, precision):
    dt = np.float32 if precision == "fp32" else np.float64
    prob, st1 = W.config2(n=40, images=6, seed=5)
    _, st2 = W.config2(n=40, images=6, seed=6)
    ref = native.StringContext(prob, st1.n_images, precision)
    ref.set_state(st2)
    ref.nlcg_steps(4)
    want_e = ref.image_scalars()["fenergy"]
    want = ref.get_state()

    c = native.StringContext(prob, st1.n_images, precision)
    c.set_state(st1)
    h1, h2 = pinned(st1, dt), pinned(st2, dt)
    c.stage_state(*(h.data_ptr() for h in h1))   # replaced below, never installed
    c.stage_state(*(h.data_ptr() for h in h2))
    c.nlcg_steps(3)                              # runs while the copy is in flight
    c.set_staged_state()
    got0 = c.get_state()
    for g, w in zip((got0.a, got0.psi_1, got0.psi_2), (st2.a, st2.psi_1, st2.psi_2)):
        np.testing.assert_array_equal(g, np.asarray(w, dt))
    c.nlcg_steps(4)
    np.testing.assert_array_equal(c.image_scalars()["fenergy"], want_e)
    got = c.get_state()
    np.testing.assert_array_equal(got.psi_1, want.psi_1)
    np.testing.assert_array_equal(got.a, want.a)


def test_set_staged_state_without_stage_fails(native):
    prob, st = W.config2(n=24, images=4)
    c = native.StringContext(prob, st.n_images, "fp64")
    c.set_state(st)
    with pytest.raises(native.MepglError):
        c.set_staged_state()
