"""The reference's own CUDA build (its unmodified nlcg.cu and parallel_sum.cu
compiled for this GPU by oracle/ref_cuda_build.py) against this library on the
same input: after the same NLCG steps with the reference's options the
per-image energies of the last step agree.  Skipped where the reference sources were not
staged into baseline/_ref (they come from the reference tree, which only some
machines have)."""
import numpy as np
import pytest

from mepgl_gb300 import workloads as W
from oracle import ref_cuda_build as RC

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def native():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if not RC.staged():
        pytest.skip("reference CUDA sources not staged")
    from mepgl_gb300 import build
    build.build()
    from mepgl_gb300 import native as N
    return N


@pytest.mark.parametrize("cfg, prec, steps, rtol", [(1, "f64", 6, 1e-10), (2, "f32", 2, 2e-5)])
def test_reference_cuda_build_matches_the_library(native, cfg, prec, steps, rtol):
    """Same calls as the reference's loop(): nlcgSteps(1) then nlcgSteps(steps)."""
    prob, st = W.config1(n=64, images=8) if cfg == 1 else W.config2(n=64, images=8)
    warmup = 1
    ref = RC.run(prob, st, prec, steps, warmup)
    assert ref["n"] == prob.nx and ref["images"] == st.n_images
    c = native.StringContext(prob, st.n_images, "fp64" if prec == "f64" else "fp32")
    c.set_state(st)
    c.nlcg_steps(warmup)
    c.nlcg_steps(steps)
    got = c.image_scalars()["fenergy"]        # F before the last update, as the reference reports it
    np.testing.assert_allclose(got, ref["fenergy"], rtol=rtol)
    c.close()
