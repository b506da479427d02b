"""Failure detection of the library on the GPU, without a GPU fault.

Non-finite data is a host-side input here: a NaN or infinity written into
the state that is uploaded.  Every kernel loop is bounded by counts, not by
values (the line-search scan runs a fixed grid, the exact search two Newton
steps per root, the resample walk ends at an infinite sentinel), so NaN
fields only produce NaN numbers.  The library reports them instead of
returning NaN energies as the reference does:

* after NLCG steps a small launch checks every image's energy and |g|^2;
  the next synchronising call returns MEPGL_ERR_NAN naming the image;
* a string of zero arc length (all images equal), where the reference
  divides 0 by 0 (mepgl/src/interpolation.cu:126-140), returns
  MEPGL_ERR_NAN and a linear resample keeps the images;
* two equal adjacent images (a zero-length segment) resample to finite
  fields;
* a cubic reparametrization of fewer than four images is an argument error.

After each error the context is still usable.
"""
import numpy as np
import pytest

from mepgl_gb300 import workloads as W

pytestmark = pytest.mark.gpu

NAN_STATUS, ARG_STATUS = 3, 1


@pytest.fixture(scope="module", autouse=True)
def native():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mepgl_gb300 import build
    build.build()
    from mepgl_gb300 import native as N
    return N


def _ctx(native, prob, st, precision="fp64", **opt):
    c = native.StringContext(prob, st.n_images, precision, **opt)
    c.set_state(st)
    return c


def _with_nan(st, image, value=np.nan):
    bad = st.__class__(a=st.a.copy(), psi_1=st.psi_1.copy(), psi_2=None if st.psi_2 is None else st.psi_2.copy())
    bad.psi_1[image, 7, 9, 0] = value
    return bad


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_nan_fields_are_reported_after_nlcg_steps(native, precision):
    prob, st = W.config2(n=24, images=5)
    c = _ctx(native, prob, _with_nan(st, 3), precision, line_polynomial=native.POLY_EXACT)
    c.nlcg_steps(3)                      # asynchronous: the check runs on the device
    with pytest.raises(native.MepglError) as e:
        c.image_scalars()
    assert e.value.status == NAN_STATUS and "image 3" in str(e.value)
    # the flag was consumed; a finite state steps normally afterwards
    c.set_state(st)
    c.nlcg_steps(3)
    assert np.all(np.isfinite(c.image_scalars()["fenergy"]))
    c.close()


def test_infinite_field_in_a_batch_names_the_string(native):
    prob, st = W.config1(n=20, images=4)
    prob2, st2 = W.config1(n=24, images=6)
    b = native.StringBatch([prob, prob2], [4, 6], "fp64")
    b.set_string_state(0, st)
    b.set_string_state(1, _with_nan(st2, 4, np.inf))
    b.nlcg_steps(2)
    with pytest.raises(native.MepglError) as e:
        b.synchronize()
    assert e.value.status == NAN_STATUS and "string 1 image 4" in str(e.value)
    b.close()


def test_free_energy_of_nan_fields_is_an_error(native):
    prob, st = W.config1(n=20, images=4)
    c = _ctx(native, prob, _with_nan(st, 1))
    with pytest.raises(native.MepglError) as e:
        c.compute_free_energy()
    assert e.value.status == NAN_STATUS and "image 1" in str(e.value)
    c.close()


def test_string_of_equal_images_has_no_arc_length(native):
    prob, st = W.config1(n=20, images=5)
    same = st.__class__(a=np.repeat(st.a[:1], 5, axis=0), psi_1=np.repeat(st.psi_1[:1], 5, axis=0))
    c = _ctx(native, prob, same)
    for metric in (native.METRIC_FIELDS, native.METRIC_JB):
        with pytest.raises(native.MepglError) as e:
            c.arc_length(metric)
        assert e.value.status == NAN_STATUS and "arc length" in str(e.value)
    with pytest.raises(native.MepglError) as e:
        c.redistribute_linear()
    assert e.value.status == NAN_STATUS
    got = c.get_state()          # the resample kept every image exactly
    np.testing.assert_array_equal(got.psi_1, same.psi_1)
    np.testing.assert_array_equal(got.a, same.a)
    with pytest.raises(native.MepglError) as e:
        c.loop_iteration("L", 2)
    assert e.value.status == NAN_STATUS
    c.set_state(st)              # usable again with a proper string
    c.loop_iteration("L", 2)
    assert np.all(np.isfinite(c.compute_free_energy()))
    c.close()


def test_equal_adjacent_images_resample_to_finite_fields(native):
    prob, st = W.config1(n=20, images=6)
    dup = st.__class__(a=st.a.copy(), psi_1=st.psi_1.copy())
    dup.a[1], dup.psi_1[1] = dup.a[0], dup.psi_1[0]
    c = _ctx(native, prob, dup, metric=native.METRIC_FIELDS)
    s = c.arc_length()
    assert s[0] == s[1] == 0.0 and s[-1] == 1.0
    c.redistribute_linear()
    got = c.get_state()
    assert np.all(np.isfinite(got.psi_1)) and np.all(np.isfinite(got.a))
    np.testing.assert_array_equal(got.psi_1[0], dup.psi_1[0])
    c.close()


def test_cubic_reparametrization_needs_four_images(native):
    prob, st = W.config1(n=20, images=3)
    c = _ctx(native, prob, st)
    with pytest.raises(native.MepglError) as e:
        c.redistribute_cubic()
    assert e.value.status == ARG_STATUS and "at least 4 images" in str(e.value)
    with pytest.raises(native.MepglError) as e:
        c.loop_iteration("C", 1)
    assert e.value.status == ARG_STATUS
    c.loop_iteration("L", 1)     # the context is unchanged and still usable
    c.close()
