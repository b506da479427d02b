"""GPU parity: the CUDA library (through the C ABI) against the reference's
golden vectors and against the C oracle.

Tolerances (FP64): per-image energies 1e-12 relative, gradients 1e-12 of
their max-norm, arc lengths 1e-13 absolute, trajectories 1e-10 relative on
energies (the reference's step is a point of a 2.5 % geometric grid, so a
step may legitimately differ by one grid point; it is compared within one
grid step).  FP32 runs are compared with the FP32 oracle at 2e-5 relative.
"""
import numpy as np
import pytest

from mepgl_gb300 import workloads as W
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


def make(prob, st, precision="fp64", **opt):
    from mepgl_gb300.native import StringContext
    c = StringContext(prob, st.n_images, precision, **opt)
    c.set_state(st)
    return c


def relmax(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


GRID_STEP = np.log(1.025) * 1.0001


# ----------------------------------------------------------------- goldens
def test_energy_golden(golden):
    prob, st, z = golden
    e = make(prob, st).compute_free_energy()
    np.testing.assert_allclose(e, z["fenergy"], rtol=1e-12)


def test_gradient_golden(golden):
    prob, st, z = golden
    _, g = make(prob, st).energy_grad()
    assert relmax(g[0], z["grad_a"]) < 1e-12
    assert relmax(g[1], z["grad_psi_1"]) < 1e-12
    if prob.multicomponent:
        assert relmax(g[2], z["grad_psi_2"]) < 1e-12


def test_jb_and_arc_length_golden(golden):
    prob, st, z = golden
    c = make(prob, st)
    b, j1, j2 = c.compute_jb()
    assert relmax(b, z["b"]) < 1e-12 and relmax(j1, z["j_1"]) < 1e-12
    if prob.multicomponent:
        assert relmax(j2, z["j_2"]) < 1e-12
    np.testing.assert_allclose(c.arc_length(), z["s"], atol=1e-13)
    np.testing.assert_allclose(c.arc_length_jb(), z["s_jb"], atol=1e-13)


@pytest.mark.parametrize("cubic", [False, True])
def test_redistribution_golden(golden, cubic):
    prob, st, z = golden
    F = st.n_images
    for fnew in (F, F + 3):
        c = make(prob, st)
        if cubic:
            c.redistribute_cubic(fnew)
        else:
            c.redistribute_linear(fnew)
        got = c.get_state().psi_1
        assert got.shape[0] == fnew
        want = z[f"{'cubic' if cubic else 'linear'}_{fnew}"]
        assert relmax(got, want) < 1e-11, fnew


@pytest.mark.parametrize("cubic", [False, True])
def test_redistribution_golden_fp32(golden, cubic):
    """FP32 fields: the linear resample in float, the cubic one in float
    arithmetic as the reference's FP32 build computes its spline (plan and
    factors in double); against the reference kernels' FP64 goldens."""
    prob, st, z = golden
    F = st.n_images
    for fnew in (F, F + 3):
        c = make(prob, st, "fp32")
        if cubic:
            c.redistribute_cubic(fnew)
        else:
            c.redistribute_linear(fnew)
        got = c.get_state().psi_1
        assert got.shape[0] == fnew
        want = z[f"{'cubic' if cubic else 'linear'}_{fnew}"]
        assert relmax(got, want) < 2e-5, fnew


def test_loop_golden(golden):
    """Whole runs of the reference's loop() in each mode, compat options."""
    prob, st, z = golden
    modes = sorted({k.split("_")[1] for k in z if k.startswith("loop_") and k.endswith("_cfg")})
    for mode in modes:
        iters, relax = (int(v) for v in z[f"loop_{mode}_cfg"])
        c = make(prob, st)
        hist = []
        for _ in range(iters):
            c.loop_iteration(mode, relax)
            hist.append(c.image_scalars()["fenergy"])
        sc = c.image_scalars()
        fin = c.get_state()
        ref_hist = z[f"loop_{mode}_history"]
        assert np.max(np.abs(np.array(hist) - ref_hist) / np.abs(ref_hist)) < 1e-10, mode
        assert relmax(fin.psi_1, z[f"loop_{mode}_psi_1"]) < 1e-8, mode
        assert relmax(fin.a, z[f"loop_{mode}_a"]) < 1e-8, mode
        assert np.all(np.abs(np.log(sc["alpha"] / z[f"loop_{mode}_alpha"])) < GRID_STEP), mode


# ------------------------------------------------------------ vs C oracle
CASES = [
    dict(n=(37, 37), mc=True, film=False, uniform=True),
    dict(n=(40, 23), mc=False, film=False, uniform=True),
    dict(n=(33, 9), mc=True, film=True, uniform=True),
    dict(n=(21, 30), mc=True, film=False, uniform=False),
    dict(n=(2, 2), mc=False, film=False, uniform=True),
]


def _case(i):
    spec = CASES[i]
    rng = np.random.default_rng(500 + i)
    nx, ny = spec["n"]
    prob = W.random_problem(rng, n=max(nx, ny), multicomponent=spec["mc"], thin_film=spec["film"],
                            uniform=spec["uniform"])
    # crop to the rectangle
    from mepgl_gb300.problem import PARAM_NAMES
    kw = {k: getattr(prob, k)[:ny, :nx].copy() for k in PARAM_NAMES + ("comp_domain", "sc_domain")}
    prob = prob.with_(nx=nx, ny=ny, **kw)
    st = W.random_state(rng, prob, images=3)
    return prob, st


@pytest.mark.parametrize("i", range(len(CASES)))
def test_energy_gradient_vs_oracle(i):
    prob, st = _case(i)
    o = cref.Oracle(prob)
    c = make(prob, st)
    e, g = c.energy_grad()
    np.testing.assert_allclose(e, o.energy(st.a, st.psi_1, st.psi_2), rtol=1e-12)
    go = o.gradient(st.a, st.psi_1, st.psi_2)
    for k in range(1 + prob.ncomp):
        assert relmax(g[k], go[k]) < 1e-12, k


@pytest.mark.parametrize("i", range(len(CASES) - 1))
@pytest.mark.parametrize("opts", [dict(), dict(line_search=1, line_polynomial=1)])
def test_nlcg_steps_vs_oracle(i, opts):
    prob, st = _case(i)
    ls = opts.get("line_search", 0)
    compat = opts.get("line_polynomial", 0) == 0
    sv = cref.Oracle(prob).solver(st, ls_mode=ls, poly_compat=compat)
    c = make(prob, st, **opts)
    for k in range(3):
        sv.nlcg_steps(2)
        c.nlcg_steps(2)
        r = sv.get()
        sc = c.image_scalars()
        np.testing.assert_allclose(sc["fenergy"], r["fenergy"], rtol=1e-11)
        if ls == 0:
            assert np.all(np.abs(np.log(sc["alpha"] / r["alpha"])) < GRID_STEP)
        else:
            np.testing.assert_allclose(sc["alpha"], r["alpha"], rtol=1e-9)
    fin = c.get_state()
    assert relmax(fin.psi_1, r["psi_1"]) < 1e-9


@pytest.mark.parametrize("i", range(len(CASES) - 1))   # the 2 x 2 case converges to round-off: its step is arbitrary
@pytest.mark.parametrize("maxwell", [False, True])
def test_fp32_nlcg_steps_vs_oracle_fp32(i, maxwell):
    """The FP32 NLCG passes (the warp-strip kernels, with the packed stencils
    for two components) against the FP32 oracle, on the ragged, thin-film,
    and per-site cases.  Exact line polynomial and exact line search
    keep the step continuous in the data, so rounding differences stay
    small: energies 2e-5 relative, steps 1e-3, fields 1e-4 of their max-norm
    after six steps; Maxwell-only steps leave psi untouched."""
    prob, st = _case(i)
    o = cref.Oracle(prob, np.float32)
    scale = np.max(np.abs(o.energy(st.a, st.psi_1, st.psi_2)))   # energies may converge to round-off
    sv = o.solver(st, ls_mode=1, poly_compat=False)
    c = make(prob, st, precision="fp32", line_search=1, line_polynomial=1)
    for k in range(3):
        sv.nlcg_steps(2, maxwell=maxwell)
        c.nlcg_steps(2, maxwell=maxwell)
        r = sv.get()
        sc = c.image_scalars()
        np.testing.assert_allclose(sc["fenergy"], r["fenergy"], rtol=2e-5, atol=2e-5 * scale)
        np.testing.assert_allclose(sc["alpha"], r["alpha"], rtol=1e-3)
    fin = c.get_state()
    assert relmax(fin.a, r["a"]) < 1e-4
    assert relmax(fin.psi_1, r["psi_1"]) < 1e-4
    if maxwell:
        np.testing.assert_array_equal(fin.psi_1, st.psi_1.astype(np.float32))


@pytest.mark.parametrize("mc", [True, False])
def test_fused_fp32_steps_equal_pass_kernels(mc):
    """The fused persistent launch runs the same tile code with the same
    partial-sum order as the two pass kernels: identical results, bit for
    bit, over calls of odd and even step counts (ragged lattice, several
    tiles per image, two strings in one batch)."""
    from mepgl_gb300.native import StringBatch, FP32_STEPS_FUSED, FP32_STEPS_PASSES
    rng = np.random.default_rng(77)
    probs, sts = [], []
    for n in (70, 45):
        prob = W.random_problem(rng, n=n, multicomponent=mc)
        probs.append(prob)
        sts.append(W.random_state(rng, prob, images=5))
    out = []
    for mode in (FP32_STEPS_FUSED, FP32_STEPS_PASSES):
        b = StringBatch(probs, [5, 5], "fp32", line_polynomial=1, fp32_steps=mode)
        for i, st in enumerate(sts):
            b.set_string_state(i, st)
        for k in (3, 4, 1):
            b.nlcg_steps(k)
        out.append([(b.string_scalars(i)["fenergy"], b.get_string_state(i).psi_1, b.get_string_state(i).a)
                    for i in range(2)])
    for (e0, p0, a0), (e1, p1, a1) in zip(*out):
        np.testing.assert_array_equal(e0, e1)
        np.testing.assert_array_equal(p0, p1)
        np.testing.assert_array_equal(a0, a1)


def test_fused_waits_are_bounded_and_reported():
    """A fused launch whose queue skips the gradient items: every direction
    item waits for an image stage that nothing sets, gives up after its poll
    limit and raises the device status flag, which the host reads back.  The
    context is unharmed: its next steps equal those of a fresh context."""
    import time
    from mepgl_gb300.native import FP32_STEPS_FUSED
    prob, st = W.config2(n=40, images=4)
    a = make(prob, st, precision="fp32", line_polynomial=1, fp32_steps=FP32_STEPS_FUSED)
    t0 = time.perf_counter()
    assert a.fused_wait_selftest()
    assert time.perf_counter() - t0 < 30.0
    b = make(prob, st, precision="fp32", line_polynomial=1, fp32_steps=FP32_STEPS_FUSED)
    a.nlcg_steps(3)
    b.nlcg_steps(3)
    np.testing.assert_array_equal(a.image_scalars()["fenergy"], b.image_scalars()["fenergy"])
    np.testing.assert_array_equal(a.get_state().psi_1, b.get_state().psi_1)


def test_graph_and_direct_launches_agree():
    prob, st = _case(0)
    a = make(prob, st, use_graphs=1)
    b = make(prob, st, use_graphs=0)
    for k in (4, 3, 5):
        a.nlcg_steps(k)
        b.nlcg_steps(k)
    np.testing.assert_array_equal(a.image_scalars()["fenergy"], b.image_scalars()["fenergy"])
    np.testing.assert_array_equal(a.get_state().psi_1, b.get_state().psi_1)


def test_deterministic_reductions():
    prob, st = W.config2(n=48, images=5)
    r = []
    for _ in range(2):
        c = make(prob, st)
        c.nlcg_steps(6)
        r.append((c.image_scalars()["fenergy"], c.get_state().psi_2))
    np.testing.assert_array_equal(r[0][0], r[1][0])
    np.testing.assert_array_equal(r[0][1], r[1][1])


@pytest.mark.parametrize("mode", "LC")
def test_modes_with_fmm_spline_and_exact_step_vs_oracle(mode):
    prob, st = W.config1(n=24, images=6)
    sv = cref.Oracle(prob).solver(st, ls_mode=1, poly_compat=False)
    c = make(prob, st, line_search=1, line_polynomial=1, spline=1)
    for _ in range(3):
        sv.iteration(mode, 5, spline=1)
        c.loop_iteration(mode, 5)
    np.testing.assert_allclose(c.image_scalars()["fenergy"], sv.get()["fenergy"], rtol=1e-10)


def test_maxwell_mode_freezes_psi():
    prob, st = W.config2(n=20, images=3)
    c = make(prob, st)
    c.nlcg_steps(4, maxwell=True)
    fin = c.get_state()
    np.testing.assert_array_equal(fin.psi_1, st.psi_1)
    np.testing.assert_array_equal(fin.psi_2, st.psi_2)
    assert np.max(np.abs(fin.a - st.a)) > 0


def test_fp32_vs_oracle_fp32():
    prob, st = W.config2(n=32, images=4)
    o = cref.Oracle(prob, np.float32)
    c = make(prob, st, precision="fp32")
    e, g = c.energy_grad()
    np.testing.assert_allclose(e, o.energy(st.a, st.psi_1, st.psi_2), rtol=2e-6)
    go = o.gradient(st.a, st.psi_1, st.psi_2)
    for k in range(3):
        assert relmax(g[k], go[k]) < 1e-5


def test_precision_switch_keeps_state():
    prob, st = W.config2(n=24, images=4)
    c = make(prob, st, precision="fp32", line_polynomial=1)
    c.nlcg_steps(10)
    s32 = c.get_state()
    c.set_precision("fp64")
    s64 = c.get_state()
    assert s64.psi_1.dtype == np.float64
    np.testing.assert_array_equal(s64.psi_1, s32.psi_1.astype(np.float64))
    e64 = c.compute_free_energy()
    c.nlcg_steps(10)
    assert np.all(c.compute_free_energy() <= e64 + 1e-9)


def test_invalid_arguments_raise():
    from mepgl_gb300.native import MepglError
    prob, st = W.config1(n=8, images=3)
    c = make(prob, st)
    with pytest.raises(MepglError):
        c.loop_iteration("X", 1)
    with pytest.raises(MepglError):
        c.redistribute_cubic()      # cubic needs at least 4 images
    with pytest.raises(MepglError):
        c.reset_cg(2, 99)


def test_full_size_mixed_precision_config():
    """The benchmark workload at full size (256 x 256, 64 images, two
    components): FP32 and FP64 energies agree, the exact-polynomial NLCG
    decreases every image's energy, and the CUDA energy equals the oracle's
    on a few images."""
    prob, st = W.config2()
    c64 = make(prob, st)
    e64 = c64.compute_free_energy()
    c32 = make(prob, st, precision="fp32")
    np.testing.assert_allclose(c32.compute_free_energy(), e64, rtol=1e-5)
    sub = st.__class__(a=st.a[:3], psi_1=st.psi_1[:3], psi_2=st.psi_2[:3])
    np.testing.assert_allclose(cref.Oracle(prob).energy(sub.a, sub.psi_1, sub.psi_2), e64[:3], rtol=1e-12)
    c = make(prob, st, precision="fp32", line_polynomial=1)
    c.nlcg_steps(20)
    assert np.all(c.compute_free_energy() < e64)
