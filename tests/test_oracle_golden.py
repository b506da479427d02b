"""The C oracle against the golden vectors produced by the reference's own kernels.

These run anywhere (CPU, no reference tree needed): the fixtures in
tests/golden/ were generated by tests/golden/make_golden.py from the
reference kernels host-compiled in oracle/_ref.
"""
import numpy as np

from oracle import cref


def rel(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_energy(golden):
    prob, st, z = golden
    e = cref.Oracle(prob).energy(st.a, st.psi_1, st.psi_2)
    assert np.max(np.abs(e - z["fenergy"]) / np.abs(z["fenergy"])) < 1e-13


def test_gradient(golden):
    prob, st, z = golden
    g = cref.Oracle(prob).gradient(st.a, st.psi_1, st.psi_2)
    assert rel(g[0], z["grad_a"]) < 1e-13
    assert rel(g[1], z["grad_psi_1"]) < 1e-13
    if prob.multicomponent:
        assert rel(g[2], z["grad_psi_2"]) < 1e-13


def test_polynomial_and_line_search(golden):
    prob, st, z = golden
    o = cref.Oracle(prob)
    e, poly = o.polynomial(st.a, st.psi_1, st.psi_2, z["dir_a"], z["dir_psi_1"], z["dir_psi_2"], compat=True)
    assert np.max(np.abs(e - z["poly_energy"]) / np.abs(z["poly_energy"])) < 1e-13
    for k in range(4):
        assert rel(poly[:, k], z["poly"][:, k]) < 1e-12
    # the step is a point of the geometric grid: equal given the reference's own coefficients
    np.testing.assert_array_equal(o.line_search(z["poly_energy"], z["poly"]), z["alpha"])


def test_jb_and_arc_lengths(golden):
    prob, st, z = golden
    o = cref.Oracle(prob)
    b, j1, j2 = o.jb(st.a, st.psi_1, st.psi_2)
    assert rel(b, z["b"]) < 1e-13 and rel(j1, z["j_1"]) < 1e-13
    if prob.multicomponent:
        assert rel(j2, z["j_2"]) < 1e-13
    flds = [st.a, st.psi_1] + ([st.psi_2] if prob.multicomponent else [])
    np.testing.assert_allclose(o.arc_length(*flds), z["s"], rtol=0, atol=1e-14)
    jfl = [z["b"], z["j_1"]] + ([z["j_2"]] if prob.multicomponent else [])
    np.testing.assert_allclose(o.arc_length(*jfl), z["s_jb"], rtol=0, atol=1e-14)


def test_redistribution(golden):
    prob, st, z = golden
    o = cref.Oracle(prob)
    F = st.a.shape[0]
    for fnew in (F, F + 3):
        lin = o.redistribute(z["s_jb"], st.psi_1, fnew)
        assert rel(lin, z[f"linear_{fnew}"]) < 1e-14
        cub = o.redistribute(z["s_jb"], st.psi_1, fnew, cubic=True, spline=cref.SPLINE_COMPAT)
        assert rel(cub, z[f"cubic_{fnew}"]) < 1e-12


def test_loop_trajectories(golden):
    """Whole runs of loop() in each mode: final state, energies, steps, arc lengths."""
    prob, st, z = golden
    o = cref.Oracle(prob)
    modes = sorted({k.split("_")[1] for k in z if k.startswith("loop_") and k.endswith("_cfg")})
    assert modes
    for mode in modes:
        iters, relax = (int(v) for v in z[f"loop_{mode}_cfg"])
        sv = o.solver(st)
        hist = []
        for _ in range(iters):
            sv.iteration(mode, relax)
            hist.append(sv.get()["fenergy"])
        r = sv.get()
        ref_hist = z[f"loop_{mode}_history"]
        assert np.max(np.abs(np.array(hist) - ref_hist) / np.abs(ref_hist)) < 1e-10, mode
        assert rel(r["psi_1"], z[f"loop_{mode}_psi_1"]) < 1e-9, mode
        assert rel(r["a"], z[f"loop_{mode}_a"]) < 1e-9, mode
        # the step length is a point of the 2.5 % grid; equal within one grid point
        ra = np.abs(np.log(r["alpha"] / z[f"loop_{mode}_alpha"]))
        assert np.all(ra < 0.0247), mode
        if mode in "LC":
            np.testing.assert_allclose(r["s_jb"], z[f"loop_{mode}_s_jb"], atol=1e-12)
