"""The gauge-link (Peierls) functional on the oracle: exact invariance under
a random lattice gauge transform, gradient against central differences,
and agreement with the reference discretisation as dx -> 0."""
import numpy as np

from mepgl_gb300 import workloads as W
from mepgl_gb300.problem import Problem, StringState
from oracle import cref


def lattice_gauge(prob, st, chi):
    """psi_c -> psi_c exp(i q_c chi), A_e(s) -> A_e(s) + (chi(s+e) - chi(s)) / dx
    (chi: (F, ny, nx); links leaving the lattice keep their value)."""
    a = st.a.copy()
    a[..., :-1, 0] += (chi[..., 1:] - chi[..., :-1]) / prob.dx
    a[..., :-1, :, 1] += (chi[..., 1:, :] - chi[..., :-1, :]) / prob.dx
    out = [a]
    for p, q in ((st.psi_1, prob.q_1), (st.psi_2, prob.q_2)):
        if p is None:
            out.append(None)
            continue
        z = (p[..., 0] + 1j * p[..., 1]) * np.exp(1j * q * chi)
        out.append(np.stack([z.real, z.imag], axis=-1))
    return StringState(a=out[0], psi_1=out[1], psi_2=out[2])


def _case(seed, mc=True, film=False):
    rng = np.random.default_rng(seed)
    prob = W.random_problem(rng, n=14, multicomponent=mc, thin_film=film, uniform=False)
    prob = prob.with_(q_2=prob.q_1)       # eta and delta couple psi_1 psi_2*: invariant for equal charges
    return rng, prob, W.random_state(rng, prob, images=3)


def test_link_energy_is_exactly_gauge_invariant():
    for mc in (True, False):
        rng, prob, st = _case(21, mc)
        o = cref.Oracle(prob)
        chi = rng.uniform(-4, 4, (st.n_images, prob.ny, prob.nx))
        g = lattice_gauge(prob, st, chi)
        e0 = o.energy_link(st.a, st.psi_1, st.psi_2)
        np.testing.assert_allclose(o.energy_link(g.a, g.psi_1, g.psi_2), e0, rtol=1e-13)
        # the reference's linearised differences are not invariant for large chi
        assert np.max(np.abs(o.energy(g.a, g.psi_1, g.psi_2) / o.energy(st.a, st.psi_1, st.psi_2) - 1)) > 1e-2


def test_link_gradient_matches_central_differences():
    for mc, film in ((True, False), (False, False), (True, True)):
        rng, prob, st = _case(22, mc, film)
        o = cref.Oracle(prob)
        g = o.gradient_link(st.a, st.psi_1, st.psi_2)
        fields = [st.a, st.psi_1] + ([st.psi_2] if mc else [])
        h = 1e-6
        for f, arr in enumerate(fields):
            if film and f == 0:
                continue            # thin film: A is frozen and its gradient reported as zero
            for _ in range(12):
                idx = tuple(int(rng.integers(0, s)) for s in arr.shape)
                plus = [x.copy() for x in fields]
                minus = [x.copy() for x in fields]
                plus[f][idx] += h
                minus[f][idx] -= h
                fd = (o.energy_link(*plus)[idx[0]] - o.energy_link(*minus)[idx[0]]) / (2 * h)
                assert abs(fd - g[f][idx]) <= 2e-7 * max(1.0, abs(fd)), (f, idx, fd, g[f][idx])


def test_link_and_reference_agree_as_dx_shrinks():
    """Smooth fields on a fixed physical square: the two discretisations
    differ by O(dx)."""
    L = 6.0
    diffs = []
    for n in (24, 48, 96):
        dx = L / n
        x = (np.arange(n) + 0.5) * dx
        X, Y = np.meshgrid(x, x, indexing="xy")
        psi = (0.8 + 0.1 * np.sin(2 * np.pi * X / L)) * np.exp(1j * (2 * np.pi * Y / L + 0.3 * np.sin(np.pi * X / L)))
        a = np.stack([0.2 * np.cos(2 * np.pi * Y / L), 0.1 * np.sin(2 * np.pi * X / L)], axis=-1)
        prob = Problem.uniform(n, n, dx, h=0.5)
        st = StringState(a=a[None], psi_1=np.stack([psi.real, psi.imag], axis=-1)[None])
        o = cref.Oracle(prob)
        e_ref = o.energy(st.a, st.psi_1)[0]
        e_link = o.energy_link(st.a, st.psi_1)[0]
        diffs.append(abs(e_link - e_ref) / abs(e_ref))
    assert diffs[0] > diffs[1] > diffs[2]
    assert diffs[1] / diffs[2] > 1.8
