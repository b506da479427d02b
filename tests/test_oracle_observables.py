"""The observables restatement on CPU: the winding loop visits every edge
step once, and a vortex inside the loop winds by 2 pi (the linearised phase
steps converge to the angle as the loop grows)."""
import numpy as np

from oracle import observables as O


def test_loop_is_closed_and_counter_clockwise():
    steps = O.loop_sites(7, 5, inset=1)
    assert len(steps) == 2 * (5 - 1) + 2 * (3 - 1)
    for (a, b), (c, _) in zip(steps, steps[1:] + steps[:1]):
        assert b == c
    assert steps[0][0] == (1, 1) and steps[0][1] == (2, 1)


def test_vortex_winds_by_two_pi_and_meissner_by_zero():
    n = 64
    jj, ii = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    th = np.arctan2(jj - 31.7, ii - 32.3)
    vortex = np.stack([np.cos(th), np.sin(th)], axis=-1)[None]
    flat = np.stack([np.ones((n, n)), np.zeros((n, n))], axis=-1)[None]
    w = O.winding(np.concatenate([vortex, flat]), inset=2)
    assert abs(w[0] - 2 * np.pi) < 0.01 and abs(w[1]) < 1e-12
    assert np.all(np.isnan(O.winding(np.zeros((1, 8, 8, 2)))))


def test_flux_of_uniform_field():
    b = np.full((2, 5, 6), 0.7)
    np.testing.assert_allclose(O.flux(b, 0.5), 0.7 * 30 * 0.25)
