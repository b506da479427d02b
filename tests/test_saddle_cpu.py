"""The CPU restatement of the stationary-point refinement (oracle/saddle_ref.py)
and the committed barrier golden, without a GPU.

* The gauge orbit map U_chi keeps |psi| and shifts A by the lattice
  gradient; a constant chi (a global phase) leaves the energy unchanged.
* The orbit gradient dE/dc = g . J phi matches a central difference of the
  energy along the exact orbit.
* A minimum refinement of a small two-component image converges and lowers
  the energy; at the result the gauge-orbit gradient vanishes too.
* tests/golden/saddle_cfg1.json is self-consistent: the barrier is the
  difference of its energies, the saddle has exactly one negative curvature,
  and it lies above the string's own estimate.
* The CG preconditioner's solve (mepgl_gb300/csrc/refine.cu, k_pc_extend /
  k_pc_scale / k_pc_extract): mirroring a field to 2 ny x 2 nx, a real FFT,
  division by sigma + c_x (2 - 2 cos(pi kx / nx)) + c_y (2 - 2 cos(pi ky / ny))
  and the inverse FFT is the exact inverse of sigma - c_x d_xx - c_y d_yy with
  Neumann (mirror) boundaries, on odd and even lattices.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR
from mepgl_gb300 import workloads as W
from oracle import cref, saddle_ref as SR


@pytest.fixture(scope="module")
def small():
    prob, st = W.config2(n=10, images=2)
    o = cref.Oracle(prob)
    return prob, st, o, SR.Refiner(o, deg=2)


def test_gauge_orbit_keeps_modulus_and_shifts_a(small):
    prob, st, o, R = small
    x = R.pack(st.a[:1], st.psi_1[:1], st.psi_2[:1])
    chi = 0.3 * R.basis[0] + 0.1 * R.basis[4]
    y = R.gauge(x, chi)
    a0, p10, p20 = R.unpack(x)
    a1, p11, p21 = R.unpack(y)
    for p0, p1 in ((p10, p11), (p20, p21)):
        np.testing.assert_allclose(np.hypot(p1[..., 0], p1[..., 1]), np.hypot(p0[..., 0], p0[..., 1]), rtol=1e-13,
                                   atol=1e-15)
    gx, gy = R._cgrad(chi)
    np.testing.assert_allclose(a1[0, ..., 0] - a0[0, ..., 0], gx, atol=1e-14)
    np.testing.assert_allclose(a1[0, ..., 1] - a0[0, ..., 1], gy, atol=1e-14)
    # a global phase is an exact symmetry of the reference functional
    z = R.gauge(x, np.full_like(chi, 0.7))
    np.testing.assert_allclose(R.energy(z), R.energy(x), rtol=1e-13)


def test_orbit_gradient_matches_energy_differences(small):
    prob, st, o, R = small
    x = R.pack(st.a[:1], st.psi_1[:1], st.psi_2[:1])
    gg = R.gauge_grad(x, R.grad(x))
    h = 1e-5
    for m in range(len(R.basis)):
        fd = (R.energy(R.gauge(x, h * R.basis[m])) - R.energy(R.gauge(x, -h * R.basis[m]))) / (2 * h)
        np.testing.assert_allclose(gg[m], fd, rtol=1e-6, atol=1e-9)


def test_minimum_refinement_converges(small):
    prob, st, o, R = small
    x = R.pack(st.a[1:2], st.psi_1[1:2], st.psi_2[1:2])
    e0 = R.energy(x)
    y, rep = R.refine(x, SR.MINIMUM, g_tol=1e-8, max_newton=30)
    assert rep["g_norm"] <= 1e-8
    assert rep["energy"] < e0
    assert np.max(np.abs(R.gauge_grad(y, R.grad(y)))) < 1e-7


def test_saddle_golden_is_consistent():
    with open(os.path.join(GOLDEN_DIR, "saddle_cfg1.json")) as f:
        z = json.load(f)
    assert z["barrier"] == pytest.approx(z["e_saddle"] - z["e_min"], rel=1e-14)
    assert z["min_curvature"] < 0 and len(z["negative_ritz"]) == 1
    assert z["g_min"] <= 1e-9 and z["g_saddle"] <= 1e-9
    assert z["string_barrier"] < z["barrier"]
    assert z["dbarrier_dH"] == pytest.approx(z["dF_dH_saddle"] - z["dF_dH_min"], rel=1e-12)


def _neumann_second_difference(n):
    """-d_xx on n sites with mirror boundaries: tridiag(-1, 2, -1), corners 1."""
    L = 2 * np.eye(n) - np.eye(n, k=1) - np.eye(n, k=-1)
    L[0, 0] = L[-1, -1] = 1.0
    return L


@pytest.mark.parametrize("nx,ny,sigma,cx,cy", [(6, 5, 0.3, 1.0, 0.5), (7, 8, 0.05, 0.0, 1.0), (9, 9, 1.0, 2.0, 2.0)])
def test_mirrored_fft_solve_inverts_the_neumann_model(nx, ny, sigma, cx, cy):
    rng = np.random.default_rng(nx * 100 + ny)
    r = rng.standard_normal((ny, nx))
    M = sigma * np.eye(nx * ny) + cx * np.kron(np.eye(ny), _neumann_second_difference(nx)) + \
        cy * np.kron(_neumann_second_difference(ny), np.eye(nx))
    z_ref = np.linalg.solve(M, r.ravel()).reshape(ny, nx)
    # the device path: mirror, R2C, divide, C2R, top-left block
    e = np.zeros((2 * ny, 2 * nx))
    e[:ny, :nx] = r
    e[:ny, nx:] = r[:, ::-1]
    e[ny:, :] = e[:ny, :][::-1, :]
    ex = 2 - 2 * np.cos(np.pi * np.arange(nx + 1) / nx)
    ey = 2 - 2 * np.cos(np.pi * np.arange(2 * ny) / ny)
    spec = np.fft.rfft2(e) / (sigma + cx * ex[None, :] + cy * ey[:, None])
    z = np.fft.irfft2(spec, s=e.shape)[:ny, :nx]
    np.testing.assert_allclose(z, z_ref, rtol=1e-10, atol=1e-12)
