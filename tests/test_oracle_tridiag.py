"""The oracle's tridiagonal solver (oracle/tridiag.h) against LAPACK dgtsv.

The reference solves its cubic-spline systems with cuSPARSE gtsv2
(mepgl/src/interpolation.cu:443-454); the oracle and the CUDA resample plan
use the published LAPACK gtsv algorithm (Gaussian elimination with partial
pivoting) restated in tridiag.h.  This compares that restatement with
scipy's LAPACK dgtsv on random systems that need pivoting and on the
Forsythe-Malcolm-Moler spline matrices of random arc lengths
(interpolation.cu:252-322), with several right-hand sides each.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import cref

lapack = pytest.importorskip("scipy.linalg.lapack")


def _solve(dl, d, du, B):
    """dl[k] = A[k+1][k] (scipy layout, n - 1 entries)."""
    n = d.size
    L = cref.lib()
    f = L.glo_gtsv_d
    f.restype = C.c_int
    f.argtypes = [C.c_int] + [C.c_void_p] * 4 + [C.c_int]
    ours_dl = np.concatenate([[0.0], dl])
    ours_du = np.concatenate([du, [0.0]])
    b = np.ascontiguousarray(B.T, np.float64).copy()      # rhs one after another
    info = f(n, *(np.ascontiguousarray(a).ctypes.data for a in (ours_dl, d, ours_du)), b.ctypes.data, B.shape[1])
    assert info == 0
    return b.T


def _lapack(dl, d, du, B):
    _, _, _, x, info = lapack.dgtsv(dl.copy(), d.copy(), du.copy(), B.copy())
    assert info == 0
    return x


@pytest.mark.parametrize("n", [2, 3, 7, 64, 257])
def test_random_systems_with_pivoting(n):
    rng = np.random.default_rng(n)
    dl, du = rng.normal(size=n - 1), rng.normal(size=n - 1)
    d = 0.3 * rng.normal(size=n)          # weak diagonal: rows get swapped
    B = rng.normal(size=(n, 3))
    x, y = _solve(dl, d, du, B), _lapack(dl, d, du, B)
    np.testing.assert_allclose(x, y, rtol=1e-10, atol=1e-12 * np.max(np.abs(y)))


@pytest.mark.parametrize("F", [4, 5, 16, 64, 300])
def test_spline_matrices_of_random_arc_lengths(F):
    rng = np.random.default_rng(100 + F)
    s = np.concatenate([[0.0], np.cumsum(rng.uniform(0.2, 1.0, F - 1))])
    s /= s[-1]
    h = np.diff(s)                         # h[k-1] = s[k] - s[k-1]
    d = np.empty(F)
    dl, du = np.empty(F - 1), np.empty(F - 1)
    d[0], du[0] = -h[0], h[0]
    for k in range(1, F - 1):
        dl[k - 1], d[k], du[k] = h[k - 1], 2 * (h[k - 1] + h[k]), h[k]
    dl[F - 2], d[F - 1] = h[F - 2], -h[F - 2]
    B = rng.normal(size=(F, 4))
    x, y = _solve(dl, d, du, B), _lapack(dl, d, du, B)
    np.testing.assert_allclose(x, y, rtol=1e-10, atol=1e-12 * np.max(np.abs(y)))
