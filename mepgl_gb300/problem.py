"""Problem description of a gauged Ginzburg-Landau string.

A :class:`Problem` carries everything the reference bakes into its generated
headers and reads from ``input_data/`` (mepgl/src/config.cuh,
mepgl/src/io.cu:10-126): lattice size and spacing, the two domain masks,
per-site GL parameters, the charges and couplings, the component count and
the thin-film switch.  A :class:`StringState` holds the F images of the
fields (A, psi_1[, psi_2]).

Layout (used by the CUDA library, the C-ABI and the oracle alike): site
(i, j) is stored at ``i + nx*j`` -- x fastest -- so a lattice array has numpy
shape ``(ny, nx)`` indexed ``[j, i]``.  That is the transpose of the
reference's ``.npy`` files, which are indexed ``[i, j]`` (meshgrid
``indexing="ij"``, mepgl/mepgl_lib/builder.py:34); the transposition done by
the reference's loader (io.cu:69-88) is done by :mod:`mepgl_gb300.npyio`.
A field of F images is ``(F, ny, nx, 2)`` with the last axis the (x, y) or
(Re, Im) pair -- the reference's ``real2`` device layout.
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace

import numpy as np

PARAM_NAMES = ("a_1", "b_1", "m_xx_1", "m_yy_1", "a_2", "b_2", "m_xx_2", "m_yy_2", "h")


@dataclass
class Problem:
    nx: int
    ny: int
    dx: float
    comp_domain: np.ndarray
    sc_domain: np.ndarray
    a_1: np.ndarray
    b_1: np.ndarray
    m_xx_1: np.ndarray
    m_yy_1: np.ndarray
    a_2: np.ndarray
    b_2: np.ndarray
    m_xx_2: np.ndarray
    m_yy_2: np.ndarray
    h: np.ndarray
    q_1: float = 1.0
    q_2: float = 1.0
    eta: float = 0.0
    gamma: float = 0.0
    delta: float = 0.0
    multicomponent: bool = False
    thin_film: bool = False

    @property
    def ncomp(self) -> int:
        return 2 if self.multicomponent else 1

    @property
    def sites(self) -> int:
        return self.nx * self.ny

    def validate(self) -> None:
        shape = (self.ny, self.nx)
        for name in ("comp_domain", "sc_domain") + PARAM_NAMES:
            a = getattr(self, name)
            if np.shape(a) != shape:
                raise ValueError(f"{name} has shape {np.shape(a)}, expected {shape}")
        if self.nx < 2 or self.ny < 2:
            raise ValueError("lattice must be at least 2 x 2")
        if not (self.dx > 0):
            raise ValueError("dx must be positive")

    def with_(self, **kw) -> "Problem":
        return replace(self, **kw)

    @staticmethod
    def uniform(nx: int, ny: int, dx: float, *, a=(-1.0, -1.0), b=(1.0, 1.0), m_xx=(1.0, 1.0),
                m_yy=(1.0, 1.0), h=0.0, q=(1.0, 1.0), eta=0.0, gamma=0.0, delta=0.0,
                multicomponent=False, thin_film=False, comp_domain=None, sc_domain=None) -> "Problem":
        """Uniform parameters on a rectangular lattice (masks default to all-ones).

        As in the reference launcher (mepgl/config.py:91-114), the applied
        field array is ``h * comp_domain``.
        """
        ones = np.ones((ny, nx))
        comp = np.ones((ny, nx), np.int32) if comp_domain is None else np.asarray(comp_domain, np.int32)
        sc = comp.copy() if sc_domain is None else np.asarray(sc_domain, np.int32)
        p = Problem(
            nx=nx, ny=ny, dx=float(dx), comp_domain=comp, sc_domain=sc,
            a_1=a[0] * ones, b_1=b[0] * ones, m_xx_1=m_xx[0] * ones, m_yy_1=m_yy[0] * ones,
            a_2=a[1] * ones, b_2=b[1] * ones, m_xx_2=m_xx[1] * ones, m_yy_2=m_yy[1] * ones,
            h=h * comp.astype(np.float64), q_1=float(q[0]), q_2=float(q[1]), eta=float(eta),
            gamma=float(gamma), delta=float(delta), multicomponent=bool(multicomponent),
            thin_film=bool(thin_film))
        p.validate()
        return p


@dataclass
class StringState:
    """F images of (A, psi_1[, psi_2]); each array is (F, ny, nx, 2)."""

    a: np.ndarray
    psi_1: np.ndarray
    psi_2: np.ndarray | None = None
    extra: dict = field(default_factory=dict)

    @property
    def n_images(self) -> int:
        return int(self.a.shape[0])

    def astype(self, dtype) -> "StringState":
        return StringState(self.a.astype(dtype), self.psi_1.astype(dtype),
                           None if self.psi_2 is None else self.psi_2.astype(dtype))

    def copy(self) -> "StringState":
        return self.astype(self.a.dtype)


def neighbour_codes(domain: np.ndarray) -> np.ndarray:
    """8-bit neighbour code per site (bit order 0:+x 1:+x+y 2:+y 3:-x+y 4:-x
    5:-x-y 6:-y 7:+x-y), as buildNearestNeighbourMap (mepgl/src/nlcg.cu:48-103):
    a bit is set when both the site and that neighbour are in the domain."""
    d = np.asarray(domain) != 0
    ny, nx = d.shape
    out = np.zeros((ny, nx), np.uint8)
    offs = [(1, 0), (1, 1), (0, 1), (-1, 1), (-1, 0), (-1, -1), (0, -1), (1, -1)]
    pad = np.zeros((ny + 2, nx + 2), bool)
    pad[1:-1, 1:-1] = d
    for bit, (di, dj) in enumerate(offs):
        nb = pad[1 + dj:1 + dj + ny, 1 + di:1 + di + nx]
        out |= ((d & nb).astype(np.uint8) << bit)
    return out
