"""ctypes wrapper of ``oracle/_ref`` -- the reference's own kernels run on the CPU.

Test infrastructure only: imported by ``tests/`` and by
``tests/golden/make_golden.py``.  The library is built on demand from the
reference sources by ``oracle/ref_build.py`` and exists only where those
sources are present.

Array conventions (shared with ``oracle.cref`` and the CUDA library): a
lattice of N x N sites is stored with x fastest, i.e. numpy shape
``(N_y, N_x)`` indexed ``[j, i]`` (the transpose of the reference's ``.npy``
files, which are indexed ``[i, j]``, mepgl/src/io.cu:69-88).  A field of F
images is ``(F, N, N, 2)`` with the last axis the (x, y) or (Re, Im) pair,
which is exactly the reference's ``real2`` device layout.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import ref_build

_P = C.c_void_p


class _RefParams(C.Structure):
    _fields_ = [(n, _P) for n in (
        "comp_nn", "sc_nn", "a_1", "b_1", "m_xx_1", "m_yy_1", "a_2", "b_2", "m_xx_2", "m_yy_2",
        "h", "q_1", "q_2", "eta", "gamma", "delta")]


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_P)


class RefKernels:
    """One host-compiled variant (N, dx, components, precision, thin film)."""

    def __init__(self, n: int, dx: float, comps: int, prec: str = "f64", film: bool = False):
        self.path = ref_build.build(n, dx, comps, prec, film)
        self.lib = C.CDLL(self.path)
        self.N = n
        self.dx = dx
        self.comps = comps
        self.dtype = np.float64 if prec == "f64" else np.float32
        self.film = film
        assert self.lib.ref_N() == n and self.lib.ref_components() == comps
        self._keep = []

    # ---------------------------------------------------------------- helpers
    def _f(self, a):
        return np.ascontiguousarray(a, dtype=self.dtype)

    def nn_map(self, domain: np.ndarray) -> np.ndarray:
        dom = np.ascontiguousarray(domain, dtype=np.int32)
        out = np.zeros_like(dom)
        self.lib.ref_nn_map(_ptr(dom), _ptr(out))
        return out

    def params(self, prob) -> _RefParams:
        """Parameter block from a ``oracle.problem.Problem``."""
        keep = []

        def arr(x):
            a = self._f(x)
            keep.append(a)
            return _ptr(a)

        comp_nn = self.nn_map(prob.comp_domain)
        sc_nn = self.nn_map(prob.sc_domain)
        keep += [comp_nn, sc_nn]
        p = _RefParams(
            _ptr(comp_nn), _ptr(sc_nn),
            arr(prob.a_1), arr(prob.b_1), arr(prob.m_xx_1), arr(prob.m_yy_1),
            arr(prob.a_2), arr(prob.b_2), arr(prob.m_xx_2), arr(prob.m_yy_2), arr(prob.h),
            arr([prob.q_1]), arr([prob.q_2]), arr([prob.eta]), arr([prob.gamma]), arr([prob.delta]))
        p._keep = keep
        return p

    def _state(self, a, p1, p2):
        a = self._f(a).copy()
        p1 = self._f(p1).copy()
        p2 = self._f(np.zeros_like(p1) if p2 is None else p2).copy()
        return a, p1, p2

    # ---------------------------------------------------------------- kernels
    def free_energy(self, prob, a, p1, p2=None, density=False):
        a, p1, p2 = self._state(a, p1, p2)
        F = a.shape[0]
        out = np.zeros(F, self.dtype)
        dens = np.zeros(a.shape[:3], self.dtype) if density else None
        P = self.params(prob)
        self.lib.ref_free_energy(F, C.byref(P), _ptr(a), _ptr(p1), _ptr(p2), _ptr(out),
                                 _ptr(dens) if density else None)
        return (out, dens) if density else out

    def gradient(self, prob, a, p1, p2=None, maxwell=False):
        a, p1, p2 = self._state(a, p1, p2)
        F = a.shape[0]
        ga, g1, g2 = (np.zeros_like(a) for _ in range(3))
        P = self.params(prob)
        self.lib.ref_gradient(F, C.byref(P), _ptr(a), _ptr(p1), _ptr(p2), _ptr(ga), _ptr(g1), _ptr(g2),
                              int(maxwell))
        return ga, g1, g2

    def polynomial(self, prob, a, p1, p2, da, d1, d2):
        a, p1, p2 = self._state(a, p1, p2)
        da, d1, d2 = self._state(da, d1, d2)
        F = a.shape[0]
        fe = np.zeros(F, self.dtype)
        poly = np.zeros((F, 4), self.dtype)
        P = self.params(prob)
        self.lib.ref_polynomial(F, C.byref(P), _ptr(a), _ptr(p1), _ptr(p2), _ptr(da), _ptr(d1), _ptr(d2),
                                _ptr(fe), _ptr(poly))
        return fe, poly

    def line_search(self, fenergy, poly):
        fe = self._f(fenergy)
        po = self._f(poly)
        alpha = np.zeros(fe.shape[0], self.dtype)
        self.lib.ref_line_search(fe.shape[0], _ptr(fe), _ptr(po), _ptr(alpha))
        return alpha

    def jb(self, prob, a, p1, p2=None):
        a, p1, p2 = self._state(a, p1, p2)
        F = a.shape[0]
        b = np.zeros(a.shape[:3], self.dtype)
        j1 = np.zeros_like(a)
        j2 = np.zeros_like(a)
        P = self.params(prob)
        self.lib.ref_jb(F, C.byref(P), _ptr(a), _ptr(p1), _ptr(p2), _ptr(b), _ptr(j1), _ptr(j2))
        return b, j1, j2

    def arc_length(self, a, p1, p2=None):
        a, p1, p2 = self._state(a, p1, p2)
        s = np.zeros(a.shape[0], self.dtype)
        self.lib.ref_arc_length(a.shape[0], _ptr(a), _ptr(p1), _ptr(p2), _ptr(s))
        return s

    def arc_length_jb(self, b, j1, j2=None):
        b = self._f(b)
        j1 = self._f(j1)
        j2 = self._f(np.zeros_like(j1) if j2 is None else j2)
        s = np.zeros(b.shape[0], self.dtype)
        self.lib.ref_arc_length_jb(b.shape[0], _ptr(b), _ptr(j1), _ptr(j2), _ptr(s))
        return s

    def redistribute(self, s, f, f_new: int, cubic=False):
        s = self._f(s)
        f = self._f(f)
        out = np.zeros((f_new,) + f.shape[1:], self.dtype)
        fn = self.lib.ref_redistribute_cubic if cubic else self.lib.ref_redistribute_linear
        fn(f.shape[0], _ptr(s), _ptr(f), int(f_new), _ptr(out))
        return out

    def loop(self, prob, a, p1, p2, mode: str, iterations: int, relaxation_steps: int, nlcg=True,
             history=False):
        """One run of the reference binary's ``loop()``; returns the final state and scalars."""
        a, p1, p2 = self._state(a, p1, p2)
        F = a.shape[0]
        fe, al, gn, s, sjb = (np.zeros(F, self.dtype) for _ in range(5))
        hist = np.zeros((iterations, F), self.dtype) if history else None
        P = self.params(prob)
        self.lib.ref_loop(F, C.byref(P), _ptr(a), _ptr(p1), _ptr(p2), C.c_char(mode.encode()),
                          int(iterations), int(relaxation_steps), int(nlcg), _ptr(fe), _ptr(al), _ptr(gn),
                          _ptr(s), _ptr(sjb), _ptr(hist) if history else None)
        out = dict(a=a, psi_1=p1, psi_2=p2, fenergy=fe, alpha=al, g_norm2=gn, s=s, s_jb=sjb)
        if history:
            out["history"] = hist
        return out


_cache: dict = {}


def available() -> bool:
    return ref_build.reference_available() or os.path.isdir(ref_build.OUT_ROOT)


def load_ref(n: int, dx: float, comps: int, prec: str = "f64", film: bool = False) -> RefKernels:
    key = (n, dx, comps, prec, film)
    if key not in _cache:
        _cache[key] = RefKernels(n, dx, comps, prec, film)
    return _cache[key]
