"""ctypes wrapper of the C oracle ``oracle/gl_oracle.c`` (TEST INFRASTRUCTURE).

Only ``tests/``, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
import this module.  Arrays follow :mod:`mepgl_gb300.problem`'s layout.
Per-image scalars are float64 in both precisions.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(LIB_DIR, "libgl_oracle.so")
# The timed CPU baseline: the same source optimised (-O3, FMA contraction
# allowed, unrolled), so its results differ from the checker's in the last
# bits.  No -march=native: the library must build alike on every host.
LIB_FAST = os.path.join(LIB_DIR, "libgl_oracle_fast.so")
SOURCES = ("gl_oracle.c", "gl_oracle_impl.h", "gl_oracle.h", "tridiag.h")
FAST_FLAGS = ["-O3", "-ffp-contract=fast", "-funroll-loops"]

_lock = threading.Lock()
_lib = None
_lib_fast = None

LS_COMPAT, LS_EXACT = 0, 1
SPLINE_COMPAT, SPLINE_FMM = 0, 1


def build(force: bool = False, fast: bool = False) -> str:
    """Compile the oracle with the platform's C compiler: the checker (no FMA
    contraction, identical results on x86-64 and AArch64) or, with fast=True,
    the optimised build that the CPU baseline times."""
    src = [os.path.join(HERE, s) for s in SOURCES]
    path = LIB_FAST if fast else LIB_PATH
    if not force and os.path.isfile(path):
        if os.path.getmtime(path) >= max(os.path.getmtime(s) for s in src):
            return path
    os.makedirs(LIB_DIR, exist_ok=True)
    tmp = path + f".{os.getpid()}.tmp"
    flags = ["-std=gnu11"] + FAST_FLAGS if fast else ["-std=c11", "-O2", "-ffp-contract=off"]
    subprocess.run([os.environ.get("CC", "gcc")] + flags + ["-fPIC", "-shared", "-fopenmp", "-o", tmp, src[0],
                                                          "-lm"], check=True)
    os.replace(tmp, path)
    return path


def lib(fast: bool = False):
    global _lib, _lib_fast
    with _lock:
        if fast:
            if _lib_fast is None:
                _lib_fast = C.CDLL(build(fast=True))
            return _lib_fast
        if _lib is None:
            _lib = C.CDLL(build())
    return _lib


def threads(fast: bool = False) -> int:
    """Host threads the oracle uses (OpenMP over images)."""
    return int(lib(fast).glo_max_threads())


def set_threads(n: int) -> None:
    lib().glo_set_threads(int(n))


_P = C.c_void_p


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


def _problem_struct(real):
    class Prob(C.Structure):
        _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("ncomp", C.c_int), ("thin_film", C.c_int),
                    ("dx", real), ("comp_nn", _P), ("sc_nn", _P),
                    ("a", _P * 2), ("b", _P * 2), ("mxx", _P * 2), ("myy", _P * 2), ("h", _P),
                    ("q", real * 2), ("eta", real), ("gamma", real), ("delta", real)]
    return Prob


_PROB = {np.float64: _problem_struct(C.c_double), np.float32: _problem_struct(C.c_float)}


class Oracle:
    """The C oracle bound to one problem and one precision."""

    def __init__(self, prob, dtype=np.float64, fast: bool = False):
        from mepgl_gb300.problem import neighbour_codes  # layout helper, no compute
        self.prob = prob
        self.dtype = np.dtype(dtype).type
        self.sfx = "_d" if self.dtype is np.float64 else "_f"
        self.L = lib(fast)
        f = lambda x: np.ascontiguousarray(x, dtype=self.dtype)
        self._keep = [
            np.ascontiguousarray(neighbour_codes(prob.comp_domain)),
            np.ascontiguousarray(neighbour_codes(prob.sc_domain)),
            f(prob.a_1), f(prob.a_2), f(prob.b_1), f(prob.b_2), f(prob.m_xx_1), f(prob.m_xx_2),
            f(prob.m_yy_1), f(prob.m_yy_2), f(prob.h)]
        k = self._keep
        S = _PROB[self.dtype]()
        S.nx, S.ny, S.ncomp, S.thin_film = prob.nx, prob.ny, prob.ncomp, int(prob.thin_film)
        S.dx = prob.dx
        S.comp_nn, S.sc_nn = _ptr(k[0]), _ptr(k[1])
        S.a[0], S.a[1] = _ptr(k[2]), _ptr(k[3])
        S.b[0], S.b[1] = _ptr(k[4]), _ptr(k[5])
        S.mxx[0], S.mxx[1] = _ptr(k[6]), _ptr(k[7])
        S.myy[0], S.myy[1] = _ptr(k[8]), _ptr(k[9])
        S.h = _ptr(k[10])
        S.q[0], S.q[1] = prob.q_1, prob.q_2
        S.eta, S.gamma, S.delta = prob.eta, prob.gamma, prob.delta
        self.S = S

    def _fn(self, name):
        return getattr(self.L, name + self.sfx)

    def _f(self, a):
        return np.ascontiguousarray(a, dtype=self.dtype)

    def _state(self, a, p1, p2):
        a = self._f(a)
        p1 = self._f(p1)
        p2 = self._f(np.zeros_like(p1) if p2 is None else p2)
        return a, p1, p2

    def energy(self, a, p1, p2=None):
        a, p1, p2 = self._state(a, p1, p2)
        out = np.zeros(a.shape[0])
        self._fn("glo_energy")(C.byref(self.S), a.shape[0], _ptr(a), _ptr(p1), _ptr(p2), _ptr(out))
        return out

    def gradient(self, a, p1, p2=None, maxwell=False):
        a, p1, p2 = self._state(a, p1, p2)
        ga, g1, g2 = (np.zeros_like(a) for _ in range(3))
        self._fn("glo_gradient")(C.byref(self.S), a.shape[0], _ptr(a), _ptr(p1), _ptr(p2), _ptr(ga), _ptr(g1),
                                 _ptr(g2), int(maxwell))
        return ga, g1, g2

    def energy_link(self, a, p1, p2=None):
        """Per-image energy of the gauge-link (Peierls) discretisation."""
        a, p1, p2 = self._state(a, p1, p2)
        out = np.zeros(a.shape[0])
        self._fn("glo_energy_link")(C.byref(self.S), a.shape[0], _ptr(a), _ptr(p1), _ptr(p2), _ptr(out))
        return out

    def gradient_link(self, a, p1, p2=None, maxwell=False):
        a, p1, p2 = self._state(a, p1, p2)
        ga, g1, g2 = (np.zeros_like(a) for _ in range(3))
        self._fn("glo_gradient_link")(C.byref(self.S), a.shape[0], _ptr(a), _ptr(p1), _ptr(p2), _ptr(ga), _ptr(g1),
                                      _ptr(g2), int(maxwell))
        return ga, g1, g2

    def param_adjoint(self, a, p1, p2=None):
        """(F, 3): per-image dF/dH (uniform shift of h), dF/deta, dF/dgamma at fixed fields."""
        a, p1, p2 = self._state(a, p1, p2)
        out = np.zeros((a.shape[0], 3))
        self._fn("glo_param_adjoint")(C.byref(self.S), a.shape[0], _ptr(a), _ptr(p1), _ptr(p2), _ptr(out))
        return out

    def polynomial(self, a, p1, p2, da, d1, d2, compat=True):
        a, p1, p2 = self._state(a, p1, p2)
        da, d1, d2 = self._state(da, d1, d2)
        F = a.shape[0]
        e = np.zeros(F)
        poly = np.zeros((F, 4))
        self._fn("glo_polynomial")(C.byref(self.S), F, _ptr(a), _ptr(p1), _ptr(p2), _ptr(da), _ptr(d1), _ptr(d2),
                                   int(compat), _ptr(e), _ptr(poly))
        return e, poly

    def line_search(self, energy, poly, mode=LS_COMPAT):
        e = np.ascontiguousarray(energy, np.float64)
        p = np.ascontiguousarray(poly, np.float64)
        out = np.zeros(e.shape[0])
        self._fn("glo_line_search")(e.shape[0], _ptr(e), _ptr(p), int(mode), _ptr(out))
        return out

    def jb(self, a, p1, p2=None):
        a, p1, p2 = self._state(a, p1, p2)
        b = np.zeros(a.shape[:3], self.dtype)
        j1, j2 = np.zeros_like(a), np.zeros_like(a)
        self._fn("glo_jb")(C.byref(self.S), a.shape[0], _ptr(a), _ptr(p1), _ptr(p2), _ptr(b), _ptr(j1), _ptr(j2))
        return b, j1, j2

    def arc_length(self, *fields):
        """Arc length over the given per-image arrays (each (F, ny, nx[, 2]))."""
        fl = [self._f(f) for f in fields]
        F = fl[0].shape[0]
        M = self.prob.sites
        widths = (C.c_int * len(fl))(*[1 if f.ndim == 3 else 2 for f in fl])
        ptrs = (_P * len(fl))(*[_ptr(f) for f in fl])
        s = np.zeros(F)
        self._fn("glo_arc_length")(F, C.c_long(M), len(fl), ptrs, widths, _ptr(s))
        return s

    def redistribute(self, s, f, f_new, cubic=False, spline=SPLINE_COMPAT):
        s = np.ascontiguousarray(s, np.float64)
        f = self._f(f)
        out = np.zeros((f_new,) + f.shape[1:], self.dtype)
        M = self.prob.sites
        if cubic:
            self._fn("glo_redistribute_cubic")(f.shape[0], C.c_long(M), _ptr(s), _ptr(f), int(f_new), _ptr(out),
                                               int(spline))
        else:
            self._fn("glo_redistribute_linear")(f.shape[0], C.c_long(M), _ptr(s), _ptr(f), int(f_new), _ptr(out))
        return out

    # ------------------------------------------------------------- solver
    def solver(self, state, ls_mode=LS_COMPAT, poly_compat=True):
        return OracleSolver(self, state, ls_mode, poly_compat)


class OracleSolver:
    """The nlcgSteps / loop() state machine of the oracle (one string)."""

    def __init__(self, orc: Oracle, state, ls_mode=LS_COMPAT, poly_compat=True):
        self.o = orc
        a, p1, p2 = orc._state(state.a, state.psi_1, state.psi_2)
        self.F = a.shape[0]
        self.shape = a.shape
        fn = orc._fn("glo_solver_create")
        fn.restype = _P
        self.h = fn(C.byref(orc.S), self.F, _ptr(a), _ptr(p1), _ptr(p2), int(ls_mode), int(poly_compat))

    def __del__(self):
        try:
            self.o._fn("glo_solver_destroy")(C.c_void_p(self.h))
        except Exception:
            pass

    def nlcg_steps(self, iters, use_cg=True, maxwell=False):
        self.o._fn("glo_solver_nlcg_steps")(C.c_void_p(self.h), int(iters), int(use_cg), int(maxwell))

    def iteration(self, mode, relaxation_steps, use_cg=True, spline=SPLINE_COMPAT):
        self.o._fn("glo_solver_iteration")(C.c_void_p(self.h), C.c_char(mode.encode()), int(relaxation_steps),
                                           int(use_cg), int(spline))

    def get(self):
        a, p1, p2 = (np.zeros(self.shape, self.o.dtype) for _ in range(3))
        fe, gn, al, s, sjb = (np.zeros(self.F) for _ in range(5))
        self.o._fn("glo_solver_get")(C.c_void_p(self.h), _ptr(a), _ptr(p1), _ptr(p2), _ptr(fe), _ptr(gn), _ptr(al),
                                     _ptr(s), _ptr(sjb))
        return dict(a=a, psi_1=p1, psi_2=p2, fenergy=fe, g_norm2=gn, alpha=al, s=s, s_jb=sjb)
