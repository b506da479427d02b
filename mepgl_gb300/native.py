"""ctypes binding of libmepgl_gb300.so (include/mepgl.h) and the Python
mirror of the reference's host operators.

:class:`StringContext` is the reference-facing object: its methods carry the
names of the reference functions they replace (``compute_free_energy`` for
computeFreeEnergy, ``nlcg_steps`` for nlcgSteps, ``compute_jb`` for
computeJB, ``arc_length`` / ``arc_length_jb`` for arcLength / arcLengthJB,
``redistribute_linear`` / ``redistribute_cubic``, ``loop_iteration`` for one
pass of loop()).  All compute runs in the CUDA library; this module only
moves arguments.  There is no CPU fallback: a missing library raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from .problem import Problem, StringState

LIB_PATH = os.environ.get("MEPGL_LIB",
                          os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libmepgl_gb300.so"))

FP32, FP64 = 0, 1
HOST, DEVICE = 0, 1
LS_COMPAT, LS_EXACT = 0, 1
POLY_COMPAT, POLY_EXACT = 0, 1
SPLINE_COMPAT, SPLINE_FMM = 0, 1
METRIC_FIELDS, METRIC_JB = 0, 1
REDIST_LINEAR, REDIST_CUBIC = 0, 1

_STATUS = {0: "OK", 1: "INVALID_ARG", 2: "CUDA", 3: "NAN", 4: "IO", 5: "UNSUPPORTED", 6: "STATE"}


class MepglError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"mepgl error {_STATUS.get(status, status)}: {message}")
        self.status = status


class MepglProblem(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("n_images", C.c_int32), ("multicomponent", C.c_int32),
                ("thin_film", C.c_int32), ("precision", C.c_int32), ("dx", C.c_double), ("q_1", C.c_double),
                ("q_2", C.c_double), ("eta", C.c_double), ("gamma", C.c_double), ("delta", C.c_double)] + \
               [(n, C.c_void_p) for n in ("a_1", "b_1", "m_xx_1", "m_yy_1", "a_2", "b_2", "m_xx_2", "m_yy_2", "h",
                                          "comp_domain", "sc_domain")]


class MepglOptions(C.Structure):
    _fields_ = [("line_search", C.c_int32), ("line_polynomial", C.c_int32), ("spline", C.c_int32),
                ("metric", C.c_int32), ("use_graphs", C.c_int32), ("tile_rows", C.c_int32)]


_lib = None
_lock = threading.Lock()

_SIGS = {
    "mepgl_default_options": (None, [C.c_void_p]),
    "mepgl_version": (C.c_char_p, []),
    "mepgl_last_error": (C.c_char_p, [C.c_void_p]),
    "mepgl_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "mepgl_destroy": (C.c_int, [C.c_void_p]),
    "mepgl_set_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "mepgl_get_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "mepgl_free_energy": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mepgl_energy_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "mepgl_nlcg_steps": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "mepgl_reset_cg": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "mepgl_image_scalars": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mepgl_compute_jb": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "mepgl_arc_length": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "mepgl_redistribute": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "mepgl_iteration": (C.c_int, [C.c_void_p, C.c_char, C.c_int, C.c_int]),
    "mepgl_set_precision": (C.c_int, [C.c_void_p, C.c_int]),
    "mepgl_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int64)]),
    "mepgl_synchronize": (C.c_int, [C.c_void_p]),
    "mepgl_profile_passes": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    "mepgl_free_energy_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double]
                                  + [C.c_void_p] * 11 + [C.c_double] * 5 + [C.c_void_p] * 5),
    "mepgl_noalloc_last_error": (C.c_char_p, []),
}


def lib():
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"libmepgl_gb300.so not found at {LIB_PATH}: run "
                                   "`python -c 'import __graft_entry__ as g; g.build()'` first")
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in _SIGS.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def exported_symbols():
    return sorted(_SIGS)


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(C.c_void_p)
    return C.c_void_p(int(a))


def default_options(**kw) -> MepglOptions:
    o = MepglOptions()
    lib().mepgl_default_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, int(v))
    return o


class StringContext:
    """One string on the GPU: the drop-in for the reference's engine state."""

    def __init__(self, prob: Problem, n_images: int, precision: str = "fp64", stream=None, **options):
        prob.validate()
        self.L = lib()
        self.prob = prob
        self.prec = FP64 if precision == "fp64" else FP32
        self.dtype = np.float64 if self.prec == FP64 else np.float32
        keep = []

        def arr(x, dt=np.float64):
            a = np.ascontiguousarray(x, dtype=dt)
            keep.append(a)
            return a.ctypes.data

        p = MepglProblem()
        p.nx, p.ny, p.n_images = prob.nx, prob.ny, int(n_images)
        p.multicomponent, p.thin_film, p.precision = int(prob.multicomponent), int(prob.thin_film), self.prec
        p.dx, p.q_1, p.q_2, p.eta, p.gamma, p.delta = prob.dx, prob.q_1, prob.q_2, prob.eta, prob.gamma, prob.delta
        for n in ("a_1", "b_1", "m_xx_1", "m_yy_1", "a_2", "b_2", "m_xx_2", "m_yy_2", "h"):
            setattr(p, n, arr(getattr(prob, n)))
        p.comp_domain = arr(prob.comp_domain, np.int32)
        p.sc_domain = arr(prob.sc_domain, np.int32)
        self.options = default_options(**options)
        h = C.c_void_p()
        st = self.L.mepgl_create(C.byref(p), C.byref(self.options),
                                 None if stream is None else C.c_void_p(int(stream)), C.byref(h))
        if st != 0:
            raise MepglError(st, self.L.mepgl_last_error(None).decode())
        self.h = h
        self.F = int(n_images)

    # ------------------------------------------------------------- plumbing
    def _check(self, st):
        if st != 0:
            raise MepglError(st, self.L.mepgl_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.mepgl_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def ncomp(self):
        return self.prob.ncomp

    def _shape(self):
        return (self.F, self.prob.ny, self.prob.nx, 2)

    # ---------------------------------------------------------------- state
    def set_state(self, state: StringState):
        a = np.ascontiguousarray(state.a, self.dtype)
        p1 = np.ascontiguousarray(state.psi_1, self.dtype)
        p2 = np.ascontiguousarray(state.psi_2, self.dtype) if self.ncomp == 2 else None
        if a.shape != self._shape():
            raise ValueError(f"state shape {a.shape} != {self._shape()}")
        self._check(self.L.mepgl_set_state(self.h, _ptr(a), _ptr(p1), _ptr(p2), HOST))

    def set_state_device(self, a, psi_1, psi_2=None):
        """Device pointers (ints, e.g. torch ``data_ptr()``) of the context precision."""
        self._check(self.L.mepgl_set_state(self.h, _ptr(a), _ptr(psi_1), _ptr(psi_2), DEVICE))

    def get_state(self) -> StringState:
        a, p1 = np.empty(self._shape(), self.dtype), np.empty(self._shape(), self.dtype)
        p2 = np.empty(self._shape(), self.dtype) if self.ncomp == 2 else None
        self._check(self.L.mepgl_get_state(self.h, _ptr(a), _ptr(p1), _ptr(p2), HOST))
        return StringState(a=a, psi_1=p1, psi_2=p2)

    def get_state_device(self, a, psi_1, psi_2=None):
        self._check(self.L.mepgl_get_state(self.h, _ptr(a), _ptr(psi_1), _ptr(psi_2), DEVICE))

    # ------------------------------------------------------------- compute
    def compute_free_energy(self) -> np.ndarray:
        out = np.zeros(self.F)
        self._check(self.L.mepgl_free_energy(self.h, _ptr(out)))
        return out

    def energy_grad(self):
        e = np.zeros(self.F)
        g = [np.empty(self._shape(), self.dtype) for _ in range(3)]
        self._check(self.L.mepgl_energy_grad(self.h, _ptr(e), _ptr(g[0]), _ptr(g[1]),
                                             _ptr(g[2]) if self.ncomp == 2 else None, HOST))
        return e, (g[0], g[1], g[2] if self.ncomp == 2 else None)

    def energy_grad_device(self, g_a, g_psi_1, g_psi_2=None, with_energy=True):
        e = np.zeros(self.F) if with_energy else None
        self._check(self.L.mepgl_energy_grad(self.h, _ptr(e), _ptr(g_a), _ptr(g_psi_1), _ptr(g_psi_2), DEVICE))
        return e

    def nlcg_steps(self, iterations: int, nlcg: bool = True, maxwell: bool = False):
        self._check(self.L.mepgl_nlcg_steps(self.h, int(iterations), int(nlcg), int(maxwell)))

    def reset_cg(self, first: int, last: int):
        self._check(self.L.mepgl_reset_cg(self.h, int(first), int(last)))

    def image_scalars(self):
        fe, gn, al = np.zeros(self.F), np.zeros(self.F), np.zeros(self.F)
        self._check(self.L.mepgl_image_scalars(self.h, _ptr(fe), _ptr(gn), _ptr(al)))
        return dict(fenergy=fe, g_norm2=gn, alpha=al)

    def compute_jb(self):
        b = np.empty(self._shape()[:3], self.dtype)
        j1 = np.empty(self._shape(), self.dtype)
        j2 = np.empty(self._shape(), self.dtype) if self.ncomp == 2 else None
        self._check(self.L.mepgl_compute_jb(self.h, _ptr(b), _ptr(j1), _ptr(j2), HOST))
        return b, j1, j2

    def arc_length(self, metric: int = METRIC_FIELDS) -> np.ndarray:
        s = np.zeros(self.F)
        self._check(self.L.mepgl_arc_length(self.h, int(metric), _ptr(s)))
        return s

    def arc_length_jb(self) -> np.ndarray:
        return self.arc_length(METRIC_JB)

    def redistribute(self, kind: int, n_new: int | None = None):
        n_new = self.F if n_new is None else int(n_new)
        self._check(self.L.mepgl_redistribute(self.h, int(kind), n_new))
        self.F = n_new

    def redistribute_linear(self, n_new: int | None = None):
        self.redistribute(REDIST_LINEAR, n_new)

    def redistribute_cubic(self, n_new: int | None = None):
        self.redistribute(REDIST_CUBIC, n_new)

    def loop_iteration(self, mode: str, relaxation_steps: int, nlcg: bool = True):
        self._check(self.L.mepgl_iteration(self.h, C.c_char(mode.encode()), int(relaxation_steps), int(nlcg)))

    def set_precision(self, precision: str):
        p = FP64 if precision == "fp64" else FP32
        self._check(self.L.mepgl_set_precision(self.h, p))
        self.prec = p
        self.dtype = np.float64 if p == FP64 else np.float32

    def info(self):
        n, p, k = C.c_int(), C.c_int(), C.c_int64()
        self._check(self.L.mepgl_info(self.h, C.byref(n), C.byref(p), C.byref(k)))
        return dict(n_images=n.value, precision="fp64" if p.value else "fp32", kernel_launches=k.value)

    def profile_passes(self, steps: int, nlcg: bool = True):
        """Mean milliseconds of (gradient pass, direction/line pass) over `steps` real steps."""
        a, b = C.c_double(), C.c_double()
        self._check(self.L.mepgl_profile_passes(self.h, int(steps), int(nlcg), C.byref(a), C.byref(b)))
        return a.value, b.value

    def synchronize(self):
        self._check(self.L.mepgl_synchronize(self.h))
