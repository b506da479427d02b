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
HOST, DEVICE, STAGED = 0, 1, 2
LS_COMPAT, LS_EXACT = 0, 1
POLY_COMPAT, POLY_EXACT = 0, 1
SPLINE_COMPAT, SPLINE_FMM = 0, 1
METRIC_FIELDS, METRIC_JB = 0, 1
REDIST_LINEAR, REDIST_CUBIC = 0, 1
DISC_REFERENCE, DISC_LINK = 0, 1
FP64_NATIVE, FP64_PAIRED = 0, 1
FP32_STEPS_AUTO, FP32_STEPS_PASSES, FP32_STEPS_FUSED = 0, 1, 2

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
                ("metric", C.c_int32), ("use_graphs", C.c_int32), ("tile_rows", C.c_int32),
                ("discretization", C.c_int32), ("fp64_arith", C.c_int32), ("fp32_steps", C.c_int32)]


class MepglVortex(C.Structure):
    _fields_ = [("component", C.c_int32), ("pad", C.c_int32), ("x", C.c_void_p), ("y", C.c_void_p),
                ("winding", C.c_void_p)]


class MepglRefineOptions(C.Structure):
    _fields_ = [("g_tol", C.c_double), ("max_newton", C.c_int32), ("max_cg", C.c_int32),
                ("lanczos_steps", C.c_int32), ("gauge_degree", C.c_int32), ("mu0", C.c_double),
                ("cg_eta", C.c_double), ("max_retries", C.c_int32), ("gauge_refresh", C.c_int32),
                ("precondition", C.c_int32), ("forcing", C.c_int32)]


class MepglRefineReport(C.Structure):
    _fields_ = [("energy", C.c_double), ("g_norm", C.c_double), ("min_curvature", C.c_double), ("mu", C.c_double),
                ("newton_iterations", C.c_int32), ("cg_iterations", C.c_int32),
                ("gradient_evaluations", C.c_int32), ("converged", C.c_int32), ("preconditioned", C.c_int32)]


STATIONARY_MINIMUM, STATIONARY_SADDLE, STATIONARY_SKIP = 0, 1, 2


class MepglGuess(C.Structure):
    _fields_ = [("x0", C.c_double), ("y0", C.c_double), ("psi_abs_1", C.c_double), ("psi_abs_2", C.c_double),
                ("noise", C.c_double), ("b_z", C.c_double), ("gauge", C.c_int32), ("profile", C.c_int32),
                ("seed", C.c_uint64), ("vortices", C.c_void_p), ("n_vortices", C.c_int32), ("pad", C.c_int32)]


GAUGES = {None: 0, "none": 0, "Landau_x": 1, "Landau_y": 2, "symmetric": 3}

_lib = None
_lock = threading.Lock()

_SIGS = {
    "mepgl_default_options": (None, [C.c_void_p]),
    "mepgl_version": (C.c_char_p, []),
    "mepgl_last_error": (C.c_char_p, [C.c_void_p]),
    "mepgl_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "mepgl_destroy": (C.c_int, [C.c_void_p]),
    "mepgl_set_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "mepgl_stage_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
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
    "mepgl_pass_kernels": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mepgl_fused_wait_selftest": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mepgl_free_energy_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double]
                                  + [C.c_void_p] * 11 + [C.c_double] * 5 + [C.c_void_p] * 5),
    "mepgl_noalloc_last_error": (C.c_char_p, []),
    "mepgl_create_batch": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "mepgl_string_count": (C.c_int, [C.c_void_p]),
    "mepgl_batch_info": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.c_int)]),
    "mepgl_batch_set_state": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "mepgl_batch_get_state": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "mepgl_batch_free_energy": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "mepgl_batch_image_scalars": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mepgl_batch_arc_length": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    "mepgl_param_adjoint": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mepgl_observables": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mepgl_generate_string": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mepgl_batch_generate_string": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "mepgl_batch_observables": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mepgl_batch_param_adjoint": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mepgl_default_refine_options": (None, [C.c_void_p]),
    "mepgl_refine_stationary": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                          C.c_void_p, C.c_void_p]),
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


def _fill_problem(p: MepglProblem, prob: Problem, n_images: int, prec: int, keep: list):
    """Fill one mepgl_problem; `keep` holds the host arrays alive until create returns."""
    prob.validate()

    def arr(x, dt=np.float64):
        a = np.ascontiguousarray(x, dtype=dt)
        keep.append(a)
        return a.ctypes.data

    p.nx, p.ny, p.n_images = prob.nx, prob.ny, int(n_images)
    p.multicomponent, p.thin_film, p.precision = int(prob.multicomponent), int(prob.thin_film), prec
    p.dx, p.q_1, p.q_2, p.eta, p.gamma, p.delta = prob.dx, prob.q_1, prob.q_2, prob.eta, prob.gamma, prob.delta
    for n in ("a_1", "b_1", "m_xx_1", "m_yy_1", "a_2", "b_2", "m_xx_2", "m_yy_2", "h"):
        setattr(p, n, arr(getattr(prob, n)))
    p.comp_domain = arr(prob.comp_domain, np.int32)
    p.sc_domain = arr(prob.sc_domain, np.int32)


class StringContext:
    """One string on the GPU: the drop-in for the reference's engine state."""

    def __init__(self, prob: Problem, n_images: int, precision: str = "fp64", stream=None, **options):
        self.L = lib()
        self.prob = prob
        self.prec = FP64 if precision == "fp64" else FP32
        self.dtype = np.float64 if self.prec == FP64 else np.float32
        keep = []
        p = MepglProblem()
        _fill_problem(p, prob, n_images, self.prec, keep)
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

    def stage_state(self, a, psi_1, psi_2=None, memory: int = HOST):
        """Start the upload of the next state on the context's copy stream
        (pointers as ints, e.g. of pinned torch tensors; ``memory`` HOST or
        DEVICE) and return at once; ``set_staged_state`` installs it."""
        self._check(self.L.mepgl_stage_state(self.h, _ptr(a), _ptr(psi_1), _ptr(psi_2), int(memory)))

    def set_staged_state(self):
        """Wait for the staged upload and make it the current state (the
        history reset of ``set_state``)."""
        self._check(self.L.mepgl_set_state(self.h, None, None, None, STAGED))

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

    def param_adjoint(self):
        """(F, 3): per-image dF/dH (uniform shift of h), dF/deta, dF/dgamma at the current fields."""
        h, e, g = np.zeros(self.F), np.zeros(self.F), np.zeros(self.F)
        self._check(self.L.mepgl_param_adjoint(self.h, _ptr(h), _ptr(e), _ptr(g)))
        return np.stack([h, e, g], axis=1)

    def generate_string(self, vortices=(), x0=0.0, y0=0.0, psi_abs_1=1.0, psi_abs_2=1.0, noise=0.0, b_z=0.0,
                        gauge=None, profile="builder", seed=0):
        """Build the initial string on the device (mepgl_generate_string).

        vortices: (component, x[F], y[F], winding[F]) tracks in physical
        coordinates; site (i, j) is at (x0 + i dx, y0 + j dx).  profile
        "builder" is the reference builder's tanh(-r^2) envelope, "tanh"
        is tanh(r / sqrt 2); gauge None / "Landau_x" / "Landau_y" /
        "symmetric" sets A from b_z."""
        keep = []
        vs = (MepglVortex * max(1, len(vortices)))()
        for k, (comp, xv, yv, wv) in enumerate(vortices):
            xa = np.ascontiguousarray(np.broadcast_to(xv, (self.F,)), np.float64)
            ya = np.ascontiguousarray(np.broadcast_to(yv, (self.F,)), np.float64)
            wa = np.ascontiguousarray(np.broadcast_to(wv, (self.F,)), np.int32)
            keep += [xa, ya, wa]
            vs[k].component, vs[k].x, vs[k].y, vs[k].winding = int(comp), xa.ctypes.data, ya.ctypes.data, wa.ctypes.data
        g = MepglGuess()
        g.x0, g.y0, g.psi_abs_1, g.psi_abs_2, g.noise, g.b_z = x0, y0, psi_abs_1, psi_abs_2, noise, b_z
        g.gauge = GAUGES[gauge]
        g.profile = {"builder": 0, "tanh": 1}[profile]
        g.seed = int(seed)
        g.vortices = C.cast(vs, C.c_void_p)
        g.n_vortices = len(vortices)
        self._check(self.L.mepgl_generate_string(self.h, C.byref(g)))

    def observables(self, inset: int = 0):
        """Per-image flux dx^2 sum B and winding sums of psi_1 (and psi_2) around
        the rectangle `inset` sites inside the lattice edge."""
        phi, w1 = np.zeros(self.F), np.zeros(self.F)
        w2 = np.zeros(self.F) if self.ncomp == 2 else None
        self._check(self.L.mepgl_observables(self.h, int(inset), _ptr(phi), _ptr(w1), _ptr(w2)))
        return dict(phi=phi, w_1=w1, w_2=w2)

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

    def pass_kernels(self):
        """(gradient pass, direction/line pass, fused steps or "") kernel names
        for the current precision."""
        g, d, f = C.c_char_p(), C.c_char_p(), C.c_char_p()
        self._check(self.L.mepgl_pass_kernels(self.h, C.byref(g), C.byref(d), C.byref(f)))
        return g.value.decode(), d.value.decode(), f.value.decode()

    def fused_wait_selftest(self) -> bool:
        """Run the fused launch's bounded-wait self-test; True when its waits
        ran out and were reported (the expected outcome)."""
        t = C.c_int()
        self._check(self.L.mepgl_fused_wait_selftest(self.h, C.byref(t)))
        return bool(t.value)

    def profile_passes(self, steps: int, nlcg: bool = True):
        """Mean milliseconds of (gradient pass, direction/line pass) over `steps` real steps."""
        a, b = C.c_double(), C.c_double()
        self._check(self.L.mepgl_profile_passes(self.h, int(steps), int(nlcg), C.byref(a), C.byref(b)))
        return a.value, b.value

    def synchronize(self):
        self._check(self.L.mepgl_synchronize(self.h))

    def refine_stationary(self, kinds, mode: StringState | None = None, **options):
        """Refine the images in place to stationary points (mepgl_refine_stationary).

        kinds: per image STATIONARY_MINIMUM / _SADDLE / _SKIP.  mode: initial
        direction of each saddle image (fields' shape; None continues from the
        previous call's modes).  options: fields of mepgl_refine_options.
        Returns a list of per-image report dicts."""
        k = np.ascontiguousarray(kinds, np.int32)
        if k.shape != (self.F,):
            raise ValueError(f"need {self.F} kinds")
        o = MepglRefineOptions()
        self.L.mepgl_default_refine_options(C.byref(o))
        for key, v in options.items():
            setattr(o, key, v)
        rep = (MepglRefineReport * self.F)()
        ptrs = [None, None, None]
        keep = []
        if mode is not None:
            for f, arr in enumerate((mode.a, mode.psi_1, mode.psi_2 if self.ncomp == 2 else None)):
                if arr is not None:
                    a = np.ascontiguousarray(arr, np.float64)
                    if a.shape != self._shape():
                        raise ValueError(f"mode shape {a.shape} != {self._shape()}")
                    keep.append(a)
                    ptrs[f] = _ptr(a)
        self._check(self.L.mepgl_refine_stationary(self.h, _ptr(k), *ptrs, HOST, C.byref(o), rep))
        return [{f: getattr(r, f) for f, _ in MepglRefineReport._fields_} for r in rep]


class StringBatch(StringContext):
    """Several independent strings advanced by the same launches.

    The reference runs a parameter sweep as one process per string
    (mepgl/batch_run.py:9-21); here the strings share one context and every
    NLCG step covers all of them.  ``problems[k]`` with ``n_images[k]`` images
    is string ``k``; the per-string calls take that index.  Whole-context
    calls (``nlcg_steps``, ``loop_iteration``, ``set_precision``,
    ``redistribute_*`` without a new image count) act on every string.
    """

    def __init__(self, problems, n_images, precision: str = "fp64", stream=None, **options):
        self.L = lib()
        self.problems = list(problems)
        if isinstance(n_images, int):
            n_images = [n_images] * len(self.problems)
        self.Fs = [int(f) for f in n_images]
        if len(self.Fs) != len(self.problems) or not self.problems:
            raise ValueError("need one image count per problem")
        self.prob = self.problems[0]
        self.prec = FP64 if precision == "fp64" else FP32
        self.dtype = np.float64 if self.prec == FP64 else np.float32
        keep = []
        arr = (MepglProblem * len(self.problems))()
        for k, (pr, F) in enumerate(zip(self.problems, self.Fs)):
            _fill_problem(arr[k], pr, F, self.prec, keep)
        self.options = default_options(**options)
        h = C.c_void_p()
        st = self.L.mepgl_create_batch(arr, len(self.problems), C.byref(self.options),
                                       None if stream is None else C.c_void_p(int(stream)), C.byref(h))
        if st != 0:
            raise MepglError(st, self.L.mepgl_last_error(None).decode())
        self.h = h
        self.F = self.Fs[0]

    def __len__(self):
        return self.L.mepgl_string_count(self.h)

    def _shape_of(self, k):
        pr = self.problems[k]
        return (self.Fs[k], pr.ny, pr.nx, 2)

    def set_string_state(self, k: int, state: StringState):
        a = np.ascontiguousarray(state.a, self.dtype)
        p1 = np.ascontiguousarray(state.psi_1, self.dtype)
        p2 = np.ascontiguousarray(state.psi_2, self.dtype) if self.ncomp == 2 else None
        if a.shape != self._shape_of(k):
            raise ValueError(f"state shape {a.shape} != {self._shape_of(k)}")
        self._check(self.L.mepgl_batch_set_state(self.h, int(k), _ptr(a), _ptr(p1), _ptr(p2), HOST))

    def get_string_state(self, k: int) -> StringState:
        shp = self._shape_of(k)
        a, p1 = np.empty(shp, self.dtype), np.empty(shp, self.dtype)
        p2 = np.empty(shp, self.dtype) if self.ncomp == 2 else None
        self._check(self.L.mepgl_batch_get_state(self.h, int(k), _ptr(a), _ptr(p1), _ptr(p2), HOST))
        return StringState(a=a, psi_1=p1, psi_2=p2)

    def string_free_energy(self, k: int) -> np.ndarray:
        out = np.zeros(self.Fs[k])
        self._check(self.L.mepgl_batch_free_energy(self.h, int(k), _ptr(out)))
        return out

    def string_scalars(self, k: int):
        F = self.Fs[k]
        fe, gn, al = np.zeros(F), np.zeros(F), np.zeros(F)
        self._check(self.L.mepgl_batch_image_scalars(self.h, int(k), _ptr(fe), _ptr(gn), _ptr(al)))
        return dict(fenergy=fe, g_norm2=gn, alpha=al)

    def string_arc_length(self, k: int, metric: int = METRIC_FIELDS) -> np.ndarray:
        s = np.zeros(self.Fs[k])
        self._check(self.L.mepgl_batch_arc_length(self.h, int(k), int(metric), _ptr(s)))
        return s

    def string_info(self, k: int):
        nx, ny, F = C.c_int(), C.c_int(), C.c_int()
        self._check(self.L.mepgl_batch_info(self.h, int(k), C.byref(nx), C.byref(ny), C.byref(F)))
        return dict(nx=nx.value, ny=ny.value, n_images=F.value)

    def redistribute(self, kind: int, n_new: int | None = None):
        if n_new is not None and len(self.problems) > 1:
            raise ValueError("a batch of strings keeps its image counts; resample one string at a time")
        self._check(self.L.mepgl_redistribute(self.h, int(kind), -1 if n_new is None else int(n_new)))
        if n_new is not None:
            self.Fs[0] = self.F = int(n_new)
