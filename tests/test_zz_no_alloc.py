"""The allocation-free free-energy entry point (mepgl_free_energy_noalloc).

It exists for callers that cannot allocate device memory -- an embedding
that owns a fixed device arena, a host framework whose memory pool owns the
device, or a process that forbids cudaMalloc after start-up.  The test
allocates its inputs itself (a test may; the entry point may not), calls the
entry point through the C ABI twice in a row on different strings -- the second call reuses the fixed scratch the
first one left behind -- and compares each result with the context-based
mepgl_free_energy.  Collected last so that a stop-at-first-failure run has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from mepgl_gb300 import workloads as W
from mepgl_gb300.problem import PARAM_NAMES, neighbour_codes

pytestmark = pytest.mark.gpu

RTOL = 1e-12   # the energy tolerance of the other FP64 parity tests


def _device(torch, x, dtype):
    return torch.from_numpy(np.ascontiguousarray(x, dtype=dtype)).cuda()


def _noalloc_energy(native, torch, prob, st):
    L = native.lib()
    F = st.n_images
    keep = []

    def dev(x, dtype=np.float64):
        t = _device(torch, x, dtype)
        keep.append(t)
        return C.c_void_p(t.data_ptr())

    params = [dev(getattr(prob, n)) for n in PARAM_NAMES]
    p2 = st.psi_2 if prob.multicomponent else np.zeros_like(st.psi_1)
    out = torch.full((F,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    status = L.mepgl_free_energy_noalloc(
        prob.nx, prob.ny, F, int(prob.multicomponent), int(prob.thin_film), prob.dx,
        dev(neighbour_codes(prob.comp_domain), np.int32), dev(neighbour_codes(prob.sc_domain), np.int32),
        *params, prob.q_1, prob.q_2, prob.eta, prob.gamma, prob.delta,
        dev(st.a), dev(st.psi_1), dev(p2), C.c_void_p(out.data_ptr()), None)
    assert status == 0, L.mepgl_noalloc_last_error().decode()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_energy_matches_context_energy_twice_in_a_row():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mepgl_gb300 import build, native
    build.build()
    cases = [W.config2(n=40, images=5), W.config1(n=37, images=6)]
    for prob, st in cases:
        ctx = native.StringContext(prob, st.n_images, "fp64")
        ctx.set_state(st)
        want = ctx.compute_free_energy()
        ctx.close()
        got = _noalloc_energy(native, torch, prob, st)
        np.testing.assert_allclose(got, want, rtol=RTOL, atol=0)


def test_noalloc_rejects_oversize_strings():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mepgl_gb300 import native
    L = native.lib()
    dummy = C.c_void_p(1)
    status = L.mepgl_free_energy_noalloc(4096, 4096, 64, 0, 0, 0.5, *([dummy] * 11), 1.0, 1.0, 0.0, 0.0, 0.0,
                                         dummy, dummy, None, dummy, None)
    assert status == 1
    assert "too large" in L.mepgl_noalloc_last_error().decode()
    # few tiles, but a tile column past the 16-bit tile coordinates
    status = L.mepgl_free_energy_noalloc(1280000, 2, 1, 0, 0, 0.5, *([dummy] * 11), 1.0, 1.0, 0.0, 0.0, 0.0,
                                         dummy, dummy, None, dummy, None)
    assert status == 1
    assert "lattice too large" in L.mepgl_noalloc_last_error().decode()
