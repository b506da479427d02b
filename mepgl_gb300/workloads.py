"""Seeded synthetic strings for the benchmark configurations.

Each builder returns ``(Problem, StringState)`` for one of the five workload
families the project is measured on.  There is no public dataset involved:
inputs are drawn from ``numpy.random.default_rng(seed)`` with the shapes,
parameters and noise levels of each configuration, and the initial string
is built the way the reference's launcher builds one
(mepgl/mepgl_lib/builder.py:107-189): image 0 is the Meissner state, the last
image holds the vortex, intermediate images interpolate linearly, and every
image gets i.i.d. Gaussian noise on Re psi, Im psi (masked by the
superconducting domain) and on A (masked by the computational domain).

Vortex profile: psi = psi_inf * tanh(r / sqrt(2)) * exp(i theta), r in
physical units (the reference builder's tanh(-r^2) is a known slip; the
configurations specify the tanh(r/sqrt2) profile).

Every builder takes ``n`` and ``images`` overrides so the same physics can be
run at test sizes.
"""
from __future__ import annotations

import numpy as np

from .problem import Problem, StringState


def _margin_domain(n: int, margin: int) -> np.ndarray:
    d = np.zeros((n, n), np.int32)
    d[margin:n - margin, margin:n - margin] = 1
    return d


def _vortex(n, dx, i0, j0, psi_inf, winding=1):
    jj, ii = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    xr = (ii - i0) * dx
    yr = (jj - j0) * dx
    r = np.sqrt(xr ** 2 + yr ** 2)
    th = winding * np.arctan2(yr, xr)
    mag = psi_inf * np.tanh(r / np.sqrt(2.0))
    return np.stack([mag * np.cos(th), mag * np.sin(th)], axis=-1)


def _meissner(n, psi_inf, phase=0.0):
    out = np.zeros((n, n, 2))
    out[..., 0] = psi_inf * np.cos(phase)
    out[..., 1] = psi_inf * np.sin(phase)
    return out


def _interp_string(start, end, images):
    t = np.linspace(0.0, 1.0, images)[:, None, None, None]
    return (1 - t) * start[None] + t * end[None]


def _noisy(rng, f, sigma, mask):
    return (f + sigma * rng.standard_normal(f.shape)) * mask[None, :, :, None]


def config1(n: int = 64, images: int = 16, seed: int = 1001, dx: float = 0.5, margin: int = 4):
    """Plain method, small: single component, a=-1, b=1, m=1, q=1 (kappa=2),
    H=0.8, 64x64 at dx=0.5, vacuum margin of 4 sites, 16 images; the last
    image has one vortex at lattice (8, 32) (scaled with n)."""
    rng = np.random.default_rng(seed)
    comp = np.ones((n, n), np.int32)
    sc = _margin_domain(n, margin)
    prob = Problem.uniform(n, n, dx, a=(-1.0, -1.0), b=(1.0, 1.0), h=0.8, q=(1.0, 1.0),
                           comp_domain=comp, sc_domain=sc)
    end = _vortex(n, dx, i0=8 * n / 64.0, j0=n / 2.0, psi_inf=1.0)
    psi = _interp_string(_meissner(n, 1.0), end, images)
    a = np.zeros_like(psi)
    psi = _noisy(rng, psi, 1e-3, sc)
    a = _noisy(rng, a, 1e-3, comp)
    return prob, StringState(a=a, psi_1=psi)


def config2(n: int = 256, images: int = 64, seed: int = 1002, dx: float = 0.4, margin: int = 4):
    """Mixed precision: two components, a1=-1 b1=1, a2=-0.6 b2=1, m1=(1,1),
    m2=(1,2), eta=-0.5, gamma=0.2, H=0.9, 256x256 at dx=0.4, 64 images;
    Meissner to one fractional vortex per component, the two cores 2 lattice
    units apart near the left edge."""
    rng = np.random.default_rng(seed)
    comp = np.ones((n, n), np.int32)
    sc = _margin_domain(n, margin)
    prob = Problem.uniform(n, n, dx, a=(-1.0, -0.6), b=(1.0, 1.0), m_xx=(1.0, 1.0), m_yy=(1.0, 2.0),
                           h=0.9, q=(1.0, 1.0), eta=-0.5, gamma=0.2, delta=0.0, multicomponent=True,
                           comp_domain=comp, sc_domain=sc)
    p1, p2 = 1.0, np.sqrt(0.6)
    i0 = margin + max(4.0, 0.05 * n)
    end1 = _vortex(n, dx, i0=i0, j0=n / 2.0, psi_inf=p1)
    end2 = _vortex(n, dx, i0=i0 + 2, j0=n / 2.0, psi_inf=p2)
    s1 = _noisy(rng, _interp_string(_meissner(n, p1), end1, images), 1e-3, sc)
    s2 = _noisy(rng, _interp_string(_meissner(n, p2), end2, images), 1e-3, sc)
    a = _noisy(rng, np.zeros((images, n, n, 2)), 1e-3, comp)
    return prob, StringState(a=a, psi_1=s1, psi_2=s2)


def _gaussian_field(rng, n, corr, amp):
    k = np.fft.fftfreq(n)
    kk = np.sqrt(k[:, None] ** 2 + k[None, :] ** 2)
    filt = np.exp(-0.5 * (2 * np.pi * kk * corr) ** 2)
    w = rng.standard_normal((n, n))
    f = np.real(np.fft.ifft2(np.fft.fft2(w) * filt))
    return amp * f / (np.std(f) + 1e-300)


def config3(n: int = 512, images: int = 32, seed: int = 1003, dx: float = 0.3):
    """Differentiation: two components, eta=-0.3, gamma=0.1, delta=0.05,
    H=1.0, 512x512 at dx=0.3, 32 images of random smooth fields:
    |psi| = 0.8 +- 0.1, random smooth phase, A a Gaussian random field of
    correlation length 5 and amplitude 0.2."""
    rng = np.random.default_rng(seed)
    prob = Problem.uniform(n, n, dx, a=(-1.0, -1.0), b=(1.0, 1.0), h=1.0, q=(1.0, 1.0), eta=-0.3,
                           gamma=0.1, delta=0.05, multicomponent=True)
    psis = []
    for _ in range(2):
        mag = 0.8 + 0.1 * rng.uniform(-1, 1, (images, n, n))
        ph = np.stack([_gaussian_field(rng, n, 5.0, np.pi) for _ in range(images)])
        psis.append(np.stack([mag * np.cos(ph), mag * np.sin(ph)], axis=-1))
    a = np.stack([np.stack([_gaussian_field(rng, n, 5.0, 0.2) for _ in range(2)], axis=-1)
                  for _ in range(images)])
    return prob, StringState(a=a, psi_1=psis[0], psi_2=psis[1])


def config4_string(s: int, n: int | None = None, images: int | None = None, dx: float = 0.5):
    """String ``s`` of the batched sweep: single component, N ~ U{96..384},
    F ~ U{24..64}, H ~ U[0.5, 1.2], kappa ~ U[1, 4] (m = kappa / 2 with
    a=-1, b=1, q=1), Meissner to one vortex."""
    rng = np.random.default_rng(1400 + s)
    n_ = int(rng.integers(96, 385)) if n is None else n
    f_ = int(rng.integers(24, 65)) if images is None else images
    hz = float(rng.uniform(0.5, 1.2))
    kappa = float(rng.uniform(1.0, 4.0))
    m = kappa / 2.0
    margin = 4
    comp = np.ones((n_, n_), np.int32)
    sc = _margin_domain(n_, margin)
    prob = Problem.uniform(n_, n_, dx, m_xx=(m, m), m_yy=(m, m), h=hz, comp_domain=comp, sc_domain=sc)
    end = _vortex(n_, dx, i0=margin + 4, j0=n_ / 2.0, psi_inf=1.0)
    psi = _noisy(rng, _interp_string(_meissner(n_, 1.0), end, f_), 1e-3, sc)
    a = _noisy(rng, np.zeros_like(psi), 1e-3, comp)
    return prob, StringState(a=a, psi_1=psi)


def config5(n: int = 2048, images: int = 128, seed: int = 1005, dx: float = 0.25, radius: float | None = None):
    """Large: two components q1=1, q2=0.5, delta=0.1, eta=0, gamma=0.3,
    2048x2048 at dx=0.25 masked to a disk of radius 1000 lattice units,
    128 images, H=1.1, composite vortex 20 units inside the rim."""
    rng = np.random.default_rng(seed)
    r0 = (1000.0 * n / 2048.0) if radius is None else radius
    jj, ii = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    c = (n - 1) / 2.0
    disk = (((ii - c) ** 2 + (jj - c) ** 2) <= r0 ** 2).astype(np.int32)
    comp = np.ones((n, n), np.int32)
    prob = Problem.uniform(n, n, dx, a=(-1.0, -1.0), b=(1.0, 1.0), h=1.1, q=(1.0, 0.5), eta=0.0, gamma=0.3,
                           delta=0.1, multicomponent=True, comp_domain=comp, sc_domain=disk)
    i0 = c - r0 + 20 * n / 2048.0
    end1 = _vortex(n, dx, i0=i0, j0=c, psi_inf=1.0)
    end2 = _vortex(n, dx, i0=i0, j0=c, psi_inf=1.0)
    s1 = _noisy(rng, _interp_string(_meissner(n, 1.0), end1, images), 1e-4, disk)
    s2 = _noisy(rng, _interp_string(_meissner(n, 1.0), end2, images), 1e-4, disk)
    a = _noisy(rng, np.zeros_like(s1), 1e-4, comp)
    return prob, StringState(a=a, psi_1=s1, psi_2=s2)


def random_problem(rng, n=12, multicomponent=True, thin_film=False, masked=True, uniform=True):
    """Small random problem for parity tests: holes in both masks (so every
    boundary branch is exercised), random couplings and charges."""
    comp = np.ones((n, n), np.int32)
    sc = np.ones((n, n), np.int32)
    if masked:
        sc[rng.random((n, n)) < 0.12] = 0
        sc[0, :] = 0
        comp[rng.random((n, n)) < 0.05] = 0
    prob = Problem.uniform(
        n, n, float(rng.uniform(0.2, 0.6)),
        a=(float(rng.uniform(-1.2, -0.5)), float(rng.uniform(-1.0, -0.4))),
        b=(float(rng.uniform(0.7, 1.3)), float(rng.uniform(0.7, 1.3))),
        m_xx=(float(rng.uniform(0.6, 1.5)), float(rng.uniform(0.6, 1.5))),
        m_yy=(float(rng.uniform(0.6, 1.5)), float(rng.uniform(0.6, 2.0))),
        h=float(rng.uniform(0.3, 1.2)), q=(float(rng.choice([1.0, -1.0, 0.5])), float(rng.choice([1.0, -0.7]))),
        eta=float(rng.uniform(-0.5, 0.5)), gamma=float(rng.uniform(-0.2, 0.4)), delta=float(rng.uniform(-0.1, 0.2)),
        multicomponent=multicomponent, thin_film=thin_film, comp_domain=comp, sc_domain=sc)
    if not uniform:
        for name in ("a_1", "b_1", "m_xx_1", "m_yy_1", "a_2", "b_2", "m_xx_2", "m_yy_2", "h"):
            arr = getattr(prob, name)
            setattr(prob, name, arr * (1.0 + 0.1 * rng.uniform(-1, 1, arr.shape)))
    return prob


def random_state(rng, prob, images=4, amp=0.3):
    n_y, n_x = prob.ny, prob.nx
    sh = (images, n_y, n_x, 2)
    a = amp * rng.standard_normal(sh)
    p1 = 0.8 + amp * rng.standard_normal(sh)
    p2 = 0.6 + amp * rng.standard_normal(sh) if prob.multicomponent else None
    return StringState(a=a, psi_1=p1, psi_2=p2)


def config5_device(n: int = 2048, images: int = 128, seed: int = 1005, dx: float = 0.25, dtype=None,
                   device="cuda"):
    """The large workload built directly in device memory: ``config5``'s
    problem and end states, the linear interpolation and the noise formed by
    torch on the GPU (a 2048^2 x 128 string is 13 GB in FP32; the noise comes
    from torch's generator seeded with ``seed``, not from numpy's stream).
    Returns (Problem, (a, psi_1, psi_2)) with CUDA tensors (F, n, n, 2)."""
    import torch
    dtype = dtype or torch.float32
    r0 = 1000.0 * n / 2048.0
    jj, ii = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    c = (n - 1) / 2.0
    disk = (((ii - c) ** 2 + (jj - c) ** 2) <= r0 ** 2).astype(np.int32)
    comp = np.ones((n, n), np.int32)
    prob = Problem.uniform(n, n, dx, a=(-1.0, -1.0), b=(1.0, 1.0), h=1.1, q=(1.0, 0.5), eta=0.0, gamma=0.3,
                           delta=0.1, multicomponent=True, comp_domain=comp, sc_domain=disk)
    i0 = c - r0 + 20 * n / 2048.0
    end = torch.tensor(_vortex(n, dx, i0=i0, j0=c, psi_inf=1.0), dtype=dtype, device=device)
    start = torch.tensor(_meissner(n, 1.0), dtype=dtype, device=device)
    sc = torch.tensor(disk, dtype=dtype, device=device)[None, :, :, None]
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    t = torch.linspace(0.0, 1.0, images, dtype=dtype, device=device)[:, None, None, None]
    out = []
    for k in range(2):
        p = (1 - t) * start[None] + t * end[None]
        p += 1e-4 * torch.randn(p.shape, generator=g, dtype=dtype, device=device)
        out.append((p * sc).contiguous())
    a = (1e-4 * torch.randn((images, n, n, 2), generator=g, dtype=dtype, device=device)).contiguous()
    return prob, (a, out[0], out[1])
