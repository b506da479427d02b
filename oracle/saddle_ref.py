"""CPU restatement of the stationary-point refinement (TEST INFRASTRUCTURE).

Checks mepgl_refine_stationary (mepgl_gb300/csrc/refine.cu) with the C
oracle's energy and gradient (oracle/gl_oracle.c, which restates
mepgl/src/nlcg.cu:105-888 and is pinned to the reference's own kernels).
Only tests import this module.

The algorithm is the same in outline, written in numpy:

* gauge step: minimise F(U_chi x) over chi = sum_m c_m P_a(X) P_b(Y)
  (Legendre products, 1 <= a + b <= degree, by default max(nx, ny) / 8
  within 4..16 and at most min(nx, ny) / 2) by Newton on the coefficients, with U_chi: A -> A + grad chi
  (central differences, one-sided at the lattice edge),
  psi_a -> psi_a exp(i q_a chi);
* saddles: lowest Hessian mode by Lanczos (full reorthogonalisation),
  uphill Newton step along it;
* shifted conjugate gradients (H + mu) p = -g in the complement;
* the step is kept when |g|^2 decreases (mu / 4), else mu * 4;

with Hessian-vector products as central differences of the gradient.  Both
implementations converge to the same stationary points, which is what the
tests compare (energy, barrier and |g| there), not their iterates.
"""
from __future__ import annotations

import numpy as np
from numpy.polynomial import legendre as _leg

MINIMUM, SADDLE = 0, 1


class Refiner:
    def __init__(self, orc, deg: int | None = None):
        self.o = orc
        self.p = orc.prob
        self.nc = self.p.ncomp
        ny, nx = self.p.ny, self.p.nx
        if deg is None:     # the library's automatic degree
            deg = min(16, max(4, max(nx, ny) // 8), max(1, min(nx, ny) // 2))
        J, I = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
        X = (2.0 * I - (nx - 1)) / (nx - 1)
        Y = (2.0 * J - (ny - 1)) / (ny - 1)
        self.basis = []
        for d in range(1, deg + 1):
            for k in range(d + 1):
                cx = np.zeros(d - k + 1)
                cx[-1] = 1
                cy = np.zeros(k + 1)
                cy[-1] = 1
                self.basis.append(_leg.legval(X, cx) * _leg.legval(Y, cy))
        self.shape = (1, ny, nx, 2)
        self.n_grad = 0

    # ---------------------------------------------------------- packing
    def pack(self, a, p1, p2=None):
        parts = [a.ravel(), p1.ravel()] + ([p2.ravel()] if self.nc == 2 else [])
        return np.concatenate(parts)

    def unpack(self, x):
        n = x.size // (1 + self.nc)
        f = [x[k * n:(k + 1) * n].reshape(self.shape) for k in range(1 + self.nc)]
        return f[0], f[1], (f[2] if self.nc == 2 else None)

    def grad(self, x):
        self.n_grad += 1
        ga, g1, g2 = self.o.gradient(*self.unpack(x))
        return self.pack(ga, g1, g2)

    def energy(self, x):
        return float(self.o.energy(*self.unpack(x))[0])

    # ------------------------------------------------------------ gauge
    def _cgrad(self, chi):
        dx = self.p.dx
        gx, gy = np.zeros_like(chi), np.zeros_like(chi)
        gx[:, 1:-1] = (chi[:, 2:] - chi[:, :-2]) / (2 * dx)
        gx[:, 0] = (chi[:, 1] - chi[:, 0]) / dx
        gx[:, -1] = (chi[:, -1] - chi[:, -2]) / dx
        gy[1:-1, :] = (chi[2:, :] - chi[:-2, :]) / (2 * dx)
        gy[0, :] = (chi[1, :] - chi[0, :]) / dx
        gy[-1, :] = (chi[-1, :] - chi[-2, :]) / dx
        return gx, gy

    def gauge(self, x, chi):
        a, p1, p2 = (None if f is None else f.copy() for f in self.unpack(x))
        gx, gy = self._cgrad(chi)
        a[0, ..., 0] += gx
        a[0, ..., 1] += gy
        out = [a]
        for p, q in ((p1, self.p.q_1), (p2, self.p.q_2))[:self.nc]:
            z = (p[0, ..., 0] + 1j * p[0, ..., 1]) * np.exp(1j * q * chi)
            out.append(np.stack([z.real, z.imag], -1)[None])
        return self.pack(*out)

    def gauge_grad(self, x, g):
        """dE/dc_m = g . J phi_m at x."""
        a, p1, p2 = self.unpack(x)
        ga, g1, g2 = self.unpack(g)
        w = 0.0
        for p, gp, q in ((p1, g1, self.p.q_1), (p2, g2, self.p.q_2))[:self.nc]:
            w = w + q * (p[0, ..., 0] * gp[0, ..., 1] - p[0, ..., 1] * gp[0, ..., 0])
        out = []
        for phi in self.basis:
            gx, gy = self._cgrad(phi)
            out.append(float(np.sum(ga[0, ..., 0] * gx + ga[0, ..., 1] * gy + w * phi)))
        return np.array(out)

    def gauge_step(self, x, h=1e-4):
        m = len(self.basis)
        if m == 0 or self.p.thin_film:
            return x
        g0 = self.gauge_grad(x, self.grad(x))
        H = np.zeros((m, m))
        for i, phi in enumerate(self.basis):
            xp, xm = self.gauge(x, h * phi), self.gauge(x, -h * phi)
            H[:, i] = (self.gauge_grad(xp, self.grad(xp)) - self.gauge_grad(xm, self.grad(xm))) / (2 * h)
        H = 0.5 * (H + H.T)
        try:
            L = np.linalg.cholesky(H)
            c = -np.linalg.solve(L.T, np.linalg.solve(L, g0))
        except np.linalg.LinAlgError:
            w, V = np.linalg.eigh(H)
            keep = w > 1e-12 * abs(w[-1])
            c = -V[:, keep] @ ((V[:, keep].T @ g0) / w[keep])
        return self.gauge(x, sum(ci * b for ci, b in zip(c, self.basis)))

    # ------------------------------------------------------------ Newton
    def hv(self, x, v):
        nv = np.linalg.norm(v)
        if nv == 0:
            return np.zeros_like(v)
        h = 1e-6 * np.sqrt(x.size) / nv
        return (self.grad(x + h * v) - self.grad(x - h * v)) / (2 * h)

    def _lanczos(self, x, v0, m):
        V, al, be = [], [], []
        v = v0 / np.linalg.norm(v0)
        for _ in range(m):
            V.append(v)
            w = self.hv(x, v)
            al.append(v @ w)
            for _ in range(2):
                for u in V:
                    w = w - (u @ w) * u
            b = np.linalg.norm(w)
            be.append(b)
            if b == 0:
                break
            v = w / b
        k = len(al)
        T = np.diag(al) + np.diag(be[:k - 1], 1) + np.diag(be[:k - 1], -1)
        return V, T

    def lanczos(self, x, v0, m):
        V, T = self._lanczos(x, v0, m)
        ev, U = np.linalg.eigh(T)
        y = np.array(V).T @ U[:, 0]
        return ev[0], y / np.linalg.norm(y)

    def cg(self, x, b, mu, v1, tol, maxit):
        P = (lambda u: u - (v1 @ u) * v1) if v1 is not None else (lambda u: u)
        s = np.zeros_like(b)
        r = P(b.copy())
        p = r.copy()
        rr = r @ r
        r0 = np.sqrt(rr)
        if r0 == 0:
            return s
        for _ in range(maxit):
            Ap = P(self.hv(x, p) + mu * p)
            pAp = p @ Ap
            if pAp <= 0:
                break
            a = rr / pAp
            s += a * p
            r -= a * Ap
            rn = r @ r
            if np.sqrt(rn) <= tol * r0:
                break
            p = r + (rn / rr) * p
            rr = rn
        return s

    def refine(self, x, kind, mode=None, g_tol=1e-8, max_newton=40, mu=1e-3, lanczos_steps=12, max_cg=3000):
        """Refine one image (packed fields x) to a minimum or an index-1 saddle.
        Returns (x, report dict)."""
        lam1, v1 = None, None
        if kind == SADDLE:
            v1 = mode
        first = True
        it = 0
        for it in range(max_newton + 1):
            g = self.grad(x)
            gn = np.linalg.norm(g)
            if gn <= g_tol or it == max_newton:
                break
            x = self.gauge_step(x)
            g = self.grad(x)
            gn = np.linalg.norm(g)
            if kind == SADDLE:
                lam1, v1 = self.lanczos(x, v1, 30 if first else lanczos_steps)
                first = False
                g1 = v1 @ g
                p1 = np.clip(g1 / max(abs(lam1), 1e-8), -1.0, 1.0)
                rhs = -(g - g1 * v1)
            else:
                p1, rhs = 0.0, -g
            eta = min(0.1, max(np.sqrt(gn), 0.5 * g_tol / gn))
            for _ in range(9):
                s = self.cg(x, rhs, mu, v1, eta, max_cg)
                step = s + (p1 * v1 if v1 is not None else 0.0)
                gt = self.grad(x + step)
                if np.isfinite(gt @ gt) and gt @ gt < gn * gn * (1 - 1e-4):
                    x = x + step
                    mu = max(mu / 4, 1e-12)
                    break
                mu *= 4
        g = self.grad(x)
        return x, dict(energy=self.energy(x), g_norm=float(np.linalg.norm(g)), min_curvature=lam1, newton=it)

    def morse_negatives(self, x, v0, m=40):
        """Negative Ritz values of H at x after m Lanczos steps (an estimate of the Morse index)."""
        _, T = self._lanczos(x, v0, m)
        ev = np.linalg.eigvalsh(T)
        return ev[ev < 0]
