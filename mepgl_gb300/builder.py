"""Initial-guess builder with the interface of the reference's StringBuilder.

``config.py`` files written for the reference build their initial string with
``StringBuilder`` (mepgl/mepgl_lib/builder.py): a meshgrid with
``indexing="ij"``, domain shape functions, vortices per image and gauge
potentials.  This class offers the same constructor, attributes and methods
so such files run unchanged under ``python -m mepgl_gb300.run`` (which maps
``mepgl_lib.builder`` to this module).  The vortex profile is the
reference's ``tanh(-r**2)`` envelope and the noise is unseeded by default,
as in the reference; pass ``seed=`` for reproducible strings.
"""
from __future__ import annotations

import numpy as np


class StringBuilder:
    def __init__(self, F, Nx, Ny, x_lim, y_lim, multicomponent, B_z=0, seed=None):
        self.F = int(F)
        self.Nx, self.Ny = int(Nx), int(Ny)
        self.x_lim, self.y_lim = x_lim, y_lim
        self.multicomponent = multicomponent
        self.B_z = B_z
        self.rng = np.random.default_rng(seed) if seed is not None else None
        self.x_ax = np.linspace(x_lim[0], x_lim[1], self.Nx)
        self.y_ax = np.linspace(y_lim[0], y_lim[1], self.Ny)
        self.x, self.y = np.meshgrid(self.x_ax, self.y_ax, indexing="ij")
        inside = lambda x, y: (x >= x_lim[0]) & (x <= x_lim[1]) & (y >= y_lim[0]) & (y <= y_lim[1])
        self.comp_domain_shape_fun = inside
        self.sc_domain_shape_fun = inside
        self.phase_fun = lambda x, y: 0
        self.vortices_1, self.vortices_2 = [], []

    # ------------------------------------------------------------ settings
    def set_comp_domain(self, shape_fun):
        self.comp_domain_shape_fun = shape_fun

    def set_sc_domain(self, shape_fun):
        self.sc_domain_shape_fun = shape_fun

    def add_phase_diff(self, phase_fun):
        self.phase_fun = phase_fun

    def add_vortex(self, xv, yv, Nv, component):
        (self.vortices_1 if component == 1 else self.vortices_2).append([xv, yv, Nv])

    # ------------------------------------------------------------- outputs
    def _mask(self, fun):
        m = np.vectorize(lambda a, b: bool(fun(a, b)))(self.x, self.y)
        return m.astype(np.intc)

    def get_domain_matrices(self):
        return self._mask(self.comp_domain_shape_fun), self._mask(self.sc_domain_shape_fun)

    def _noise(self, scale):
        if scale == 0:
            return 0.0
        g = self.rng.standard_normal if self.rng is not None else np.random.randn
        return scale * (g((self.Nx, self.Ny)) if self.rng is not None else g(self.Nx, self.Ny))

    def _component(self, vortices, psi_abs, phase0, noise, sc):
        u = np.ones((self.F, self.Nx, self.Ny))
        v = np.ones((self.F, self.Nx, self.Ny))
        for n in range(self.F):
            mag = psi_abs + 0 * self.x
            th = phase0 + 0 * self.x
            for xv, yv, wv in vortices:
                if wv[n] != 0:
                    r = np.sqrt((self.x - xv[n]) ** 2 + (self.y - yv[n]) ** 2)
                    mag = mag * np.tanh(-(r ** 2))
                    th = th + wv[n] * np.arctan2(self.y - yv[n], self.x - xv[n])
            u[n] = (mag * np.cos(th) + self._noise(noise)) * sc
            v[n] = (mag * np.sin(th) + self._noise(noise)) * sc
        return u, v

    def generate_matter_fields(self, psi_abs_1=1.0, psi_abs_2=1.0, noise=0.0):
        sc = self._mask(self.sc_domain_shape_fun)
        u1, v1 = self._component(self.vortices_1, psi_abs_1, 0 * self.x, noise, sc)
        if self.multicomponent:
            u2, v2 = self._component(self.vortices_2, psi_abs_2, self.phase_fun(self.x, self.y), noise, sc)
        else:
            u2, v2 = np.ones_like(u1), np.ones_like(v1)
        return u1, v1, u2, v2

    def generate_vector_potential(self, gauge="symmetric"):
        comp = self._mask(self.comp_domain_shape_fun)
        ax = np.zeros((self.F, self.Nx, self.Ny))
        ay = np.zeros((self.F, self.Nx, self.Ny))
        for n in range(self.F):
            if gauge == "Landau_x":
                ax[n] = -self.B_z * self.y
            elif gauge == "Landau_y":
                ay[n] = self.B_z * self.x
            elif gauge == "symmetric":
                ax[n] = -0.5 * self.B_z * self.y
                ay[n] = 0.5 * self.B_z * self.x
            else:
                raise ValueError(f"unknown gauge {gauge!r}")
            ax[n] *= comp
            ay[n] *= comp
        return ax, ay
