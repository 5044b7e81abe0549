"""Synthetic box-test inputs (the shapes of the Mehlmann et al. 2021 benchmark).

The reference ships formulas, not data, for this case: the domain and initial
state follow run/make_init_benchmark.py:7-36, the cyclone profile
physics/src/modules/AtmosphereBoundaryModule/BenchmarkAtmosphere.cpp:41-73 and
the ocean current BenchmarkOcean.cpp:31-36, evaluated, like the reference, at
x = i*dx, y = j*dy of cell (i, j).  The forcing constants are those of the
workload this library is measured on: a 0.1 m/s rotating ocean current and a
cyclone of 15 m/s maximum wind whose centre moves diagonally at 10 m/s,
convergence angle 72 degrees, radial decay scale 100 km.

Every array is in the ModelArray layout (element index i + nx*j).  The same
generator feeds the GPU kernel and the CPU oracle.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class BoxTest:
    nx: int
    ny: int | None = None
    L: float = 512e3            # domain side [m]
    dt: float = 120.0           # model time step [s]
    seed: int = 0               # phases of the h undulation, ensemble perturbations
    ocean_max: float = 0.1      # [m/s]
    wind_max: float = 15.0      # maximum wind speed of the cyclone [m/s]
    wind_speed: float = 10.0    # speed of the cyclone centre along the diagonal [m/s]
    convergence_deg: float = 72.0
    decay: float = 100e3        # radial decay scale 1/k [m]
    start: tuple = field(default=None)  # cyclone centre at t = 0 (default: domain centre)
    h_noise: float = 0.0        # std of seeded Gaussian noise added to h [m]
    land_ring: bool = True      # outer ring of cells is land (make_init_benchmark.py:20-24)
    distort: float = 0.0        # vertex displacement, fraction of the box (0: the regular box)

    def __post_init__(self):
        if self.ny is None:
            self.ny = self.nx
        if self.start is None:
            self.start = (0.5 * self.L, 0.5 * self.L)
        rng = np.random.default_rng(self.seed)
        self._phase = (0.0, 0.0) if self.seed == 0 else tuple(rng.uniform(0, 2 * math.pi, 2))
        self._noise = rng.standard_normal(self.nx * self.ny) * self.h_noise if self.h_noise else None

    @property
    def nelements(self) -> int:
        return self.nx * self.ny

    @property
    def dx(self) -> float:
        return self.L / self.nx

    @property
    def dy(self) -> float:
        return self.L / self.ny

    def coords(self) -> np.ndarray:
        """Vertices ((nx+1)*(ny+1), 2): x_i = i*L/nx, y_j = j*L/ny; with
        distort > 0 displaced as the reference's distorted test mesh
        (Advection_test.cpp:213-217): x += L d sin(3 pi i/nx) sin(pi j/ny),
        y += L d sin(2 pi j/ny) sin(2 pi i/nx), which makes the elements
        general quadrilaterals (the boundary stays straight)."""
        i = np.arange(self.nx + 1)
        j = np.arange(self.ny + 1)
        I, J = np.meshgrid(i, j)
        X = self.L * I / self.nx
        Y = self.L * J / self.ny
        if self.distort:
            d = self.distort
            X = X + self.L * d * np.sin(np.pi * I / self.nx * 3.0) * np.sin(np.pi * J / self.ny)
            Y = Y + self.L * d * np.sin(np.pi * J / self.ny * 2.0) * np.sin(np.pi * I / self.nx * 2.0)
        return np.stack([X.ravel(), Y.ravel()], axis=1)

    def mask(self) -> np.ndarray:
        m = np.ones((self.ny, self.nx))
        if self.land_ring:
            m[0, :] = m[-1, :] = 0.0
            m[:, 0] = m[:, -1] = 0.0
        return m

    def _cell_xy(self):
        x = np.arange(self.nx) * self.dx
        y = np.arange(self.ny) * self.dy
        X, Y = np.meshgrid(x, y)
        return X.ravel(), Y.ravel()

    def hice(self) -> np.ndarray:
        x, y = self._cell_xy()
        h = 0.3 + 0.005 * (np.sin(6e-5 * x + self._phase[0]) + np.sin(3e-5 * y + self._phase[1]))
        if self._noise is not None:
            h = h + self._noise
        return h

    def cice(self) -> np.ndarray:
        return np.ones(self.nelements)

    def damage(self) -> np.ndarray:
        return np.ones(self.nelements)

    def ocean(self):
        x, y = self._cell_xy()
        u = self.ocean_max * (2.0 * y - self.L) / self.L
        v = -self.ocean_max * (2.0 * x - self.L) / self.L
        return u, v

    def wind(self, t: float):
        """Cyclone wind at time t [s] since the start."""
        x, y = self._cell_xy()
        s = self.wind_speed * t / math.sqrt(2.0)
        cx, cy = self.start[0] + s, self.start[1] + s
        xp, yp = x - cx, y - cy
        k = 1.0 / self.decay
        r = np.hypot(xp, yp)
        # |wind| = wind_max (k r) exp(1 - k r): maximum wind_max at r = 1/k
        f = self.wind_max * math.e * k * np.exp(-k * r)
        a = math.radians(self.convergence_deg)
        ca, sa = math.cos(a), math.sin(a)
        u = -f * (ca * xp + sa * yp)
        v = -f * (-sa * xp + ca * yp)
        return u, v

    def device_forcing(self):
        """The same wind and ocean current as nsdg_benchmark_forcing, for the
        kernels that compute them on the device: scale = wind_A exp(-k r) with
        wind_A = wind_max e k and wind_vmax = 1 gives |wind| = wind_max at
        r = 1/k; the centre moves along the diagonal at wind_speed."""
        from . import _lib
        k = 1.0 / self.decay
        v = self.wind_speed / math.sqrt(2.0)
        return _lib.benchmark_forcing(self.L, self.L, wind_A=self.wind_max * math.e * k,
                                      wind_vmax=1.0, wind_k=k, wind_angle_deg=self.convergence_deg,
                                      centre_x=self.start[0], centre_y=self.start[1], centre_vx=v, centre_vy=v,
                                      ocean_vmax=self.ocean_max)

    def ssh(self) -> np.ndarray:
        return np.zeros(self.nelements)

    def initial_fields(self) -> dict:
        uo, vo = self.ocean()
        uw, vw = self.wind(0.0)
        z = np.zeros(self.nelements)
        return {"hice": self.hice(), "cice": self.cice(), "u": z, "v": z, "uocean": uo, "vocean": vo,
                "uwind": uw, "vwind": vw, "ssh": self.ssh()}


def setup_kernel(kernel, box: BoxTest, damage: bool = False):
    """initialise + the initial setData calls of MEVPDynamics::setData
    (core/src/modules/DynamicsModule/MEVPDynamics.cpp:37-57) plus the forcing."""
    kernel.initialise(box.coords(), False, box.mask())
    for name, arr in box.initial_fields().items():
        kernel.setData(name, arr)
    if damage:
        kernel.setData("damage", box.damage())
    return kernel


def step_forcing(kernel, box: BoxTest, step: int):
    """The per-step setData calls of MEVPDynamics::update for the time-varying wind."""
    uw, vw = box.wind(step * box.dt)
    kernel.setData("uwind", uw)
    kernel.setData("vwind", vw)
