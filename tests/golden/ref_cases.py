"""Dynamics cases run on the reference build and stored as golden fixtures.

Each case is a box test (nextsimdg_gb300.boxtest), or a lon/lat patch on the
sphere (SphereCase), stepped through the dynamics-kernel interface
(initialise, the module's setData calls, update with the time-varying wind).  make_ref_goldens.py runs them on the
reference's own code (oracle/_ref, see oracle/pyref.py) and stores the
read-outs in ref_dynamics.npz; the tests run the same cases on the
restated CPU oracle and on the GPU and compare with those read-outs.

Read-outs: the cell averages (getDG0Data) of h, A, u, v and the ice-ocean
stress (and damage for BBM), plus all DG components (getDGData) of h and A
(and damage) on the small grids.  On the 256 x 256 grid the cell averages are
kept at every 13th cell, with the full-field maxima.
"""
from __future__ import annotations

import numpy as np

from nextsimdg_gb300.boxtest import BoxTest

# name: rheology (0 mEVP, 1 BBM), DG components, alpha (= beta unless set), grid, model
# steps, sub-cycle count, land holes, mask, vertex displacement, read-out mode
CASES = {
    "mevp_dg6_a300_12x12": dict(rheology=0, dg=6, alpha=300.0, nx=12, ny=12, steps=3, sub=100),
    "mevp_dg3_a300_17x18": dict(rheology=0, dg=3, alpha=300.0, nx=17, ny=18, steps=3, sub=100),
    "mevp_dg1_a300_16x16": dict(rheology=0, dg=1, alpha=300.0, nx=16, ny=16, steps=2, sub=100),
    "mevp_dg6_a1500_32x32": dict(rheology=0, dg=6, alpha=1500.0, nx=32, ny=32, steps=4, sub=100),
    "mevp_dg6_a1500_20x15_holes": dict(rheology=0, dg=6, alpha=1500.0, nx=20, ny=15, steps=3, sub=60,
                                       holes=True),
    "mevp_dg6_a300_64x64": dict(rheology=0, dg=6, alpha=300.0, nx=64, ny=64, steps=3, sub=100, dg0_only=True),
    "mevp_dg3_a1500_64x64": dict(rheology=0, dg=3, alpha=1500.0, nx=64, ny=64, steps=3, sub=100,
                                 dg0_only=True),
    "bbm_dg6_14x14": dict(rheology=1, dg=6, alpha=1500.0, nx=14, ny=14, steps=3, sub=50),
    "bbm_dg3_16x12": dict(rheology=1, dg=3, alpha=1500.0, nx=16, ny=12, steps=2, sub=50),
    "mevp_dg6_a1500_256x256": dict(rheology=0, dg=6, alpha=1500.0, nx=256, ny=256, steps=7, sub=100,
                                   sampled=13),
    # a sea-surface height with a gradient (the SSH term of the momentum
    # equation, CGDynamicsKernel.cpp:126-258)
    "mevp_dg6_a1500_24x20_ssh": dict(rheology=0, dg=6, alpha=1500.0, nx=24, ny=20, steps=3, sub=100, ssh=0.5),
    "bbm_dg6_16x14_ssh": dict(rheology=1, dg=6, alpha=1500.0, nx=16, ny=14, steps=2, sub=50, ssh=0.5),
    # spherical meshes (coordinates in radians, DynamicsKernel.hpp:44-75)
    "mevp_sph_dg3_a1500_20x16": dict(rheology=0, dg=3, alpha=1500.0, nx=20, ny=16, steps=3, sub=100, sphere=True),
    "mevp_sph_dg6_a1500_20x16": dict(rheology=0, dg=6, alpha=1500.0, nx=20, ny=16, steps=3, sub=100, sphere=True),
    # degenerate grids and masks: two rows, two columns, one ice cell in land,
    # a checkerboard of ice and land (every ice cell's edges closed)
    "mevp_dg6_a300_9x2": dict(rheology=0, dg=6, alpha=300.0, nx=9, ny=2, steps=3, sub=100),
    "mevp_dg3_a300_2x7": dict(rheology=0, dg=3, alpha=300.0, nx=2, ny=7, steps=3, sub=100),
    "mevp_dg6_a300_7x6_one": dict(rheology=0, dg=6, alpha=300.0, nx=7, ny=6, steps=3, sub=100, mask="one"),
    "mevp_dg6_a300_33x3_checker": dict(rheology=0, dg=6, alpha=300.0, nx=33, ny=3, steps=3, sub=100,
                                       mask="checker"),
    "bbm_dg6_10x8_checker": dict(rheology=1, dg=6, alpha=1500.0, nx=10, ny=8, steps=2, sub=50, mask="checker"),
    # general quadrilaterals: the box's vertices displaced as in the
    # reference's distorted advection mesh (Advection_test.cpp:213-217), so the
    # Jacobian varies inside each element and no operator is affine
    "mevp_dg6_a300_20x18_distorted": dict(rheology=0, dg=6, alpha=300.0, nx=20, ny=18, steps=3, sub=100,
                                          distort=0.05),
    "mevp_dg3_a1500_16x16_distorted": dict(rheology=0, dg=3, alpha=1500.0, nx=16, ny=16, steps=3, sub=100,
                                           distort=0.05),
    "bbm_dg6_14x12_distorted": dict(rheology=1, dg=6, alpha=1500.0, nx=14, ny=12, steps=2, sub=50, distort=0.05),
    # unequal mEVP relaxation constants (alpha for the stress, beta for the
    # velocity): a swap of the two shows here and in no case above
    "mevp_dg6_a300_b1500_18x16": dict(rheology=0, dg=6, alpha=300.0, beta=1500.0, nx=18, ny=16, steps=3, sub=100),
    "mevp_dg3_a1500_b300_16x18": dict(rheology=0, dg=3, alpha=1500.0, beta=300.0, nx=16, ny=18, steps=3, sub=100),
    # BBM over six steps on a larger grid (damage down to 0.05): the
    # reference's own response to h x (1 + 1e-14) stays near 2e-14 here
    "bbm_dg3_40x40_6steps": dict(rheology=1, dg=3, alpha=1500.0, nx=40, ny=40, steps=6, sub=50),
}


def beta(case: dict) -> float:
    """The case's mEVP beta (equal to alpha unless the case sets it)."""
    return case.get("beta", case["alpha"])


class SphereCase:
    """A lon/lat patch (longitudes -0.3..0.3 rad, latitudes 1.0..1.3 rad) with
    a land border, smooth thickness with seeded noise, a zonal ocean current
    and a time-varying wind; the same calls as BoxTest."""

    spherical = True
    dt = 120.0

    def __init__(self, nx: int, ny: int, seed: int = 3):
        self.nx, self.ny = nx, ny
        self.lon = np.linspace(-0.3, 0.3, nx + 1)
        self.lat = np.linspace(1.0, 1.3, ny + 1)
        cx = 0.5 * (self.lon[:-1] + self.lon[1:])
        cy = 0.5 * (self.lat[:-1] + self.lat[1:])
        self.CX, self.CY = np.meshgrid(cx, cy)
        self.noise = np.random.default_rng(seed).standard_normal(nx * ny)

    def coords(self) -> np.ndarray:
        X, Y = np.meshgrid(self.lon, self.lat)
        return np.stack([X.ravel(), Y.ravel()], 1)

    def mask(self) -> np.ndarray:
        m = np.ones((self.ny, self.nx))
        m[0, :] = m[-1, :] = 0
        m[:, 0] = m[:, -1] = 0
        return m

    def initial_fields(self) -> dict:
        n = self.nx * self.ny
        return {"hice": (0.3 + 0.05 * np.sin(9 * self.CX) * np.cos(7 * self.CY)).ravel() + 0.01 * self.noise,
                "cice": np.full(n, 0.95), "u": np.zeros(n), "v": np.zeros(n),
                "uocean": 0.05 * np.cos(5 * self.CY).ravel(), "vocean": np.zeros(n), "ssh": np.zeros(n)}

    def wind(self, t: float):
        s = t / self.dt
        return (12.0 * np.cos(4 * self.CY + 0.01 * s).ravel(), 6.0 * np.sin(3 * self.CX - 0.02 * s).ravel())

DG0_NAMES = ("hice", "cice", "u", "v", "uiostress", "viostress")


def box(case: dict):
    if case.get("sphere"):
        return SphereCase(case["nx"], case["ny"])
    b = BoxTest(case["nx"], case["ny"], distort=case.get("distort", 0.0))
    if case.get("ssh"):
        # a tilted, wavy sea surface of the given amplitude (m)
        X, Y = np.meshgrid((np.arange(b.nx) + 0.5) / b.nx, (np.arange(b.ny) + 0.5) / b.ny)
        eta = case["ssh"] * (X - 0.5 + 0.3 * np.sin(2 * np.pi * Y) * np.cos(3 * np.pi * X))
        b.ssh = lambda eta=eta: eta.ravel().copy()
    if case.get("holes"):
        m = b.mask()
        rng = np.random.default_rng(5)
        for _ in range(12):
            m[rng.integers(1, case["ny"] - 1), rng.integers(1, case["nx"] - 1)] = 0.0
        b.mask = lambda m=m: m
    if case.get("mask"):
        m = np.zeros((case["ny"], case["nx"]))
        if case["mask"] == "one":
            m[case["ny"] // 2, case["nx"] // 2] = 1.0
        else:  # checkerboard
            m[(np.add.outer(np.arange(case["ny"]), np.arange(case["nx"])) % 2) == 0] = 1.0
        b.mask = lambda m=m: m
    return b


def run(kernel, case: dict, b: BoxTest | None = None):
    """initialise, the initial setData calls, then `steps` model steps."""
    b = box(case) if b is None else b
    kernel.initialise(b.coords(), getattr(b, "spherical", False), b.mask())
    for name, arr in b.initial_fields().items():
        kernel.setData(name, arr)
    if case["rheology"] == 1:
        kernel.setData("damage", b.damage())
    for s in range(case["steps"]):
        uw, vw = b.wind(s * b.dt)
        kernel.setData("uwind", uw)
        kernel.setData("vwind", vw)
        kernel.update(s * b.dt, b.dt)
    return kernel


def readouts(kernel, case: dict) -> dict:
    names = DG0_NAMES + (("damage",) if case["rheology"] == 1 else ())
    out = {}
    n = case["nx"] * case["ny"]
    idx = np.arange(0, n, case["sampled"]) if case.get("sampled") else None
    for f in names:
        a = kernel.getDG0Data(f)
        if idx is not None:
            out[f"dg0_{f}_absmax"] = np.array([np.abs(a).max()])
            a = a[idx]
        out[f"dg0_{f}"] = a
    if not case.get("dg0_only") and not case.get("sampled") and case["dg"] > 1:
        for f in ("hice", "cice") + (("damage",) if case["rheology"] == 1 else ()):
            out[f"dg_{f}"] = kernel.getDGData(f)
    return out


def max_rel(a: np.ndarray, b: np.ndarray, scale: float | None = None) -> float:
    """max |a - b| / max |b| (or / scale)."""
    s = float(np.abs(b).max()) if scale is None else scale
    return float(np.abs(a - b).max()) / max(s, 1e-300)


def compare(got: dict, want: dict) -> dict:
    """Worst relative difference per read-out, against the fixture's
    magnitude (the full-field maximum for sampled read-outs)."""
    worst = {}
    for k, w in want.items():
        if k.endswith("_absmax"):
            continue
        scale = float(want[k + "_absmax"][0]) if (k + "_absmax") in want else None
        worst[k] = max_rel(got[k], w, scale)
    return worst
