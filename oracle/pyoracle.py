"""ctypes binding of the CPU oracle (oracle/nsdg_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and bench.py's
CPU-baseline leg, as the checker.  The classes mirror the product's Python
interface (nextsimdg_gb300.dynamics) so a test can drive both with the same
calls.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, byref, c_double, c_int, c_size_t, c_void_p, c_char_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libnsdg_oracle.so"


class Params(ctypes.Structure):
    """Same layout as nsdg_params in include/nsdg.h."""

    _fields_ = [
        ("rho_ice", c_double), ("rho_atm", c_double), ("rho_ocean", c_double),
        ("C_atm", c_double), ("C_ocean", c_double),
        ("F_atm", c_double), ("F_ocean", c_double),
        ("fc", c_double), ("ocean_turning_angle", c_double), ("gravity", c_double),
        ("Pstar", c_double), ("DeltaMin", c_double),
        ("alpha", c_double), ("beta", c_double),
        ("compaction_param", c_double), ("nu0", c_double), ("young", c_double), ("P0", c_double),
        ("undamaged_time_relaxation_sigma", c_double), ("exponent_relaxation_sigma", c_double),
        ("exponent_compression_factor", c_double), ("tan_phi", c_double),
        ("compr_strength", c_double), ("C_lab", c_double),
        ("n_steps", c_int), ("precision", c_int),
    ]


def build(force: bool = False) -> Path:
    build_ice_growth(force)
    src = HERE / "nsdg_oracle.cpp"
    hdr = HERE.parent / "include" / "nsdg.h"
    if force or not LIB.exists() or LIB.stat().st_mtime < max(src.stat().st_mtime, hdr.stat().st_mtime):
        LIB.parent.mkdir(exist_ok=True)
        cxx = os.environ.get("CXX", "g++")
        subprocess.run([cxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fopenmp",
                        "-I", str(HERE.parent / "include"), "-shared", "-o", str(LIB), str(src)], check=True)
    return LIB


IG_SRC = HERE / "ice_growth_oracle.cpp"
IG_LIB = HERE / "_build" / "libice_growth_oracle.so"


def build_ice_growth(force: bool = False) -> Path:
    """The column-thermodynamics oracle (oracle/ice_growth_oracle.cpp)."""
    hdr = HERE.parent / "include" / "nsdg.h"
    if force or not IG_LIB.exists() or IG_LIB.stat().st_mtime < max(IG_SRC.stat().st_mtime, hdr.stat().st_mtime):
        IG_LIB.parent.mkdir(exist_ok=True)
        cxx = os.environ.get("CXX", "g++")
        subprocess.run([cxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                        "-I", str(HERE.parent / "include"), "-shared", "-o", str(IG_LIB), str(IG_SRC)], check=True)
    return IG_LIB


_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(str(LIB))
        sig = {
            "oracle_default_params": (None, [POINTER(Params)]),
            "oracle_kernel_create": (c_void_p, [c_int, c_int, POINTER(Params)]),
            "oracle_kernel_destroy": (None, [c_void_p]),
            "oracle_kernel_last_error": (c_char_p, [c_void_p]),
            "oracle_kernel_initialise": (c_int, [c_void_p, c_size_t, c_size_t, c_void_p, c_void_p]),
            "oracle_kernel_initialise_spherical": (c_int, [c_void_p, c_size_t, c_size_t, c_void_p, c_int, c_void_p]),
            "oracle_kernel_set_data": (c_int, [c_void_p, c_char_p, c_void_p, c_size_t, c_size_t]),
            "oracle_kernel_get_dg0": (c_int, [c_void_p, c_char_p, c_void_p, c_size_t]),
            "oracle_kernel_get_dg": (c_int, [c_void_p, c_char_p, c_void_p, c_size_t, c_size_t]),
            "oracle_kernel_update": (c_int, [c_void_p, c_double, c_double]),
            "oracle_kernel_get_cg": (c_int, [c_void_p, c_char_p, c_void_p, c_size_t]),
            "oracle_kernel_get_stress": (c_int, [c_void_p, c_char_p, c_void_p, c_size_t]),
            "oracle_kernel_mean_value": (c_double, [c_void_p, c_char_p]),
            "oracle_num_threads": (c_int, []),
            "oracle_set_num_threads": (None, [c_int]),
            "oracle_table": (c_int, [c_char_p, c_int, c_int, c_void_p]),
            "oracle_transport_create": (c_void_p, [c_int, c_size_t, c_size_t, c_void_p, c_void_p,
                                                   POINTER(c_void_p), POINTER(c_size_t), c_void_p, c_size_t,
                                                   c_int]),
            "oracle_transport_destroy": (None, [c_void_p]),
            "oracle_transport_set_velocity": (None, [c_void_p, c_void_p, c_void_p]),
            "oracle_transport_reinit": (None, [c_void_p]),
            "oracle_transport_step": (None, [c_void_p, c_double, c_void_p, c_int, c_int, c_double, c_int,
                                             c_double]),
            "oracle_transport_mean_value": (c_double, [c_void_p, c_void_p]),
            "oracle_transport_limit": (None, [c_void_p, c_void_p, c_int, c_double, c_int, c_double]),
            "oracle_transport_function2dg": (None, [c_void_p, c_int, c_double, c_void_p]),
            "oracle_transport_l2error": (c_double, [c_void_p, c_int, c_double, c_void_p]),
            "oracle_advection_golden": (c_double, [c_int, c_double, c_int, POINTER(c_double)]),
            "oracle_periodic_golden": (c_double, [c_int, c_int, POINTER(c_double)]),
            "oracle_mesh_dirichlet": (c_int, [c_size_t, c_size_t, c_void_p, POINTER(c_size_t), c_void_p,
                                              c_size_t]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class IceGrowthParams(ctypes.Structure):
    """Same layout as nsdg_ice_growth_params in include/nsdg.h."""

    _fields_ = [
        ("ks", c_double), ("h_min", c_double), ("c_min", c_double), ("h0", c_double), ("phi_m", c_double),
        ("healing_time", c_double), ("use_thermo", c_int), ("thermo_model", c_int),
        ("lateral_model", c_int), ("healing_model", c_int), ("flooding", c_int),
    ]


# the field slots of include/nsdg.h (NSDG_IG_*), in order
IG_FIELDS = ("hice", "cice", "hsnow", "tice", "qia", "dqia_dt", "qow", "qio", "sublim", "snowfall", "penSW",
             "sst", "tf", "mlbhc", "damage", "hice_updated", "cice_updated", "hsnow_updated", "hice_initial",
             "hsnow_initial", "newice", "delta_cice", "delta_hice", "tice_updated", "qic", "snow_to_ice",
             "top_melt", "bottom_melt", "snow_melt", "delta_cfreeze", "delta_cmelt", "tice_1", "tice_2",
             "tice_updated_1", "tice_updated_2")

_ig = None


def _ig_lib() -> ctypes.CDLL:
    global _ig
    if _ig is None:
        build_ice_growth()
        lib = ctypes.CDLL(str(IG_LIB))
        lib.oracle_ice_growth_default_params.restype = None
        lib.oracle_ice_growth_default_params.argtypes = [POINTER(IceGrowthParams)]
        lib.oracle_ice_growth_update.restype = None
        lib.oracle_ice_growth_update.argtypes = [c_size_t, c_void_p, POINTER(IceGrowthParams), c_double, c_void_p]
        lib.oracle_thermo_ice0.restype = None
        lib.oracle_thermo_ice0.argtypes = [c_size_t, POINTER(IceGrowthParams), c_double, c_void_p]
        lib.oracle_constant_healing.restype = c_double
        lib.oracle_constant_healing.argtypes = [c_double, c_double, c_double, c_double, c_double]
        lib.oracle_unesco_freezing.restype = c_double
        lib.oracle_unesco_freezing.argtypes = [c_double]
        _ig = lib
    return _ig


def ice_growth_params(**overrides) -> IceGrowthParams:
    p = IceGrowthParams()
    _ig_lib().oracle_ice_growth_default_params(byref(p))
    for k, v in overrides.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


def constant_healing(damage: float, cice: float, delta_ci: float, dt: float, td: float) -> float:
    return _ig_lib().oracle_constant_healing(damage, cice, delta_ci, dt, td)


def unesco_freezing(sss: float) -> float:
    return _ig_lib().oracle_unesco_freezing(float(sss))


class OracleIceGrowth:
    """IceGrowth (ThermoIce0, HiblerSpread, ConstantHealing) restated on the
    CPU, with the product's set/get-by-name interface."""

    def __init__(self, n: int, mask=None, params: IceGrowthParams | None = None, **overrides):
        self.n = n
        self.params = params if params is not None else ice_growth_params(**overrides)
        self.mask = None if mask is None else _f64(mask).ravel().copy()
        self.fields = np.zeros((len(IG_FIELDS), n))

    def setData(self, name: str, data):
        self.fields[IG_FIELDS.index(name)] = np.broadcast_to(_f64(data).ravel(), (self.n,))

    def getData(self, name: str) -> np.ndarray:
        return self.fields[IG_FIELDS.index(name)].copy()

    def update(self, dt: float):
        m = None if self.mask is None else _p(self.mask)
        _ig_lib().oracle_ice_growth_update(self.n, m, byref(self.params), float(dt), _p(self.fields))

    def thermo_only(self, dt: float):
        """ThermoIce0 alone on the true-thickness slots (the reference's
        ThermoIce0 test drives the module that way)."""
        _ig_lib().oracle_thermo_ice0(self.n, byref(self.params), float(dt), _p(self.fields))


def default_params(**overrides) -> Params:
    p = Params()
    load().oracle_default_params(byref(p))
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def set_threads(n: int):
    load().oracle_set_num_threads(n)


def num_threads() -> int:
    return load().oracle_num_threads()


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a):
    return a.ctypes.data_as(c_void_p)


class OracleKernel:
    """The reference's dynamics kernel restated on the CPU (FP64)."""

    def __init__(self, rheology: int = 0, dg_comp: int = 6, params: Params | None = None, **overrides):
        self._l = load()
        p = params if params is not None else default_params()
        for k, v in overrides.items():
            setattr(p, k, v)
        self.params = p
        self.dg = dg_comp
        self._h = self._l.oracle_kernel_create(rheology, dg_comp, byref(p))
        if not self._h:
            raise ValueError("oracle_kernel_create failed")
        self.nx = self.ny = 0

    def __del__(self):
        if getattr(self, "_h", None):
            self._l.oracle_kernel_destroy(self._h)
            self._h = None

    def _check(self, st):
        if st != 0:
            msg = self._l.oracle_kernel_last_error(self._h).decode()
            if st == 2:
                raise KeyError(msg)
            raise RuntimeError(f"[{st}] {msg}")

    @property
    def nelements(self):
        return self.nx * self.ny

    def initialise(self, coords, isSpherical, mask, nx=None, ny=None):
        mask = np.asarray(mask, dtype=np.float64)
        if nx is None:
            ny, nx = mask.shape
        c = _f64(coords).reshape(-1, 2)
        m = _f64(mask).reshape(-1)
        self._check(self._l.oracle_kernel_initialise_spherical(self._h, nx, ny, _p(c), int(bool(isSpherical)),
                                                               _p(m)))
        self.nx, self.ny = nx, ny

    def setData(self, name, data):
        a = _f64(data)
        nc = 1 if a.ndim == 1 else a.shape[-1]
        self._check(self._l.oracle_kernel_set_data(self._h, name.encode(), _p(a), self.nelements, nc))

    def getDG0Data(self, name):
        out = np.empty(self.nelements)
        self._check(self._l.oracle_kernel_get_dg0(self._h, name.encode(), _p(out), self.nelements))
        return out

    def getDGData(self, name, ncomp=None):
        nc = self.dg if ncomp is None else ncomp
        out = np.empty((self.nelements, nc))
        self._check(self._l.oracle_kernel_get_dg(self._h, name.encode(), _p(out), self.nelements, nc))
        return out if nc > 1 else out[:, 0]

    def update(self, tst, dt=None):
        start, step = (tst.start, tst.step) if hasattr(tst, "step") else (float(tst), float(dt))
        self._check(self._l.oracle_kernel_update(self._h, start, step))

    def getCG(self, name):
        n = (2 * self.nx + 1) * (2 * self.ny + 1)
        out = np.empty(n)
        self._check(self._l.oracle_kernel_get_cg(self._h, name.encode(), _p(out), n))
        return out

    def getStress(self, name):
        out = np.empty((self.nelements, 8))
        self._check(self._l.oracle_kernel_get_stress(self._h, name.encode(), _p(out), out.size))
        return out

    def meanValue(self, name):
        return self._l.oracle_kernel_mean_value(self._h, name.encode())


class OracleTransport:
    """DGTransport<DG> restated on the CPU, with the reference test helpers."""

    def __init__(self, dg, nx, ny, vertices, dirichlet, periodic=(), landmask=None, scheme="rk2"):
        self._l = load()
        self.dg, self.nx, self.ny = dg, nx, ny
        v = _f64(vertices).reshape(-1, 2)
        self._keep = [v]
        lm = None
        if landmask is not None:
            lm = np.ascontiguousarray(landmask, dtype=np.uint8)
            self._keep.append(lm)
        arrs = [np.ascontiguousarray(np.asarray(d, dtype=np.uint64).reshape(-1)) for d in dirichlet]
        self._keep += arrs
        ptrs = (c_void_p * 4)(*[a.ctypes.data if a.size else None for a in arrs])
        counts = (c_size_t * 4)(*[a.size for a in arrs])
        per = np.ascontiguousarray(np.asarray(periodic, dtype=np.uint64).reshape(-1))
        self._keep.append(per)
        sch = {"rk1": 1, "rk2": 2, "rk3": 3}[scheme]
        self._h = self._l.oracle_transport_create(dg, nx, ny, _p(v), _p(lm) if lm is not None else None, ptrs,
                                                  counts, _p(per) if per.size else None, per.size // 4, sch)

    def __del__(self):
        if getattr(self, "_h", None):
            self._l.oracle_transport_destroy(self._h)
            self._h = None

    def setVelocity(self, vx, vy):
        a, b = _f64(vx), _f64(vy)
        self._l.oracle_transport_set_velocity(self._h, _p(a), _p(b))

    def reinitnormalvelocity(self):
        self._l.oracle_transport_reinit(self._h)

    def step(self, dt, phi, nsteps=1, limit_max=None, limit_min=None):
        a = _f64(phi).copy()
        self._l.oracle_transport_step(self._h, dt, _p(a), nsteps, int(limit_max is not None),
                                      0.0 if limit_max is None else limit_max, int(limit_min is not None),
                                      0.0 if limit_min is None else limit_min)
        return a

    def meanValue(self, phi):
        a = _f64(phi)
        return self._l.oracle_transport_mean_value(self._h, _p(a))

    def limit(self, phi, limit_max=None, limit_min=None):
        a = _f64(phi).copy()
        self._l.oracle_transport_limit(self._h, _p(a), int(limit_max is not None),
                                       0.0 if limit_max is None else limit_max, int(limit_min is not None),
                                       0.0 if limit_min is None else limit_min)
        return a

    def function2dg(self, fn: int, param: float):
        out = np.empty((self.nx * self.ny, self.dg))
        self._l.oracle_transport_function2dg(self._h, fn, param, _p(out))
        return out

    def l2error(self, fn: int, param: float, phi):
        a = _f64(phi)
        return self._l.oracle_transport_l2error(self._h, fn, param, _p(a))


# Reference test functions (ids of oracle_transport_function2dg)
SMOOTH_BUMP, ROT_VX, ROT_VY, PACKMAN, RING_VX, RING_VY = range(6)


def mesh_dirichlet(nx: int, ny: int, mask) -> list:
    """The four closed-side element lists (bottom, right, top, left) the
    oracle derives from a mask (1.0 = ice), ParametricMesh.cpp:217-272."""
    m = _f64(mask)
    if m.size != nx * ny:
        raise ValueError("mask must hold nx*ny values")
    counts = (c_size_t * 4)()
    ids = np.empty(4 * nx * ny, dtype=np.uint64)
    if load().oracle_mesh_dirichlet(nx, ny, _p(m), counts, _p(ids), ids.size) != 0:
        raise RuntimeError("oracle_mesh_dirichlet failed")
    out, o = [], 0
    for c in counts:
        out.append(ids[o:o + c].astype(np.int64))
        o += c
    return out


def benchmark_forcing_fields(nx: int, ny: int, f, seconds: float):
    """(uwind, vwind, uocean, vocean) of the benchmark case on the cell
    centres, restated from the reference in numpy (element index i + nx j):
    BenchmarkCoordinates.cpp:21-40 (x = i dx, dx = length_x / nx),
    BenchmarkAtmosphere.cpp:29-77 (the cyclone; its centre moves from
    (centre_x, centre_y) at centre_v), BenchmarkOcean.cpp:15-39.  `f` holds
    the fields of nsdg_benchmark_forcing."""
    dx, dy = f.length_x / nx, f.length_y / ny
    i = np.arange(nx, dtype=np.float64)
    j = np.arange(ny, dtype=np.float64)
    x = np.tile(i * dx, ny)
    y = np.repeat(j * dy, nx)
    x0 = f.centre_x + f.centre_vx * seconds
    y0 = f.centre_y + f.centre_vy * seconds
    xp, yp = x - x0, y - y0
    a = f.wind_angle_deg / 180.0 * np.pi
    ca, sa = np.cos(a), np.sin(a)
    scale = f.wind_A * np.exp(-f.wind_k * np.hypot(xp, yp))
    uw = -scale * f.wind_vmax * (ca * xp + sa * yp)
    vw = -scale * f.wind_vmax * (-sa * xp + ca * yp)
    fx = x / (nx * dx)
    fy = y / (ny * dy)
    uo = f.ocean_vmax * (2.0 * fy - 1.0)
    vo = f.ocean_vmax * (1.0 - 2.0 * fx)
    return uw, vw, uo, vo


def rectangle_mesh(Lx, Ly, Nx, Ny, distort=0.0):
    """dynamics/test/Advection_test.cpp:198-241."""
    ix = np.arange(Nx + 1)
    iy = np.arange(Ny + 1)
    IX, IY = np.meshgrid(ix, iy)
    x = Lx * IX / Nx + Lx * distort * np.sin(np.pi * IX / Nx * 3.0) * np.sin(np.pi * IY / Ny)
    y = Ly * IY / Ny + Ly * distort * np.sin(np.pi * IY / Ny * 2.0) * np.sin(np.pi * IX / Nx * 2.0)
    verts = np.stack([x.ravel(), y.ravel()], axis=1)
    dirichlet = [list(range(Nx)), [i * Nx + Nx - 1 for i in range(Ny)],
                 [Nx * (Ny - 1) + i for i in range(Nx)], [i * Nx for i in range(Ny)]]
    return verts, dirichlet, []


def ring_mesh(R0, R1, Nx, Ny):
    """dynamics/test/AdvectionPeriodicBC_test.cpp:210-255."""
    ix = np.arange(Nx + 1)
    iy = np.arange(Ny + 1)
    IX, IY = np.meshgrid(ix, iy)
    r = R0 + (R1 - R0) * IY / Ny
    p = -2.0 * np.pi * IX / Nx
    verts = np.stack([(r * np.cos(p)).ravel(), (r * np.sin(p)).ravel()], axis=1)
    dirichlet = [list(range(Nx)), [], [Nx * (Ny - 1) + i for i in range(Nx)], []]
    periodic = [(1, (i + 1) * Nx - 1, i * Nx, i * (Nx + 1) + i) for i in range(Ny)]
    return verts, dirichlet, periodic
