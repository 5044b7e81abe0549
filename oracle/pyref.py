"""ctypes binding of the reference build (oracle/_ref/libnsdg_ref.so).

TEST INFRASTRUCTURE ONLY.  The library holds the reference's own dynamics
sources, unmodified, compiled against the project's Eigen 3.4 API subset
(oracle/eigen_min) by `make -C oracle ref`; oracle/ref_harness.cpp is its C
ABI.  It can only be built where the reference sources are, so on any other
machine `available()` is False and the tests that need it skip; the golden
fixtures under tests/golden/ carry its results there.

RefKernel mirrors the interface of the product's Python mirror
(nextsimdg_gb300.dynamics) and of oracle.pyoracle.OracleKernel, so one test
drives all three with the same calls.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, byref, c_char_p, c_double, c_int, c_size_t, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_ref" / "libnsdg_ref.so"


def reference_root() -> Path | None:
    """The reference source tree: $NSDG_REFERENCE, else the location the
    build recipe (oracle/Makefile) uses by default; None if neither holds
    the dynamics sources."""
    cands = [os.environ.get("NSDG_REFERENCE"), _recipe_default()]
    for c in cands:
        if c and (Path(c) / "dynamics" / "src" / "CGDynamicsKernel.cpp").exists():
            return Path(c)
    return None


def _recipe_default() -> str | None:
    for line in (HERE / "Makefile").read_text().splitlines():
        if line.startswith("REF_DEFAULT :="):
            return line.split(":=", 1)[1].strip()
    return None


def build(force: bool = False) -> Path | None:
    """Runs the recipe when the reference sources are present (make decides
    what is stale).  Returns the library path, or None when it cannot be
    built here."""
    root = reference_root()
    if root is None:
        return LIB if LIB.exists() else None
    cmd = ["make", "-C", str(HERE), "ref", f"REF={root}", f"-j{os.cpu_count() or 4}"]
    if force:
        cmd.insert(1, "-B")
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL)
    return LIB


def available() -> bool:
    return LIB.exists()


_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise FileNotFoundError(f"{LIB} is not built (make -C oracle ref REF=<reference sources>)")
        lib = ctypes.CDLL(str(LIB))
        sig = {
            "ref_kernel_create": (c_void_p, [c_int, c_int, c_double, c_double, c_int]),
            "ref_kernel_destroy": (None, [c_void_p]),
            "ref_kernel_last_error": (c_char_p, [c_void_p]),
            "ref_kernel_initialise": (c_int, [c_void_p, c_size_t, c_size_t, c_void_p, c_int, c_void_p]),
            "ref_kernel_set_data": (c_int, [c_void_p, c_char_p, c_void_p, c_size_t, c_size_t]),
            "ref_kernel_get_dg0": (c_int, [c_void_p, c_char_p, c_void_p, c_size_t]),
            "ref_kernel_get_dg": (c_int, [c_void_p, c_char_p, c_void_p, c_size_t, c_size_t]),
            "ref_kernel_update": (c_int, [c_void_p, c_double, c_double]),
            "ref_kernel_get_cg": (c_int, [c_void_p, c_char_p, c_void_p, c_size_t]),
            "ref_kernel_get_stress": (c_int, [c_void_p, c_char_p, c_void_p, c_size_t]),
            "ref_advection_golden": (c_double, [c_int, c_double, c_int, POINTER(c_double)]),
            "ref_periodic_golden": (c_double, [c_int, c_int, POINTER(c_double)]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a):
    return a.ctypes.data_as(c_void_p)


def advection_golden(dg: int, distort: float, it: int) -> tuple[float, float]:
    """(L2 error, relative mass loss) of Advection_test.cpp's rotating bump."""
    m = c_double()
    e = load().ref_advection_golden(dg, distort, it, byref(m))
    return e, m.value


def periodic_golden(dg: int, it: int) -> tuple[float, float]:
    """(L2 error, relative mass loss) of AdvectionPeriodicBC_test.cpp."""
    m = c_double()
    e = load().ref_periodic_golden(dg, it, byref(m))
    return e, m.value


class RefKernel:
    """MEVPDynamicsKernel<DG> (rheology 0) or BBMDynamicsKernel<DG>
    (rheology 1) of the reference, with CG2 velocity and DG-stress 8.  alpha
    and beta are the mEVP relaxation constants (the reference fixes 1500);
    n_steps the sub-cycle count (the reference fixes 100)."""

    def __init__(self, rheology: int = 0, dg_comp: int = 6, alpha: float = 1500.0, beta: float = 1500.0,
                 n_steps: int = 100):
        self._l = load()
        self.dg = dg_comp
        self._h = self._l.ref_kernel_create(rheology, dg_comp, float(alpha), float(beta), int(n_steps))
        if not self._h:
            raise ValueError("ref_kernel_create: rheology 0/1 and dg_comp 1, 3 or 6")
        self.nx = self.ny = 0

    def __del__(self):
        if getattr(self, "_h", None):
            self._l.ref_kernel_destroy(self._h)
            self._h = None

    def close(self):
        self.__del__()

    def _check(self, st):
        if st != 0:
            msg = self._l.ref_kernel_last_error(self._h).decode()
            if st == 2:
                raise KeyError(msg)
            raise RuntimeError(f"[{st}] {msg}")

    @property
    def nelements(self):
        return self.nx * self.ny

    def initialise(self, coords, isSpherical, mask):
        m = _f64(mask)
        ny, nx = m.shape
        c = _f64(coords).reshape(-1, 2)
        self._check(self._l.ref_kernel_initialise(self._h, nx, ny, _p(c), int(bool(isSpherical)),
                                                  _p(m.reshape(-1))))
        self.nx, self.ny = nx, ny

    def setData(self, name, data):
        a = _f64(data)
        nc = 1 if a.ndim == 1 else a.shape[-1]
        self._check(self._l.ref_kernel_set_data(self._h, name.encode(), _p(a), self.nelements, nc))

    def getDG0Data(self, name):
        out = np.empty(self.nelements)
        self._check(self._l.ref_kernel_get_dg0(self._h, name.encode(), _p(out), self.nelements))
        return out

    def getDGData(self, name, ncomp=None):
        nc = self.dg if ncomp is None else ncomp
        out = np.empty((self.nelements, nc))
        self._check(self._l.ref_kernel_get_dg(self._h, name.encode(), _p(out), self.nelements, nc))
        return out if nc > 1 else out[:, 0]

    def update(self, tst, dt=None):
        start, step = (tst.start, tst.step) if hasattr(tst, "step") else (float(tst), float(dt))
        self._check(self._l.ref_kernel_update(self._h, start, step))

    def getCG(self, name):
        n = (2 * self.nx + 1) * (2 * self.ny + 1)
        out = np.empty(n)
        self._check(self._l.ref_kernel_get_cg(self._h, name.encode(), _p(out), n))
        return out

    def getStress(self, name):
        out = np.empty((self.nelements, 8))
        self._check(self._l.ref_kernel_get_stress(self._h, name.encode(), _p(out), out.size))
        return out


# -- the module build (oracle/_ref/libnsdg_module.so) ----------------------
MODLIB = HERE / "_ref" / "libnsdg_module.so"
_mlib = None


def build_module() -> Path | None:
    """`make -C oracle module` where the reference sources are (needs the
    product library nextsimdg_gb300/libnsdg_gb300.so).  None when it cannot
    be built here."""
    root = reference_root()
    if root is None:
        return MODLIB if MODLIB.exists() else None
    subprocess.run(["make", "-C", str(HERE), "module", f"REF={root}", f"-j{os.cpu_count() or 4}"], check=True,
                   stdout=subprocess.DEVNULL)
    return MODLIB


def load_module() -> ctypes.CDLL:
    global _mlib
    if _mlib is None:
        if not MODLIB.exists():
            raise FileNotFoundError(f"{MODLIB} is not built (make -C oracle module REF=<reference sources>)")
        lib = ctypes.CDLL(str(MODLIB))
        sig = {
            "mod_last_error": (c_char_p, [c_void_p]),
            "mod_create": (c_void_p, [c_char_p, c_size_t, c_size_t, c_int]),
            "mod_destroy": (None, [c_void_p]),
            "mod_configure": (c_int, [c_void_p, c_char_p]),
            "mod_precision": (c_int, [c_void_p]),
            "mod_set_state": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_void_p]),
            "mod_step": (c_int, [c_void_p, c_double, c_double, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
            "mod_get": (c_int, [c_void_p, c_char_p, c_void_p, c_size_t]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _mlib = lib
    return _mlib


class DynamicsModule:
    """A dynamics module of the model: "MEVPDynamics" or "BBMDynamics" (the
    reference's own), "GPUMEVPDynamics" or "GPUBBMDynamics" (the product's
    adapters), driven as the model drives it: setData with the initial
    state, then per step the forcing put into the shared store and update."""

    def __init__(self, kind: str, nx: int, ny: int, precision: int = 0):
        self._l = load_module()
        self._h = self._l.mod_create(kind.encode(), nx, ny, precision)
        if not self._h:
            raise RuntimeError(self._l.mod_last_error(None).decode())
        self.kind, self.nx, self.ny = kind, nx, ny

    def close(self):
        if getattr(self, "_h", None):
            self._l.mod_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def _check(self, st):
        if st != 0:
            raise RuntimeError(self._l.mod_last_error(self._h).decode())

    def configure(self, text: str = ""):
        self._check(self._l.mod_configure(self._h, text.encode()))

    @property
    def precision(self) -> int:
        return self._l.mod_precision(self._h)

    def set_state(self, coords, mask, hice, cice, u, v, damage=None, spherical=False):
        arrs = [_f64(a) for a in (coords, mask, hice, cice, u, v)]
        d = None if damage is None else _f64(damage)
        self._check(self._l.mod_set_state(self._h, _p(arrs[0]), int(spherical), *[_p(a) for a in arrs[1:]],
                                          None if d is None else _p(d)))

    def step(self, t: float, dt: float, uwind=None, vwind=None, uocean=None, vocean=None, ssh=None):
        arrs = [None if a is None else _f64(a) for a in (uwind, vwind, uocean, vocean, ssh)]
        self._check(self._l.mod_step(self._h, float(t), float(dt), *[None if a is None else _p(a) for a in arrs]))

    def get(self, name: str) -> np.ndarray:
        out = np.empty(self.nx * self.ny)
        self._check(self._l.mod_get(self._h, name.encode(), _p(out), out.size))
        return out
