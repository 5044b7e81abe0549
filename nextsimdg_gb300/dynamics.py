"""Python mirror of the reference's dynamics-kernel interface, over the C ABI.

Class and method names follow the reference so that tests and callers read
like the reference's own code:

  MEVPDynamicsKernel / BBMDynamicsKernel
      dynamics/src/include/MEVPDynamicsKernel.hpp, BBMDynamicsKernel.hpp
      initialise(coords, isSpherical, mask)   DynamicsKernel.hpp:44-75
      setData(name, data)                     DynamicsKernel.hpp:93-110,
                                              CGDynamicsKernel.cpp:54-90
      getDG0Data(name) / getDGData(name)      DynamicsKernel.hpp:119-156,
                                              CGDynamicsKernel.cpp:93-118
      update(tst)                             VPCGDynamicsKernel.hpp:63-94
  DGTransport                                 dynamics/src/include/DGTransport.hpp:27-152

Arrays use the ModelArray layout: H fields have shape (N,), DG fields
(N, ncomp) with the element index i + nx*j, coordinates ((nx+1)*(ny+1), 2).
Errors map to the exception types the reference throws: an unknown field
name raises KeyError (std::out_of_range from .at()), other failures raise
NsdgError with the library's message.
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_char_p, c_double, c_float, c_int, c_size_t, c_void_p
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import NsdgError, Params

__all__ = ["TimestepTime", "MEVPDynamicsKernel", "BBMDynamicsKernel", "Ensemble", "DGTransport", "Params",
           "NsdgError", "default_params"]

default_params = _lib.default_params


@dataclass
class TimestepTime:
    """core/src/include/Time.hpp:265-268 (start and step, in seconds)."""

    start: float
    step: float


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a: np.ndarray) -> c_void_p:
    return a.ctypes.data_as(c_void_p)


def parallelogram_mismatch(coords, nx: int, ny: int, dg_comp: int = 6) -> float:
    """Host only: the largest relative FP64 difference between a Cartesian
    mesh's exact mEVP stress operators and those rebuilt from parallelogram
    coefficients (mixed-precision handles take the parallelogram kernel when
    it is at most 1e-9)."""
    lib = _lib.load()
    c = _f64(coords)
    if c.size != 2 * (nx + 1) * (ny + 1):
        raise ValueError("coords must hold (nx+1)(ny+1) vertices x 2")
    out = c_double()
    st = lib.nsdg_mesh_parallelogram_mismatch(nx, ny, _ptr(c), dg_comp, byref(out))
    if st != _lib.NSDG_OK:
        raise NsdgError(st, "parallelogram_mismatch failed")
    return out.value


def parallelogram_checks(coords, nx: int, ny: int, dg_comp: int = 6) -> dict:
    """Host only: every check that admits the parallelogram kernels
    (nsdg_mesh_parallelogram_checks): the relative FP64 mismatch of the mEVP
    stress operators, of the transport cell operators and of the BBM
    operators rebuilt from the coefficients, and M^{-1}'s relative
    off-diagonal."""
    lib = _lib.load()
    c = _f64(coords)
    if c.size != 2 * (nx + 1) * (ny + 1):
        raise ValueError("coords must hold (nx+1)(ny+1) vertices x 2")
    out = np.zeros(4)
    st = lib.nsdg_mesh_parallelogram_checks(nx, ny, _ptr(c), dg_comp, _ptr(out))
    if st != _lib.NSDG_OK:
        raise NsdgError(st, "parallelogram_checks failed")
    return {"stress": float(out[0]), "transport_cell": float(out[1]), "minv_offdiag": float(out[2]),
            "bbm": float(out[3])}


def mesh_dirichlet(mask, nx: int, ny: int) -> list:
    """Host only: the closed (Dirichlet) element sides a handle derives from
    its mask at initialise, as four ascending arrays of element ids (bottom,
    right, top, left), ParametricMesh.cpp:217-272."""
    lib = _lib.load()
    m = _f64(mask)
    if m.size != nx * ny:
        raise ValueError("mask must hold nx*ny values")
    counts = (c_size_t * 4)()
    ids = np.empty(4 * nx * ny, dtype=np.uint64)
    st = lib.nsdg_mesh_dirichlet(nx, ny, _ptr(m), counts, _ptr(ids), ids.size)
    if st != _lib.NSDG_OK:
        raise NsdgError(st, "mesh_dirichlet failed")
    out, o = [], 0
    for c in counts:
        out.append(ids[o:o + c].astype(np.int64))
        o += c
    return out


def selftest_viscosity(inv, pa, delta_min: float) -> np.ndarray:
    """P/(8 alpha Delta) of each (inv, Pa) by the three FP64 forms of the
    mixed-precision stress kernels, shape (3, n) float32 (see
    nsdg_selftest_viscosity)."""
    lib = _lib.load()
    inv = np.ascontiguousarray(inv, dtype=np.float32)
    pa = np.ascontiguousarray(pa, dtype=np.float64)
    if inv.shape != pa.shape or inv.ndim != 1:
        raise ValueError("inv and pa must be 1-D arrays of the same length")
    out = np.empty(3 * inv.size, dtype=np.float32)
    st = lib.nsdg_selftest_viscosity(inv.size, _ptr(inv), _ptr(pa), float(delta_min), _ptr(out))
    if st != _lib.NSDG_OK:
        raise NsdgError(st, "selftest_viscosity failed")
    return out.reshape(3, inv.size)


def selftest_pairs(a, x) -> np.ndarray:
    """The float-pair arithmetic of the FP64 stress kernel on (a, x) pairs,
    shape (4, n) float64 (see nsdg_selftest_pairs)."""
    lib = _lib.load()
    a = np.ascontiguousarray(a, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    if a.shape != x.shape or a.ndim != 1:
        raise ValueError("a and x must be 1-D arrays of the same length")
    out = np.empty(4 * a.size)
    st = lib.nsdg_selftest_pairs(a.size, _ptr(a), _ptr(x), _ptr(out))
    if st != _lib.NSDG_OK:
        raise NsdgError(st, "selftest_pairs failed")
    return out.reshape(a.size, 4).T.copy()


def selftest_viscosity_ff(inv, pa, delta_min: float) -> np.ndarray:
    """The same quantity by the float-pair form 3 (FP32 pipe), shape (n,)
    float32 (see nsdg_selftest_viscosity_ff)."""
    lib = _lib.load()
    inv = np.ascontiguousarray(inv, dtype=np.float32)
    pa = np.ascontiguousarray(pa, dtype=np.float64)
    if inv.shape != pa.shape or inv.ndim != 1:
        raise ValueError("inv and pa must be 1-D arrays of the same length")
    out = np.empty(inv.size, dtype=np.float32)
    st = lib.nsdg_selftest_viscosity_ff(inv.size, _ptr(inv), _ptr(pa), float(delta_min), _ptr(out))
    if st != _lib.NSDG_OK:
        raise NsdgError(st, "selftest_viscosity_ff failed")
    return out


def selftest_viscosity_checked(inv, pa, delta_min: float) -> np.ndarray:
    """The same quantity by the kernels' form 4 (float pairs checked against
    form 2's rounding, form 2 where the check fails), shape (n,) float32;
    bitwise form 2 (see nsdg_selftest_viscosity_checked)."""
    lib = _lib.load()
    inv = np.ascontiguousarray(inv, dtype=np.float32)
    pa = np.ascontiguousarray(pa, dtype=np.float64)
    if inv.shape != pa.shape or inv.ndim != 1:
        raise ValueError("inv and pa must be 1-D arrays of the same length")
    out = np.empty(inv.size, dtype=np.float32)
    st = lib.nsdg_selftest_viscosity_checked(inv.size, _ptr(inv), _ptr(pa), float(delta_min), _ptr(out))
    if st != _lib.NSDG_OK:
        raise NsdgError(st, "selftest_viscosity_checked failed")
    return out


class _KernelBase:
    rheology = _lib.RHEOLOGY_MEVP

    def __init__(self, dg_comp: int = 6, params: Params | None = None, **overrides):
        self._l = _lib.load()
        p = params if params is not None else _lib.default_params()
        for k, v in overrides.items():
            if not hasattr(p, k):
                raise AttributeError(f"unknown parameter {k}")
            setattr(p, k, v)
        self.params = p
        self.dg = dg_comp
        h = c_void_p()
        st = self._l.nsdg_kernel_create(self.rheology, dg_comp, byref(p), byref(h))
        if st != _lib.NSDG_OK:
            raise NsdgError(st, f"nsdg_kernel_create: {self._l.nsdg_status_string(st).decode()}")
        self._h = h
        self.nx = self.ny = 0

    # -- error handling ------------------------------------------------------
    def _check(self, st: int):
        if st == _lib.NSDG_OK:
            return
        msg = self._l.nsdg_kernel_last_error(self._h).decode()
        if st == _lib.NSDG_ERR_UNKNOWN_FIELD:
            raise KeyError(msg)
        raise NsdgError(st, msg)

    def close(self):
        if getattr(self, "_h", None):
            self._l.nsdg_kernel_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- the reference interface ---------------------------------------------
    @property
    def nelements(self) -> int:
        return self.nx * self.ny

    def initialise(self, coords, isSpherical: bool, mask, nx: int | None = None, ny: int | None = None):
        """coords: ((nx+1)*(ny+1), 2) vertices; mask: (nx*ny,) with 1.0 = ice.

        The reference takes nx and ny from the ModelArray dimensions; here they
        come from the mask shape (ny, nx) or the explicit arguments."""
        mask = np.asarray(mask, dtype=np.float64)
        if nx is None or ny is None:
            if mask.ndim != 2:
                raise ValueError("pass a (ny, nx) mask or explicit nx, ny")
            ny, nx = mask.shape
        coords = _f64(coords).reshape(-1, 2)
        m = _f64(mask).reshape(-1)
        self._check(self._l.nsdg_kernel_initialise(self._h, nx, ny, _ptr(coords), int(bool(isSpherical)), _ptr(m)))
        self.nx, self.ny = nx, ny

    def benchmark_ocean(self, forcing):
        """uocean, vocean of the benchmark ocean computed on the device
        (nsdg_kernel_benchmark_ocean; BenchmarkOcean.cpp:15-39)."""
        self._check(self._l.nsdg_kernel_benchmark_ocean(self._h, byref(forcing)))

    def benchmark_atmosphere(self, forcing, seconds: float):
        """uwind, vwind of the benchmark cyclone `seconds` after the first
        update, computed on the device (nsdg_kernel_benchmark_atmosphere;
        BenchmarkAtmosphere.cpp:29-77)."""
        self._check(self._l.nsdg_kernel_benchmark_atmosphere(self._h, byref(forcing), float(seconds)))

    def setData(self, name: str, data):
        a = _f64(data)
        n = self.nelements
        ncomp = 1 if a.ndim == 1 else a.shape[-1]
        if a.size != n * ncomp:
            raise NsdgError(_lib.NSDG_ERR_SIZE_MISMATCH, f"setData: {name} has {a.size} values, mesh has {n} elements")
        self._check(self._l.nsdg_kernel_set_data(self._h, name.encode(), _ptr(a), n, ncomp))

    def getDG0Data(self, name: str, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.nelements)
        elif out.dtype != np.float64 or not out.flags.c_contiguous or out.size != self.nelements:
            raise ValueError("out must be a contiguous float64 array with one value per element")
        self._check(self._l.nsdg_kernel_get_dg0(self._h, name.encode(), _ptr(out), self.nelements))
        return out

    def module_step(self, t: float, dt: float, inputs: dict, outputs) -> dict:
        """One module step in one call (nsdg_kernel_module_step): the inputs
        (name -> array of one value or n_comp values per element, as setData
        takes them), update(t, dt), then the cell averages of the outputs
        (names, or name -> preallocated contiguous float64 arrays, as
        getDG0Data fills them).  Returns name -> array."""
        keep = []
        fin = (_lib.FieldIn * max(len(inputs), 1))()
        for i, (name, arr) in enumerate(inputs.items()):
            a = np.ascontiguousarray(arr, dtype=np.float64)
            keep.append(a)
            fin[i].name = name.encode()
            fin[i].data = a.ctypes.data
            fin[i].n_comp = 1 if a.ndim == 1 else a.shape[-1]
        if not isinstance(outputs, dict):
            outputs = {n: np.empty(self.nelements) for n in outputs}
        fout = (_lib.FieldOut * max(len(outputs), 1))()
        for j, (name, buf) in enumerate(outputs.items()):
            if buf.dtype != np.float64 or not buf.flags.c_contiguous or buf.size != self.nelements:
                raise ValueError("outputs must be contiguous float64 arrays with one value per element")
            fout[j].name = name.encode()
            fout[j].data = buf.ctypes.data
        self._check(self._l.nsdg_kernel_module_step(self._h, fin, len(inputs), float(t), float(dt), fout,
                                                    len(outputs)))
        return outputs

    def getDGData(self, name: str, ncomp: int | None = None) -> np.ndarray:
        nc = self.dg if ncomp is None else ncomp
        out = np.empty((self.nelements, nc))
        self._check(self._l.nsdg_kernel_get_dg(self._h, name.encode(), _ptr(out), self.nelements, nc))
        return out if nc > 1 else out[:, 0]

    def update(self, tst: TimestepTime | float, dt: float | None = None):
        if isinstance(tst, TimestepTime):
            start, step = tst.start, tst.step
        else:
            start, step = float(tst), float(dt)
        self._check(self._l.nsdg_kernel_update(self._h, start, step))

    # -- extras ----------------------------------------------------------------
    def synchronize(self):
        self._check(self._l.nsdg_kernel_synchronize(self._h))

    def snapshot(self) -> bytes:
        n = c_size_t()
        self._check(self._l.nsdg_kernel_snapshot_size(self._h, byref(n)))
        buf = ctypes.create_string_buffer(n.value)
        self._check(self._l.nsdg_kernel_snapshot_save(self._h, buf, n.value))
        return buf.raw

    def restore(self, blob: bytes):
        buf = ctypes.create_string_buffer(blob, len(blob))
        self._check(self._l.nsdg_kernel_snapshot_load(self._h, buf, len(blob)))

    def meanValue(self, name: str) -> float:
        out = c_double()
        self._check(self._l.nsdg_kernel_mean_value(self._h, name.encode(), byref(out)))
        return out.value

    def time_updates(self, dt: float, steps: int) -> float:
        ms = c_float()
        self._check(self._l.nsdg_kernel_time_updates(self._h, dt, steps, byref(ms)))
        return ms.value

    def time_kernel(self, kernel_id: int, reps: int):
        ms = c_float()
        name = c_char_p()
        self._check(self._l.nsdg_kernel_time_kernel(self._h, kernel_id, reps, byref(ms), byref(name)))
        return ms.value, name.value.decode()

    def launches_per_update(self) -> int:
        n = c_int()
        self._check(self._l.nsdg_kernel_launches_per_update(self._h, byref(n)))
        return n.value

    STRESS_KERNELS = ("global", "tma", "affine")

    def stress_variant(self):
        """(kind, mismatch): the mixed-precision mEVP stress kernel in use
        ("global", "tma", "affine"; None for other handles) and the largest
        relative FP64 mismatch of operators rebuilt from parallelogram
        coefficients (-1 when not evaluated)."""
        kind, mism = c_int(), c_double()
        self._check(self._l.nsdg_kernel_stress_variant(self._h, byref(kind), byref(mism)))
        return (self.STRESS_KERNELS[kind.value] if kind.value >= 0 else None), mism.value

    def transport_variant(self):
        """(kernel, cell_mismatch, offdiag): the transport stage the updates
        use ("tiled", the parallelogram-mesh kernel with edge fluxes staged
        in shared memory, or "element") and the FP64 checks that admit the
        tiled kernel (rebuilt cell operators' relative mismatch, M^{-1}'s
        relative off-diagonal; -1 when not evaluated)."""
        t, cm, od = c_int(), c_double(), c_double()
        self._check(self._l.nsdg_kernel_transport_variant(self._h, byref(t), byref(cm), byref(od)))
        return ("tiled" if t.value else "element"), cm.value, od.value

    def host_direct(self) -> bool:
        """Whether pageable host arrays move by a kernel that reads or writes
        them directly (nsdg_kernel_host_direct; NSDG_HOST_DIRECT=0 turns it
        off)."""
        d = c_int()
        self._check(self._l.nsdg_kernel_host_direct(self._h, byref(d)))
        return bool(d.value)

    def viscosity_form(self) -> int:
        """The parallelogram stress kernel's evaluation of P/(8 alpha Delta)
        (nsdg_kernel_viscosity_form: 2, the default, the FP64 Newton step;
        4 float pairs checked against it, bitwise equal)."""
        f = c_int()
        self._check(self._l.nsdg_kernel_viscosity_form(self._h, byref(f)))
        return f.value

    # -- learned warm start (mEVP, mixed precision) ------------------------------
    def warm_sample(self, tst, dt, k_iters: int, net, slot: int) -> float:
        """One plain update that also records dataset sample `slot` of `net`;
        returns the plain sub-cycle's last-iteration ratio."""
        ratio = c_double()
        self._check(self._l.nsdg_kernel_warm_sample(self._h, float(tst), float(dt), int(k_iters), net._h,
                                                    int(slot), byref(ratio)))
        return ratio.value

    def set_warm_start(self, net, k_iters: int = 0, kappa: float = 0.0, audit_every: int = 0,
                       audit_tol: float = 0.0):
        """Attaches `net` (None detaches); later updates run the network plus
        `k_iters` iterations, falling back to the full count when the
        last-iteration ratio exceeds `kappa`; every `audit_every`-th update
        also runs the plain sub-cycle and keeps the warm start enabled only
        while the warm result is within `audit_tol` (relative) of it."""
        self._check(self._l.nsdg_kernel_set_warm_start(self._h, None if net is None else net._h,
                                                       int(k_iters), float(kappa), int(audit_every),
                                                       float(audit_tol)))
        self._warm_net = net  # keeps the network alive while attached

    def warm_stats(self) -> dict:
        """Counters of the attached warm start (nsdg_warm_stats as a dict)."""
        st = _lib.WarmStats()
        self._check(self._l.nsdg_kernel_warm_stats(self._h, byref(st)))
        return st.as_dict()


class MEVPDynamicsKernel(_KernelBase):
    """mEVP rheology (MEVPDynamicsKernel.hpp, VPCGDynamicsKernel.hpp)."""

    rheology = _lib.RHEOLOGY_MEVP


class BBMDynamicsKernel(_KernelBase):
    """Brittle BBM rheology (BBMDynamicsKernel.hpp, BrittleCGDynamicsKernel.hpp)."""

    rheology = _lib.RHEOLOGY_BBM


class Ensemble:
    """Several mEVP kernels (mixed precision, possibly uneven grids) stepped
    together: per step one CUDA graph, with the mEVP sub-cycle of all members
    in one element launch and one node launch per iteration.  The members keep
    their own setData / getDG0Data."""

    def __init__(self, members):
        self._l = _lib.load()
        self.members = list(members)
        arr = (c_void_p * len(self.members))(*[m._h.value for m in self.members])
        h = c_void_p()
        st = self._l.nsdg_ensemble_create(arr, len(self.members), byref(h))
        if st != _lib.NSDG_OK:
            raise NsdgError(st, f"nsdg_ensemble_create: {self._l.nsdg_status_string(st).decode()}")
        self._h = h

    def _check(self, st):
        if st != _lib.NSDG_OK:
            raise NsdgError(st, self._l.nsdg_ensemble_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._l.nsdg_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def update(self, tst, dt=None):
        start, step = (tst.start, tst.step) if isinstance(tst, TimestepTime) else (float(tst), float(dt))
        self._check(self._l.nsdg_ensemble_update(self._h, start, step))

    def synchronize(self):
        self._check(self._l.nsdg_ensemble_synchronize(self._h))

    def time_updates(self, dt, steps):
        ms = c_float()
        self._check(self._l.nsdg_ensemble_time_updates(self._h, dt, steps, byref(ms)))
        return ms.value

    def tile(self, member):
        w, h = c_int(), c_int()
        self._check(self._l.nsdg_ensemble_tile(self._h, member, byref(w), byref(h)))
        return w.value, h.value

    def launches_per_update(self):
        n = c_int()
        self._check(self._l.nsdg_ensemble_launches_per_update(self._h, byref(n)))
        return n.value

    def set_persistent(self, on: bool = True):
        """Run the sub-cycle as one persistent cooperative launch per update
        (nsdg_ensemble_set_persistent; parallelogram members only)."""
        self._check(self._l.nsdg_ensemble_set_persistent(self._h, int(bool(on))))


class DGTransport:
    """Stand-alone DG transport (DGTransport<DG>) on an explicitly described mesh.

    vertices: ((nx+1)*(ny+1), 2); landmask: (nx*ny,) nonzero = ice or None;
    dirichlet: four lists of element ids (bottom, right, top, left);
    periodic: list of (type, cell1, cell2, edge) with type 0 for X-edges and 1
    for Y-edges; scheme: "rk1", "rk2" or "rk3".
    """

    def __init__(self, dg, nx, ny, vertices, dirichlet, periodic=(), landmask=None, scheme="rk2"):
        self._l = _lib.load()
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
        h = c_void_p()
        sch = {"rk1": 1, "rk2": 2, "rk3": 3}[scheme]
        st = self._l.nsdg_transport_create(dg, nx, ny, _ptr(v), _ptr(lm) if lm is not None else None,
                                           ptrs, counts, _ptr(per) if per.size else None, per.size // 4,
                                           sch, byref(h))
        if st != _lib.NSDG_OK:
            raise NsdgError(st, f"nsdg_transport_create: {self._l.nsdg_status_string(st).decode()}")
        self._h = h

    def _check(self, st):
        if st != _lib.NSDG_OK:
            raise NsdgError(st, self._l.nsdg_transport_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._l.nsdg_transport_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setVelocity(self, vx, vy):
        a, b = _f64(vx), _f64(vy)
        self._check(self._l.nsdg_transport_set_velocity(self._h, _ptr(a), _ptr(b)))

    def reinitnormalvelocity(self):
        self._check(self._l.nsdg_transport_reinit_normal_velocity(self._h))

    def step(self, dt, phi, nsteps=1, limit_max=None, limit_min=None) -> np.ndarray:
        a = _f64(phi).copy()
        self._check(self._l.nsdg_transport_step(
            self._h, dt, _ptr(a), nsteps, int(limit_max is not None), 0.0 if limit_max is None else limit_max,
            int(limit_min is not None), 0.0 if limit_min is None else limit_min))
        return a

    def meanValue(self, phi) -> float:
        a = _f64(phi)
        out = c_double()
        self._check(self._l.nsdg_transport_mean_value(self._h, _ptr(a), byref(out)))
        return out.value
