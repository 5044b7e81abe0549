"""Restart and forcing files in ParaGridIO's NetCDF-4 layout, read through the
C ABI (nsdg_restart_* in include/nsdg.h) by the library's own HDF5-subset
reader: no netCDF or HDF5 library is needed on either machine.

Mirrors the read side of the reference's ParaGridIO (core/src/ParaGridIO.cpp):

* ``get_model_state()`` is ParaGridIO::getModelState (:87-208): every
  variable of the "data" group whose dimension names form one of the
  reference's dimension keys (:34-47), as a ModelArray-ordered array of the
  matching type; a variable with any other key raises KeyError, as the
  reference throws std::out_of_range.
* ``read_forcing_time_static(fields, t)`` is ParaGridIO::readForcingTimeStatic
  (:210-270): the record of the "time" axis with the largest time not after
  t (the first record when t precedes the axis), for each requested field
  present in the file (absent ones are skipped, as there).
* ``dump_model_state(path, state, ...)`` is ParaGridIO::dumpModelState
  (:272-348): the restart fields of the state (the reference's
  restartFields set) written with CommonRestartMetadata's groups.
* ``structure_type()`` is the "structure" group's "type" attribute
  (ParametricGrid checks it is "parametric_rectangular"), ``metadata_time()``
  the "metadata/time" variables ModelMetadata reads.

Arrays come back flat in ModelArray order (index = component +
n_components * (i + nx * j)), the layout ``MEVPDynamicsKernel.setData`` takes.
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_int, c_size_t, c_void_p
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import NsdgError

MODEL_TYPES = {0: "H", 1: "VERTEX", 2: "U", 3: "V", 4: "Z", 5: "DG", 6: "DGSTRESS", 7: "CG", -1: None}


@dataclass
class VarInfo:
    name: str
    model_type: str | None   # ModelArray::Type name, None when the dimensions form no known key
    n_components: int
    n_records: int           # entries of the leading "time" axis (1 without one)
    n_values: int            # values per record
    dim_names: tuple


class ParaGridFile:
    """One open restart, forcing or diagnostic file (read only)."""

    def __init__(self, path):
        self._lib = _lib.load()
        h = c_void_p()
        st = self._lib.nsdg_restart_open(str(path).encode(), byref(h))
        if st != _lib.NSDG_OK:
            msg = self._lib.nsdg_restart_last_error(None).decode()
            if st == _lib.NSDG_ERR_BAD_ARG:
                raise FileNotFoundError(msg)
            raise NsdgError(st, msg)
        self._h = h
        self.path = str(path)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.nsdg_restart_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()

    def _check(self, st, what):
        if st == _lib.NSDG_ERR_UNKNOWN_FIELD:
            raise KeyError(self._lib.nsdg_restart_last_error(self._h).decode() or what)
        if st != _lib.NSDG_OK:
            raise NsdgError(st, f"{what}: {self._lib.nsdg_restart_last_error(self._h).decode()}")

    def variables(self, group: str = "data") -> list[VarInfo]:
        n = c_size_t()
        self._check(self._lib.nsdg_restart_num_vars(self._h, group.encode(), byref(n)), group)
        out = []
        name = ctypes.create_string_buffer(1024)
        for i in range(n.value):
            t, nc, nr, nv = c_int(), c_size_t(), c_size_t(), c_size_t()
            self._check(self._lib.nsdg_restart_var_info(self._h, group.encode(), i, name, len(name), byref(t),
                                                        byref(nc), byref(nr), byref(nv)), group)
            vname = name.value.decode()
            path = f"{group}/{vname}" if group else vname
            out.append(VarInfo(vname, MODEL_TYPES[t.value], nc.value, nr.value, nv.value, self.dim_names(path)))
        return out

    def dim_names(self, path: str) -> tuple:
        buf = ctypes.create_string_buffer(4096)
        self._check(self._lib.nsdg_restart_dim_names(self._h, path.encode(), buf, len(buf)), path)
        return tuple(buf.value.decode().split(",")) if buf.value else ()

    def read(self, path: str, record: int = 0) -> np.ndarray:
        """Record `record` of the variable at `path` ("data/hice"), flat, as float64."""
        group, _, name = path.rpartition("/")
        info = next((v for v in self.variables(group) if v.name == name), None)
        if info is None:
            raise KeyError(f"no variable {path} in {self.path}")
        out = np.empty(info.n_values, dtype=np.float64)
        self._check(self._lib.nsdg_restart_read(self._h, path.encode(), record,
                                                out.ctypes.data_as(c_void_p), out.size), path)
        return out

    def text(self, path: str, attribute: str | None = None) -> str:
        buf = ctypes.create_string_buffer(1 << 16)
        self._check(self._lib.nsdg_restart_text(self._h, path.encode(),
                                                attribute.encode() if attribute else None, buf, len(buf)), path)
        return buf.value.decode()

    # ---- ParaGridIO's read side
    def structure_type(self) -> str:
        return self.text("structure", "type")

    def metadata_time(self) -> tuple[float, str]:
        """(seconds since the epoch, formatted) of "metadata/time": the
        formatted time is an attribute of the time variable in the files
        CommonRestartMetadata writes, a string variable in older inputs."""
        t = float(self.read("metadata/time/time")[0])
        try:
            return t, self.text("metadata/time/time", "formatted")
        except KeyError:
            return t, self.text("metadata/time/formatted")

    def get_model_state(self) -> dict[str, tuple[str, np.ndarray]]:
        state = {}
        for v in self.variables("data"):
            if v.model_type is None:
                raise KeyError(f"No ModelArray::Type corresponds to the dimensional key {''.join(v.dim_names)}")
            state[v.name] = (v.model_type, self.read(f"data/{v.name}"))
        return state

    def read_forcing_time_static(self, fields, time_seconds: float) -> dict[str, np.ndarray]:
        times = self.read("data/time")
        later = np.nonzero(times > time_seconds)[0]
        idx = int(later[0]) if later.size else times.size
        idx = max(idx - 1, 0)
        present = {v.name for v in self.variables("data")}
        return {f: self.read(f"data/{f}", idx) for f in fields if f in present}


# ParaGridIO::dumpModelState's restartFields (core/src/ParaGridIO.cpp:309-311)
RESTART_FIELDS = {"hice", "cice", "hsnow", "tice", "sst", "sss", "mask", "coords", "x", "y", "longitude",
                  "latitude", "grid_azimuth", "u", "v", "damage"}
_TYPE_CODES = {v: k for k, v in MODEL_TYPES.items() if v}


def dump_model_state(path, state: dict, nx: int, ny: int, *, nz: int = 1, dg_comp: int = 6,
                     dgstress_comp: int = 8, cg_degree: int = 2, time_seconds: int = 0,
                     time_formatted: str = "1970-01-01T00:00:00Z",
                     structure_type: str = "parametric_rectangular") -> list[str]:
    """Writes the restart fields of `state` ({name: (type name, flat array in
    ModelArray order)}) in name order, as the reference iterates its
    std::map, and returns the names written; other names are skipped."""
    lib = _lib.load()
    w = c_void_p()
    st = lib.nsdg_restart_writer_create(nx, ny, nz, dg_comp, dgstress_comp, cg_degree, structure_type.encode(),
                                        int(time_seconds), time_formatted.encode(), byref(w))
    if st != _lib.NSDG_OK:
        raise NsdgError(st, "nsdg_restart_writer_create")
    written = []
    try:
        for name in sorted(state):
            if name not in RESTART_FIELDS:
                continue
            mtype, arr = state[name]
            a = np.ascontiguousarray(arr, dtype=np.float64).ravel()
            st = lib.nsdg_restart_writer_add(w, name.encode(), _TYPE_CODES[mtype], a.ctypes.data_as(c_void_p),
                                             a.size)
            if st != _lib.NSDG_OK:
                raise NsdgError(st, f"{name}: {lib.nsdg_restart_writer_last_error(w).decode()}")
            written.append(name)
        st = lib.nsdg_restart_writer_save(w, str(path).encode())
        if st != _lib.NSDG_OK:
            raise NsdgError(st, lib.nsdg_restart_writer_last_error(w).decode())
    finally:
        lib.nsdg_restart_writer_destroy(w)
    return written


class DiagnosticFile:
    """ParaGridIO::writeDiagnosticTime (core/src/ParaGridIO.cpp:350-500):
    ``write(state, t)`` appends one record of every field of the state at time
    t (seconds since 1970); "mask" and VERTEX fields are written with the
    first record only.  Records stay in host memory until ``close()`` writes
    the file, as the reference's file is finished when ParaGridIO closes it."""

    def __init__(self, path, nx: int, ny: int, *, nz: int = 1, dg_comp: int = 6, dgstress_comp: int = 8,
                 cg_degree: int = 2, time_seconds: int = 0, time_formatted: str = "1970-01-01T00:00:00Z",
                 structure_type: str = "parametric_rectangular"):
        self._lib = _lib.load()
        self.path = str(path)
        w = c_void_p()
        st = self._lib.nsdg_diagnostic_writer_create(nx, ny, nz, dg_comp, dgstress_comp, cg_degree,
                                                     structure_type.encode(), int(time_seconds),
                                                     time_formatted.encode(), byref(w))
        if st != _lib.NSDG_OK:
            raise NsdgError(st, "nsdg_diagnostic_writer_create")
        self._w = w

    def write(self, state: dict, time_seconds: float):
        names = sorted(state)  # the reference iterates its std::map in name order
        arrays = [np.ascontiguousarray(state[n][1], dtype=np.float64).ravel() for n in names]
        c_names = (ctypes.c_char_p * len(names))(*[n.encode() for n in names])
        c_types = (c_int * len(names))(*[_TYPE_CODES[state[n][0]] for n in names])
        c_data = (c_void_p * len(names))(*[a.ctypes.data_as(c_void_p) for a in arrays])
        c_n = (c_size_t * len(names))(*[a.size for a in arrays])
        st = self._lib.nsdg_diagnostic_writer_record(self._w, float(time_seconds), len(names), c_names, c_types,
                                                     c_data, c_n)
        if st == _lib.NSDG_ERR_UNKNOWN_FIELD:
            raise KeyError(self._lib.nsdg_restart_writer_last_error(self._w).decode())
        if st != _lib.NSDG_OK:
            raise NsdgError(st, self._lib.nsdg_restart_writer_last_error(self._w).decode())

    def close(self):
        if getattr(self, "_w", None):
            try:
                st = self._lib.nsdg_restart_writer_save(self._w, self.path.encode())
                if st != _lib.NSDG_OK:
                    raise NsdgError(st, self._lib.nsdg_restart_writer_last_error(self._w).decode())
            finally:
                self._lib.nsdg_restart_writer_destroy(self._w)
                self._w = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
