"""Column thermodynamics on the GPU: the reference's IceGrowth
(physics/src/IceGrowth.cpp) with its default modules ThermoIce0, HiblerSpread
and ConstantHealing (or ThermoWinton, DummyIceThermodynamics, DummyIceSpread,
NoHealing),
through the C ABI (nsdg_ice_growth_* in include/nsdg.h).

The interface mirrors the module's data flow: the prognostic cell averages
("hice", "cice", "hsnow", "tice") and the forcing the boundary and flux
modules provide are set by name; ``update(dt)`` is IceGrowth::update for a
time step of dt seconds; the updated fields are read by the names of
IceGrowth's state ("hice_updated", "cice_updated", "hsnow_updated",
"hice_initial", ...).  ``exchange(kernel, direction)`` couples it with a
dynamics handle on the device, as PrognosticData::update does through host
arrays.
"""
from __future__ import annotations

from ctypes import byref, c_float, c_void_p

import numpy as np

from . import _lib
from ._lib import ICE_GROWTH_FIELDS, IceGrowthParams, NsdgError

THERMO_MODELS = {"ThermoIce0": 0, "DummyIceThermodynamics": 1, "ThermoWinton": 2}
LATERAL_MODELS = {"HiblerSpread": 0, "DummyIceSpread": 1}
HEALING_MODELS = {"ConstantHealing": 0, "NoHealing": 1}


def default_params(**overrides) -> IceGrowthParams:
    p = IceGrowthParams()
    _lib.load().nsdg_ice_growth_default_params(byref(p))
    for k, v in overrides.items():
        if not hasattr(p, k):
            raise AttributeError(f"unknown parameter {k}")
        setattr(p, k, v)
    return p


class IceGrowth:
    FIELDS = ICE_GROWTH_FIELDS

    def __init__(self, n_elements: int, mask=None, params: IceGrowthParams | None = None, **overrides):
        self._l = _lib.load()
        self.params = params if params is not None else default_params(**overrides)
        self.n = int(n_elements)
        self._h = c_void_p()
        m = None
        if mask is not None:
            m = np.ascontiguousarray(mask, dtype=np.float64).ravel()
            if m.size != self.n:
                raise ValueError("mask must hold one value per element")
        st = self._l.nsdg_ice_growth_create(self.n, None if m is None else m.ctypes.data_as(c_void_p),
                                            byref(self.params), byref(self._h))
        if st != _lib.NSDG_OK:
            raise NsdgError(st, "nsdg_ice_growth_create failed")

    def close(self):
        if self._h:
            self._l.nsdg_ice_growth_destroy(self._h)
            self._h = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int):
        if st != _lib.NSDG_OK:
            msg = self._l.nsdg_ice_growth_last_error(self._h)
            raise NsdgError(st, msg.decode() if msg else "")

    def setData(self, name: str, data):
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(data, dtype=np.float64).ravel(), (self.n,)))
        self._check(self._l.nsdg_ice_growth_set_field(self._h, name.encode(), a.ctypes.data_as(c_void_p), a.size))

    def getData(self, name: str) -> np.ndarray:
        out = np.empty(self.n)
        self._check(self._l.nsdg_ice_growth_get_field(self._h, name.encode(), out.ctypes.data_as(c_void_p),
                                                      out.size))
        return out

    def update(self, dt: float):
        self._check(self._l.nsdg_ice_growth_update(self._h, float(dt)))

    def time_updates(self, dt: float, reps: int) -> float:
        ms = c_float()
        self._check(self._l.nsdg_ice_growth_time_updates(self._h, float(dt), int(reps), byref(ms)))
        return ms.value

    def exchange(self, kernel, direction: int):
        """0: the dynamics' DG0 thickness, concentration (and BBM damage)
        become this step's inputs; 1: the updated cell averages go back into
        the dynamics' fields (component 0, higher components zeroed)."""
        self._check(self._l.nsdg_ice_growth_exchange(self._h, kernel._h, int(direction)))
