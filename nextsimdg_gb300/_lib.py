"""ctypes binding of libnsdg_gb300.so (the C ABI declared in include/nsdg.h).

The library is built in-tree by nextsimdg_gb300.build.  Loading fails loudly
(ImportError) when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_size_t, c_ubyte, c_void_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libnsdg_gb300.so"

NSDG_OK = 0
NSDG_ERR_BAD_ARG = 1
NSDG_ERR_UNKNOWN_FIELD = 2
NSDG_ERR_SIZE_MISMATCH = 3
NSDG_ERR_CUDA = 4
NSDG_ERR_NUMERIC = 5
NSDG_ERR_UNSUPPORTED = 6
NSDG_ERR_LOGIC = 7
NSDG_ERR_NO_DEVICE = 8

RHEOLOGY_MEVP = 0
RHEOLOGY_BBM = 1
PRECISION_FP64 = 0
PRECISION_MIXED = 1

WARM_FEATURES = 64
WARM_TARGETS = 32
WARM_USED = 26
NET_NORM_FLOATS = 192


class Params(ctypes.Structure):
    """nsdg_params (include/nsdg.h)."""

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

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class BenchmarkForcing(ctypes.Structure):
    """nsdg_benchmark_forcing (include/nsdg.h)."""

    _fields_ = [
        ("length_x", c_double), ("length_y", c_double),
        ("wind_A", c_double), ("wind_vmax", c_double), ("wind_k", c_double), ("wind_angle_deg", c_double),
        ("centre_x", c_double), ("centre_y", c_double), ("centre_vx", c_double), ("centre_vy", c_double),
        ("ocean_vmax", c_double),
    ]


class FieldIn(ctypes.Structure):
    """nsdg_field_in (include/nsdg.h)."""

    _fields_ = [("name", c_char_p), ("data", c_void_p), ("n_comp", c_size_t)]


class FieldOut(ctypes.Structure):
    """nsdg_field_out (include/nsdg.h)."""

    _fields_ = [("name", c_char_p), ("data", c_void_p)]


class WarmStats(ctypes.Structure):
    """nsdg_warm_stats (include/nsdg.h)."""

    _fields_ = [
        ("accepted", ctypes.c_longlong), ("fallbacks", ctypes.c_longlong),
        ("audited", ctypes.c_longlong), ("audit_rejected", ctypes.c_longlong),
        ("last_ratio", c_double), ("last_audit_error", c_double),
        ("enabled", c_int), ("launches_warm", c_int), ("launches_audited", c_int), ("launches_fallback", c_int),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


# (name, restype, argtypes) for every symbol in include/nsdg.h
SIGNATURES = [
    ("nsdg_default_params", None, [POINTER(Params)]),
    ("nsdg_status_string", c_char_p, [c_int]),
    ("nsdg_version", c_char_p, []),
    ("nsdg_kernel_create", c_int, [c_int, c_int, POINTER(Params), POINTER(c_void_p)]),
    ("nsdg_kernel_destroy", c_int, [c_void_p]),
    ("nsdg_kernel_last_error", c_char_p, [c_void_p]),
    ("nsdg_kernel_initialise", c_int, [c_void_p, c_size_t, c_size_t, c_void_p, c_int, c_void_p]),
    ("nsdg_kernel_set_data", c_int, [c_void_p, c_char_p, c_void_p, c_size_t, c_size_t]),
    ("nsdg_benchmark_forcing_defaults", None, [ctypes.POINTER(BenchmarkForcing), c_double, c_double]),
    ("nsdg_kernel_benchmark_ocean", c_int, [c_void_p, ctypes.POINTER(BenchmarkForcing)]),
    ("nsdg_kernel_benchmark_atmosphere", c_int, [c_void_p, ctypes.POINTER(BenchmarkForcing), c_double]),
    ("nsdg_kernel_get_dg0", c_int, [c_void_p, c_char_p, c_void_p, c_size_t]),
    ("nsdg_kernel_get_dg", c_int, [c_void_p, c_char_p, c_void_p, c_size_t, c_size_t]),
    ("nsdg_kernel_update", c_int, [c_void_p, c_double, c_double]),
    ("nsdg_kernel_synchronize", c_int, [c_void_p]),
    ("nsdg_kernel_snapshot_size", c_int, [c_void_p, POINTER(c_size_t)]),
    ("nsdg_kernel_snapshot_save", c_int, [c_void_p, c_void_p, c_size_t]),
    ("nsdg_kernel_snapshot_load", c_int, [c_void_p, c_void_p, c_size_t]),
    ("nsdg_kernel_mean_value", c_int, [c_void_p, c_char_p, POINTER(c_double)]),
    ("nsdg_kernel_time_updates", c_int, [c_void_p, c_double, c_int, POINTER(c_float)]),
    ("nsdg_kernel_time_kernel", c_int, [c_void_p, c_int, c_int, POINTER(c_float), POINTER(c_char_p)]),
    ("nsdg_kernel_launches_per_update", c_int, [c_void_p, POINTER(c_int)]),
    ("nsdg_kernel_stress_variant", c_int, [c_void_p, POINTER(c_int), POINTER(c_double)]),
    ("nsdg_kernel_transport_variant", c_int, [c_void_p, POINTER(c_int), POINTER(c_double), POINTER(c_double)]),
    ("nsdg_kernel_host_direct", c_int, [c_void_p, POINTER(c_int)]),
    ("nsdg_kernel_module_step", c_int, [c_void_p, POINTER(FieldIn), c_size_t, c_double, c_double,
                                        POINTER(FieldOut), c_size_t]),
    ("nsdg_kernel_viscosity_form", c_int, [c_void_p, POINTER(c_int)]),
    ("nsdg_transport_create", c_int, [c_int, c_size_t, c_size_t, c_void_p, c_void_p,
                                      POINTER(c_void_p), POINTER(c_size_t), c_void_p, c_size_t, c_int,
                                      POINTER(c_void_p)]),
    ("nsdg_transport_destroy", c_int, [c_void_p]),
    ("nsdg_transport_last_error", c_char_p, [c_void_p]),
    ("nsdg_transport_set_velocity", c_int, [c_void_p, c_void_p, c_void_p]),
    ("nsdg_transport_reinit_normal_velocity", c_int, [c_void_p]),
    ("nsdg_transport_step", c_int, [c_void_p, c_double, c_void_p, c_int, c_int, c_double, c_int, c_double]),
    ("nsdg_transport_mean_value", c_int, [c_void_p, c_void_p, POINTER(c_double)]),
    ("nsdg_ensemble_create", c_int, [POINTER(c_void_p), c_int, POINTER(c_void_p)]),
    ("nsdg_ensemble_destroy", c_int, [c_void_p]),
    ("nsdg_ensemble_last_error", c_char_p, [c_void_p]),
    ("nsdg_ensemble_update", c_int, [c_void_p, c_double, c_double]),
    ("nsdg_ensemble_synchronize", c_int, [c_void_p]),
    ("nsdg_ensemble_time_updates", c_int, [c_void_p, c_double, c_int, POINTER(c_float)]),
    ("nsdg_ensemble_tile", c_int, [c_void_p, c_int, POINTER(c_int), POINTER(c_int)]),
    ("nsdg_ensemble_launches_per_update", c_int, [c_void_p, POINTER(c_int)]),
    ("nsdg_ensemble_set_persistent", c_int, [c_void_p, c_int]),
    ("nsdg_net_create", c_int, [c_int, POINTER(c_int), c_int, c_int, c_int, c_int, ctypes.c_ulonglong,
                                POINTER(c_void_p)]),
    ("nsdg_net_destroy", c_int, [c_void_p]),
    ("nsdg_net_last_error", c_char_p, [c_void_p]),
    ("nsdg_net_param_count", c_int, [c_void_p, POINTER(c_size_t)]),
    ("nsdg_net_get_params", c_int, [c_void_p, c_void_p, c_size_t]),
    ("nsdg_net_set_params", c_int, [c_void_p, c_void_p, c_size_t]),
    ("nsdg_net_get_grads", c_int, [c_void_p, c_void_p, c_size_t]),
    ("nsdg_net_set_batch", c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    ("nsdg_net_forward", c_int, [c_void_p, c_int, c_void_p]),
    ("nsdg_net_time_forward", c_int, [c_void_p, c_int, c_int, POINTER(c_float)]),
    ("nsdg_net_loss_backward", c_int, [c_void_p, c_int, POINTER(c_float)]),
    ("nsdg_net_adam_step", c_int, [c_void_p, c_float, c_float, c_float, c_float]),
    ("nsdg_net_dataset_reserve", c_int, [c_void_p, c_int]),
    ("nsdg_net_dataset_normalise", c_int, [c_void_p, c_int]),
    ("nsdg_net_train", c_int, [c_void_p, c_int, c_int, c_int, c_float, ctypes.c_ulonglong, POINTER(c_float)]),
    ("nsdg_net_get_normalisation", c_int, [c_void_p, c_void_p, c_size_t]),
    ("nsdg_net_set_normalisation", c_int, [c_void_p, c_void_p, c_size_t]),
    ("nsdg_kernel_warm_sample", c_int, [c_void_p, c_double, c_double, c_int, c_void_p, c_int, POINTER(c_double)]),
    ("nsdg_kernel_set_warm_start", c_int, [c_void_p, c_void_p, c_int, c_double, c_int, c_double]),
    ("nsdg_kernel_warm_stats", c_int, [c_void_p, c_void_p]),
    ("nsdg_selftest_bounded_wait", c_int, [c_double, POINTER(c_int)]),
    ("nsdg_selftest_pairs", c_int, [c_size_t, c_void_p, c_void_p, c_void_p]),
    ("nsdg_selftest_viscosity", c_int, [c_size_t, c_void_p, c_void_p, c_double, c_void_p]),
    ("nsdg_selftest_viscosity_ff", c_int, [c_size_t, c_void_p, c_void_p, c_double, c_void_p]),
    ("nsdg_selftest_viscosity_checked", c_int, [c_size_t, c_void_p, c_void_p, c_double, c_void_p]),
    ("nsdg_mesh_parallelogram_mismatch", c_int, [c_size_t, c_size_t, c_void_p, c_int, POINTER(c_double)]),
    ("nsdg_mesh_parallelogram_checks", c_int, [c_size_t, c_size_t, c_void_p, c_int, c_void_p]),
    ("nsdg_mesh_dirichlet", c_int, [c_size_t, c_size_t, c_void_p, POINTER(c_size_t), c_void_p, c_size_t]),
    ("nsdg_mean_value_noalloc", c_int, [c_int, c_size_t, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("nsdg_ice_growth_default_params", None, [c_void_p]),
    ("nsdg_ice_growth_create", c_int, [c_size_t, c_void_p, c_void_p, POINTER(c_void_p)]),
    ("nsdg_ice_growth_destroy", c_int, [c_void_p]),
    ("nsdg_ice_growth_last_error", c_char_p, [c_void_p]),
    ("nsdg_ice_growth_set_field", c_int, [c_void_p, c_char_p, c_void_p, c_size_t]),
    ("nsdg_ice_growth_get_field", c_int, [c_void_p, c_char_p, c_void_p, c_size_t]),
    ("nsdg_ice_growth_update", c_int, [c_void_p, c_double]),
    ("nsdg_ice_growth_time_updates", c_int, [c_void_p, c_double, c_int, POINTER(c_float)]),
    ("nsdg_ice_growth_exchange", c_int, [c_void_p, c_void_p, c_int]),
    ("nsdg_restart_open", c_int, [c_char_p, POINTER(c_void_p)]),
    ("nsdg_restart_close", c_int, [c_void_p]),
    ("nsdg_restart_last_error", c_char_p, [c_void_p]),
    ("nsdg_restart_num_vars", c_int, [c_void_p, c_char_p, POINTER(c_size_t)]),
    ("nsdg_restart_var_info", c_int, [c_void_p, c_char_p, c_size_t, c_char_p, c_size_t, POINTER(c_int),
                                       POINTER(c_size_t), POINTER(c_size_t), POINTER(c_size_t)]),
    ("nsdg_restart_dim_names", c_int, [c_void_p, c_char_p, c_char_p, c_size_t]),
    ("nsdg_restart_read", c_int, [c_void_p, c_char_p, c_size_t, c_void_p, c_size_t]),
    ("nsdg_restart_text", c_int, [c_void_p, c_char_p, c_char_p, c_char_p, c_size_t]),
    ("nsdg_restart_writer_create", c_int, [c_size_t, c_size_t, c_size_t, c_int, c_int, c_int, c_char_p,
                                            ctypes.c_longlong, c_char_p, POINTER(c_void_p)]),
    ("nsdg_restart_writer_add", c_int, [c_void_p, c_char_p, c_int, c_void_p, c_size_t]),
    ("nsdg_restart_writer_save", c_int, [c_void_p, c_char_p]),
    ("nsdg_restart_writer_destroy", c_int, [c_void_p]),
    ("nsdg_restart_writer_last_error", c_char_p, [c_void_p]),
    ("nsdg_diagnostic_writer_create", c_int, [c_size_t, c_size_t, c_size_t, c_int, c_int, c_int, c_char_p,
                                               ctypes.c_longlong, c_char_p, POINTER(c_void_p)]),
    ("nsdg_diagnostic_writer_record", c_int, [c_void_p, c_double, c_size_t, POINTER(c_char_p), POINTER(c_int),
                                               POINTER(c_void_p), POINTER(c_size_t)]),
]

_lib = None


def load(path: Path | str | None = None) -> ctypes.CDLL:
    """Loads the in-tree library (once) and declares every signature."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(
            f"{p} is missing: build it with `python -m nextsimdg_gb300.build` "
            "(the dynamics kernel has no CPU fallback)")
    lib = ctypes.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class IceGrowthParams(ctypes.Structure):
    """nsdg_ice_growth_params (include/nsdg.h)."""

    _fields_ = [
        ("ks", c_double), ("h_min", c_double), ("c_min", c_double), ("h0", c_double), ("phi_m", c_double),
        ("healing_time", c_double), ("use_thermo", c_int), ("thermo_model", c_int),
        ("lateral_model", c_int), ("healing_model", c_int), ("flooding", c_int),
    ]


# the field slots of the ice-growth handle (NSDG_IG_* in include/nsdg.h), in order
ICE_GROWTH_FIELDS = (
    "hice", "cice", "hsnow", "tice", "qia", "dqia_dt", "qow", "qio", "sublim", "snowfall", "penSW", "sst", "tf",
    "mlbhc", "damage", "hice_updated", "cice_updated", "hsnow_updated", "hice_initial", "hsnow_initial", "newice",
    "delta_cice", "delta_hice", "tice_updated", "qic", "snow_to_ice", "top_melt", "bottom_melt", "snow_melt",
    "delta_cfreeze", "delta_cmelt", "tice_1", "tice_2", "tice_updated_1", "tice_updated_2")


def benchmark_forcing(length_x: float = 512e3, length_y: float = 512e3, **overrides) -> BenchmarkForcing:
    """The reference's benchmark forcing constants for a box of the given size
    (nsdg_benchmark_forcing_defaults), with overrides."""
    f = BenchmarkForcing()
    load().nsdg_benchmark_forcing_defaults(ctypes.byref(f), float(length_x), float(length_y))
    for k, v in overrides.items():
        if not hasattr(f, k):
            raise AttributeError(f"unknown forcing parameter {k}")
        setattr(f, k, float(v))
    return f


def default_params() -> Params:
    p = Params()
    load().nsdg_default_params(ctypes.byref(p))
    return p


class NsdgError(RuntimeError):
    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"[{status}] {message}")
