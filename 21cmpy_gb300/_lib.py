"""ctypes binding of the engine's C ABI (include/es_engine.h).

The library is loaded from the package directory only; there is no fallback: if it is missing
or fails to load, every engine call raises :class:`EngineUnavailable`.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libes_engine.so"

ES_OK = 0
ES_E_ARG, ES_E_CUDA, ES_E_NOMEM, ES_E_UNSUPPORTED, ES_E_DEVICE = -1, -2, -3, -4, -5
# kernel kinds reported by es_profile_read (ES_PROF_* in include/es_engine.h)
PROF_KINDS = ("col_z_fwd", "col_y_fwd", "col_z_inv_filter", "col_y_inv", "col_z_fwd_pk", "row_r2c",
              "row_r2c_pk", "row_c2r", "row_c2r_ionize", "col_z_inv", "filter_table", "final",
              "delta_T", "paint")
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "out of device memory", -4: "unsupported box size",
          -5: "device-side wait timed out"}
OPT_COL_VARIANT = 1
OPT_COL_TILE = 2
OPT_ROW_TILE = 3
OPT_L2_HINTS = 4
OPT_COL_RADIX = 5
OPT_ROW_RADIX = 6
OPT_OVERLAP = 7
OPT_ROW_CTAS = 8
OPT_COL_CTAS = 9
OPT_WAIT_LOG2 = 10
OPT_DEBUG_STALL = 11
STALL_COL_Z_INV = 1
STALL_ROW_C2R = 2
STALL_ROW_R2C = 3


class EngineUnavailable(RuntimeError):
    """The compiled CUDA engine is not built or cannot be loaded."""


class EngineError(RuntimeError):
    """A C-ABI call returned a failure code."""

    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn} failed ({ERRORS.get(code, code)}): {msg}")
        self.code = code


class es_radius(C.Structure):
    _fields_ = [("R", C.c_float), ("denom", C.c_float)]


class es_ionize_params(C.Structure):
    _fields_ = [
        ("n_radii", C.c_int), ("radii", C.POINTER(es_radius)),
        ("delta_c", C.c_float), ("fc_mean_ps", C.c_float), ("zeta", C.c_float),
        ("growth_scale", C.c_float), ("normalize_mean", C.c_int), ("filter_type", C.c_int),
        ("update", C.c_int), ("ref_compat", C.c_int), ("output", C.c_int),
    ]


class es_batch_box(C.Structure):
    _fields_ = [("n", C.c_int), ("box_len", C.c_double), ("delta", C.c_void_p), ("out", C.c_void_p),
                ("nf", C.c_void_p), ("params", es_ionize_params), ("t_factor", C.c_float), ("dT", C.c_void_p),
                ("ave", C.c_void_p), ("k2_thresholds", C.POINTER(C.c_int)), ("nbins", C.c_int),
                ("dimensional", C.c_int), ("pk", C.c_void_p)]


_PROTOS = {
    "es_plan_create": (C.c_int, [C.c_int, C.c_double, C.c_int, C.POINTER(C.c_void_p)]),
    "es_plan_destroy": (C.c_int, [C.c_void_p]),
    "es_plan_workspace_bytes": (C.c_size_t, [C.c_int, C.c_int]),
    "es_supported_sizes": (C.c_int, [C.POINTER(C.c_int), C.c_int]),
    "es_plan_set_option": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "es_plan_get_option": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "es_plan_check": (C.c_int, [C.c_void_p, C.c_void_p]),
    "es_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "es_ionize": (C.c_int, [C.c_void_p, C.POINTER(es_ionize_params), C.c_void_p, C.c_void_p, C.c_void_p]),
    "es_delta_T": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]),
    "es_delta_T_noalloc": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]),
    "es_power_spectrum": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int), C.c_int, C.c_int,
                                    C.c_void_p, C.c_void_p]),
    "es_fft_r2c": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "es_fft_c2r": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "es_profile_enable": (C.c_int, [C.c_void_p, C.c_int]),
    "es_profile_reset": (C.c_int, [C.c_void_p]),
    "es_profile_read": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_int), C.c_int]),
    "es_selftest_erfc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "es_batch_create": (C.c_int, [C.POINTER(es_batch_box), C.c_int, C.POINTER(C.c_void_p)]),
    "es_batch_run": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "es_batch_check": (C.c_int, [C.c_void_p, C.c_void_p]),
    "es_batch_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_uint),
                                C.POINTER(C.c_int)]),
    "es_batch_set_schedule": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "es_batch_profile": (C.c_int, [C.c_void_p, C.c_int]),
    "es_batch_profile_read": (C.c_int, [C.c_void_p, C.POINTER(C.c_ulonglong), C.c_int]),
    "es_batch_get_schedule": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_uint)]),
    "es_batch_queue": (C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                 C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.c_int]),
    "es_batch_destroy": (C.c_int, [C.c_void_p]),
    "es_batch_debug_stall": (C.c_int, [C.c_void_p, C.c_int, C.c_long]),
    "es_batch_last_error": (C.c_int, [C.c_char_p, C.c_int]),
    "sg_conv3d_fwd": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_void_p]),
    "sg_conv3d_wgrad": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_size_t, C.c_void_p]),
    "sg_conv3d_wgrad_workspace": (C.c_size_t, [C.c_int, C.c_int, C.c_int]),
    "sg_conv3d_set_impl": (C.c_int, [C.c_int]),
    "sg_conv3d_get_impl": (C.c_int, []),
    "sg_features": (C.c_int, [C.c_int, C.c_void_p, C.c_float, C.POINTER(C.c_uint16), C.c_void_p, C.c_void_p]),
    "sg_features_ms": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.POINTER(C.c_uint16),
                                 C.c_void_p, C.c_void_p]),
    "sg_check": (C.c_int, []),
    "sg_last_error": (C.c_int, [C.c_char_p, C.c_int]),
    "pf_plan_create": (C.c_int, [C.c_int, C.c_int, C.c_float, C.POINTER(C.c_void_p)]),
    "pf_plan_destroy": (C.c_int, [C.c_void_p]),
    "pf_move_mass": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_float,
                               C.c_float, C.c_void_p, C.c_void_p]),
    "pf_evolve_linear": (C.c_int, [C.c_longlong, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p]),
    "pf_last_error": (C.c_int, [C.c_char_p, C.c_int]),
    "ic_spectrum": (C.c_int, [C.c_int, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                              C.c_void_p, C.c_void_p]),
    "ic_shape": (C.c_int, [C.c_int, C.c_float, C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_int, C.c_void_p,
                           C.c_void_p]),
    "ic_subsample": (C.c_int, [C.c_int, C.c_int, C.c_float, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ic_last_error": (C.c_int, [C.c_char_p, C.c_int]),
    "es_last_error": (C.c_int, [C.c_char_p, C.c_int]),
    "es_version": (C.c_int, []),
}

_lock = threading.Lock()
_lib = None


def exported_symbols() -> list:
    return sorted(_PROTOS)


def load(path: Path | None = None):
    """Load libes_engine.so and declare its prototypes (idempotent)."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path is not None else LIB_PATH
        if not p.exists():
            raise EngineUnavailable(f"{p} is not built; run __graft_entry__.build() (nvcc, sm_103a)")
        try:
            lib = C.CDLL(str(p))
        except OSError as e:
            raise EngineUnavailable(f"cannot load {p}: {e}") from e
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


def last_error(lib=None) -> str:
    lib = lib or load()
    buf = C.create_string_buffer(1024)
    lib.es_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(fn: str, code: int, lib=None):
    if code != ES_OK:
        if fn[:3] in ("sg_", "pf_", "ic_"):
            lib = lib or load()
            buf = C.create_string_buffer(1024)
            {"sg_": lib.sg_last_error, "pf_": lib.pf_last_error, "ic_": lib.ic_last_error}[fn[:3]](buf, len(buf))
            raise EngineError(fn, code, buf.value.decode(errors="replace"))
        if fn.startswith("es_batch"):
            lib = lib or load()
            buf = C.create_string_buffer(1024)
            lib.es_batch_last_error(buf, len(buf))
            raise EngineError(fn, code, buf.value.decode(errors="replace"))
        raise EngineError(fn, code, last_error(lib))
