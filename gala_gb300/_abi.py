"""ctypes mirror of ``include/gala_gb300.h`` and the loader of the CUDA library.

The product path calls the CUDA library only.  If the library is missing or
cannot be loaded, every call raises: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path

from . import _build

GX_MAX_COMPONENTS = 16
GX_MAX_INLINE_PARAMS = 128
GX_NOALLOC_MAX_ORBITS = 262144
GX_BATCH_QUEUE_WORDS = 1026

GX_OK = 0
GX_ERR_INVALID_ARGUMENT = -1
GX_ERR_UNSUPPORTED = -2
GX_ERR_CUDA = -3
GX_ERR_CAPACITY = -4
GX_ERR_KERNEL_STATUS = -5

GX_POT_NULL = 0
GX_POT_KEPLER = 1
GX_POT_HERNQUIST = 2
GX_POT_PLUMMER = 3
GX_POT_MIYAMOTONAGAI = 4
GX_POT_SPHERICALNFW = 5
GX_POT_FLATTENEDNFW = 6
GX_POT_TRIAXIALNFW = 7
GX_POT_SCF = 8

GX_FRAME_STATIC = 0
GX_FRAME_CONSTANT_ROTATING = 1


class gx_component(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("n_params", C.c_int32),
        ("param_offset", C.c_int64),
        ("do_shift_rotate", C.c_int32),
        ("reserved", C.c_int32),
        ("q0", C.c_double * 3),
        ("R", C.c_double * 9),
    ]


class gx_potential(C.Structure):
    _fields_ = [
        ("n_components", C.c_int32),
        ("n_dim", C.c_int32),
        ("components", C.POINTER(gx_component)),
        ("params", C.POINTER(C.c_double)),
        ("params_device", C.c_void_p),
        ("n_params_total", C.c_int64),
        ("table_device", C.c_void_p),
    ]


class gx_frame(C.Structure):
    _fields_ = [("type", C.c_int32), ("reserved", C.c_int32), ("params", C.c_double * 3)]


class gx_body(C.Structure):
    _fields_ = [("type", C.c_int32), ("n_params", C.c_int32), ("params", C.c_double * 7)]


_P = C.c_void_p
_I64 = C.c_int64
_I32 = C.c_int32
_D = C.c_double
_PP = C.POINTER(gx_potential)
_PF = C.POINTER(gx_frame)

SIGNATURES = {
    "gx_abi_version": (C.c_int, []),
    "gx_component_table_bytes": (C.c_int64, [C.c_int32]),
    "gx_pack_component_table": (C.c_int, [_PP, _P, _I64]),
    "gx_last_error_message": (C.c_char_p, []),
    "gx_cancel_flag_create": (C.c_int, [_P, _P]),
    "gx_set_cancel_flag": (None, [_P]),
    "gx_cancel_flag_destroy": (C.c_int, [_P]),
    "gx_debug_enabled": (C.c_int, []),
    "gx_debug_read": (C.c_int, [_P, _I32]),
    "gx_potential_value": (C.c_int, [_PP, _D, _P, _I64, _P, _P]),
    "gx_potential_gradient": (C.c_int, [_PP, _D, _P, _I64, _P, _P]),
    "gx_potential_density": (C.c_int, [_PP, _D, _P, _I64, _P, _P]),
    "gx_hamiltonian_value": (C.c_int, [_PP, _PF, _D, _P, _I64, _P, _P]),
    "gx_hamiltonian_gradient": (C.c_int, [_PP, _PF, _D, _P, _I64, _P, _P]),
    "gx_leapfrog_integrate_hamiltonian": (C.c_int, [_PP, _PF, _P, _I64, _P, _I64, _I32, _P, _P]),
    "gx_ruth4_integrate_hamiltonian": (C.c_int, [_PP, _PF, _P, _I64, _P, _I64, _I32, _P, _P]),
    "gx_calibrate_fma": (C.c_int, [_I32, _I32, _I32, _I64, _P, _P]),
    "gx_selfcheck_fast64": (C.c_int, [_P, _I64, _P, _P]),
    "gx_batch_integrate_fp32": (C.c_int, [_PP, _P, _I64, _P, _P, _P, _P, _I64, _I32, _I32, _I32, _P, _P, _P]),
    "gx_batch_integrate_fp32_state": (C.c_int, [_PP, _P, _I64, _P, _P, _P, _P, _I64, _I32, _I32, _I32, _P, _P, _P, _P,
                                                _P]),
    "gx_batch_integrate_fp32_noalloc": (C.c_int, [_PP, _P, _I64, _P, _P, _P, _I32, _I32, _P, _P]),
    "gx_mlp_param_count": (C.c_int64, []),
    "gx_mlp_train_workspace_floats": (C.c_int64, [_I64]),
    "gx_mlp_forward": (C.c_int, [_P, _P, _I64, _P, _P, _P, _P]),
    "gx_mlp_train_step": (C.c_int, [_P, _P, _P, _P, _P, _P, _I64, C.c_float, C.c_float, _P, _P, _P]),
    "gx_mlp_adam": (C.c_int, [_P, _P, _P, _P, _I64, C.c_float, C.c_float, C.c_float, C.c_float, _I64, _P]),
    "gx_surrogate_gradient": (C.c_int, [_P, _P, _P, _D, _D, _D, _D, _I32, _P, _I64, _P, _P, _I32, _P]),
    "gx_surrogate_leapfrog": (C.c_int, [_P, _P, _P, _D, _D, _D, _D, _I32, _I32, _P, _I64, _I64, _D, _P, _P, _I32,
                                        _P]),
    "gx_surrogate_smem_bytes": (C.c_int, []),
    "gx_surrogate_gradient_tc": (C.c_int, [_P, _P, _P, _D, _D, _D, _D, _I32, _P, _I64, _P, _P, _I32, _P, _P]),
    "gx_surrogate_leapfrog_tc": (C.c_int, [_P, _P, _P, _D, _D, _D, _D, _I32, _P, _I64, _I64, _D, _P, _P, _I32, _P,
                                           _P]),
    "gx_surrogate_tc_smem_bytes": (C.c_int, []),
    "gx_nbody_dop853": (C.c_int, [_PP, _PF, _I64, _I32, _I32, _P, _P, _P, _I64, _D, _D, _I64, _D, _I64, _I32, _I64,
                                  _P, _P, _P, _P, _P]),
    "gx_mockstream_dop853": (C.c_int, [_PP, _PF, _I64, _I32, _P, _P, _I64, _P, _P, _I32, _P, _I64, _D, _D, _D, _D,
                                       _I64, _P, _P, _P, _P, _P, _P]),
    "gx_mockstream_dop853_fp32": (C.c_int, [_PP, _I64, _I32, _P, _P, _I64, _P, _P, _I32, _P, _I64, _D, _D, _D, _D,
                                            _I64, _P, _P, _P, _P, _P, _P]),
    "gx_mockstream_wide_scratch_bytes": (C.c_int64, [_I64, _I32]),
    "gx_mockstream_dop853_wide": (C.c_int, [_PP, _PF, _I64, _I32, _P, _P, _I64, _P, _P, _P, _I64, _D, _D, _D, _D,
                                            _I64, _P, _I64, _I32, _P, _I64, _P, _P, _P, _P, _P]),
    "gx_nbody_wide_scratch_bytes": (C.c_int64, [_I64, _I32]),
    "gx_nbody_dop853_wide": (C.c_int, [_PP, _PF, _I64, _I32, _I32, _P, _P, _P, _I64, _D, _D, _I64, _D, _I64, _I32,
                                       _I64, _P, _I64, _P, _P, _P, _P]),
    "gx_mockstream_animate_snapshots": (C.c_int64, [_I64, _I64]),
    "gx_mockstream_dop853_animate": (C.c_int, [_PP, _PF, _I64, _I32, _P, _P, _I64, _P, _D, _P, _P, _I64, _I64, _D,
                                               _D, _I64, _P, _I64, _P, _P, _P, _P, _P]),
    "gx_mockstream_dop853_animate_fp32": (C.c_int, [_PP, _I64, _I32, _P, _P, _I64, _P, _D, _P, _P, _I64, _I64, _D,
                                                    _D, _I64, _P, _I64, _P, _P, _P, _P, _P]),
    "gx_nbody_leapfrog": (C.c_int, [_PP, _I64, _I32, _I32, _P, _P, _P, _I64, _I32, _P, _P]),
    "gx_mockstream_leapfrog": (C.c_int, [_PP, _I64, _I32, _P, _P, _I64, _P, _P, _I32, _P, _I64, _D, _D, _P, _P, _P,
                                         _P]),
    "gx_mockstream_leapfrog_fp32": (C.c_int, [_PP, _I64, _I32, _P, _P, _I64, _P, _P, _I32, _P, _I64, _D, _D, _P, _P,
                                              _P, _P]),
    "gx_orbit_extrema": (C.c_int, [_P, _P, _I64, _I64, _I32, _I32, _P, _P, _P, _P, _P, _P, _P]),
    "gx_fardal_sample": (C.c_int, [_PP, _I64, _I64, _P, _I64, _P, _P, _P, _I64, _P, _D, _I32, _I32, _I32, _P, _P]),
    "gx_stream_sample": (C.c_int, [_PP, _I64, _I64, _P, _I64, _P, _P, _P, _I64, _I32, _P, _D, _I32, _I32, _I32, _P,
                                   _P]),
    "gx_batch_integrate_fp64": (C.c_int, [_PP, _P, _I64, _P, _P, _P, _P, _I64, _I32, _I32, _I32, _P, _P, _P]),
    "gx_batch_schedule_slots": (C.c_int64, [_I64, _I32]),
    "gx_batch_schedule_work_words": (C.c_int64, [_I64, _I32]),
    "gx_batch_schedule": (C.c_int, [_P, _P, _I64, _I32, _P, _I64, _P, _I64, _P]),
    "gx_dop853_integrate_hamiltonian": (
        C.c_int,
        [_PP, _PF, _P, _I64, _P, _I64, _D, _D, _I64, _D, _I64, _I32, _I32, _I64, _P, _P, _P, _P],
    ),
    "gx_fixed_fp32": (C.c_int, [_PP, _I32, _P, _I64, _P, _I64, _I32, _I64, _P, _P]),
    "gx_dop853_fp32": (C.c_int, [_PP, _PF, _P, _I64, _P, _I64, _D, _D, _I64, _D, _I64, _I32, _I64, _P, _P, _P, _P,
                                 _P, _P]),
}

_lib = None
_lib_debug = None
_lock = threading.Lock()


class GxError(RuntimeError):
    """A C-ABI call returned an error code."""

    def __init__(self, name, code, msg):
        super().__init__(f"{name} failed with code {code}: {msg}")
        self.code = code


def library_path() -> Path:
    return _build.LIB_DEBUG if _debug_requested() else _build.LIB


def _debug_requested() -> bool:
    """GALA_GB300_DEBUG=1 makes the debug library the process's library."""
    return os.environ.get("GALA_GB300_DEBUG", "") not in ("", "0")


def _bind(path: Path, debug: bool, build_if_missing: bool):
    if not path.exists() or _build._sources_newer(path):
        if not build_if_missing:
            raise RuntimeError(f"CUDA library not built: {path}")
        _build.build(debug=debug)
    lib = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.gx_abi_version() != 3:
        raise RuntimeError("gala_gb300 library ABI version mismatch")
    return lib


def load(build_if_missing: bool = True):
    """Load (building first if needed) the CUDA library and bind every symbol."""
    global _lib
    with _lock:
        if _lib is None:
            _lib = _bind(library_path(), _debug_requested(), build_if_missing)
        return _lib


def load_debug(build_if_missing: bool = True):
    """The debug library (libgala_gb300_debug.so: the same entry points with
    device-side check records, gx_debug_read), bound beside the release one."""
    global _lib_debug
    with _lock:
        if _lib_debug is None:
            _lib_debug = _bind(_build.LIB_DEBUG, True, build_if_missing)
        return _lib_debug


def call(name: str, *args) -> int:
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != GX_OK:
        msg = lib.gx_last_error_message().decode(errors="replace")
        if rc == GX_ERR_INVALID_ARGUMENT:
            raise ValueError(f"{name}: {msg}")
        if rc == GX_ERR_UNSUPPORTED:
            raise TypeError(f"{name}: {msg}")
        raise GxError(name, rc, msg)
    return rc
