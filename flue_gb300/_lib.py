"""ctypes binding of ``libflue_gb300.so`` (the C ABI of include/flue_gb300.h).

The library must have been built (``flue_gb300.build.build()``); loading
fails loudly otherwise -- there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

FLUE_OK = 0
FLUE_ERR_ARG = 1
FLUE_ERR_SHAPE = 2
FLUE_ERR_DTYPE = 3
FLUE_ERR_LAYOUT = 4
FLUE_ERR_CUDA = 5
FLUE_ERR_TIMEOUT = 6
FLUE_ERR_WORKSPACE = 7
FLUE_ERR_NOMEM = 8

C128, C64, R12 = 0, 1, 2
FORCE_LIE, FORCE_EUCLID = 0, 1
FMUNU_CLOVER, FMUNU_LOOP5 = 0, 1

OP_PLAQUETTE = 0
OP_POLYAKOV = 1
OP_WMUNU = 2
OP_FMUNU = 3
OP_MAGNETIC = 4
OP_MAGNETIC_FORCE = 5
OP_ENERGY_FORCE = 6
OP_PLAQUETTE_FORCE = 7
OP_MEANLINK = 8
OP_WFLOW = 9
OP_GLUON_PROP = 10


class FlueError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, fn: str, status: int, detail: str):
        self.status = status
        super().__init__(f"{fn} failed with status {status} ({_strerror(status)}): {detail}")


class FlueField(ctypes.Structure):
    _fields_ = [
        ("links", ctypes.c_void_p),
        ("nt", ctypes.c_int32),
        ("nx", ctypes.c_int32),
        ("ny", ctypes.c_int32),
        ("nz", ctypes.c_int32),
        ("prec", ctypes.c_int32),
    ]


_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_SZ = ctypes.c_size_t
_I64 = ctypes.c_int64
_FP = ctypes.POINTER(FlueField)

# name -> (argtypes, restype)
SIGNATURES = {
    "flue_strerror": ([_I], ctypes.c_char_p),
    "flue_last_error_detail": ([], ctypes.c_char_p),
    "flue_abi_version": ([], _I),
    "flue_stage_timing": ([_I], _I),
    "flue_kernel_launches": ([], ctypes.c_uint64),
    "flue_bounds_errors": ([], ctypes.c_int64),
    "flue_stage_times": ([_P, _I, _P], _I),
    "flue_field_bytes": ([_I, _I, _I, _I, _I], _I64),
    "flue_workspace_bytes": ([_I, _I, _I, _I, _I, _I], _SZ),
    "flue_pack_field": ([_P, _I, _P, _I, _I, _I, _I, _P, _I, _I, _P], _I),
    "flue_unpack_field": ([_FP, _P, _I, _P], _I),
    "flue_reunitarise_field": ([_FP, _P], _I),
    "flue_multiplymatmat_batch": ([_P, _P, _P, _I64, _I, _I, _P], _I),
    "flue_plaquette": ([_FP, _I, _I, _I, _P, _P, _SZ, _P], _I),
    "flue_plaquette_noalloc": ([_FP, _I, _I, _I, _P, _P], _I),
    "flue_polyakov": ([_FP, _P, _P, _SZ, _P], _I),
    "flue_wmunu": ([_FP, _I, _I, _I, _I, _I, _P, _P, _SZ, _P], _I),
    "flue_genericpath": ([_FP, _P, _P, _I, _P, _P], _I),
    "flue_fmunu": ([_FP, _I, _I, _I, _P, _P, _SZ, _P], _I),
    "flue_magnetic": ([_FP, _P, _P, _SZ, _P], _I),
    "flue_magnetic_force": ([_FP, _P, _P, _I, _P, _SZ, _P], _I),
    "flue_loop5_energy_force": ([_FP, _P, _I, _P, _P, _I, _P, _SZ, _P], _I),
    "flue_plaquette_force": ([_FP, _P, _P, _I, _P, _SZ, _P], _I),
    "flue_meanlink": ([_FP, _P, _I, _P, _P, _SZ, _P], _I),
    "flue_wflow_step": ([_FP, _D, _P, _SZ, _P], _I),
    "flue_gauge_transform": ([_FP, _P, _I, _P], _I),
    "flue_wmunu_table_bytes": ([_I, _I, _I, _I, _I, _I, _I], _SZ),
    "flue_wmunu_table": ([_FP, _I, _I, _I, _I, _P, _P, _SZ, _P], _I),
    "flue_gluon_propagator": ([_FP, _D, _I, _P, _P, _SZ, _P], _I),
    "flue_plaquette_c": ([_P, _I, _I, _I, _I, _I, _I, _I, _P, _P, _P], _I),
    "flue_genplaquette_c": ([_P, _I, _I, _I, _I, _I, _I, _I, _P, _P, _P], _I),
    "flue_polyakov_c": ([_P, _I, _I, _I, _I, _P, _P, _P], _I),
    "flue_genericpath_c": ([_P, _I, _I, _I, _I, _P, _P, _I, _P], _I),
    "flue_wmunu_c": ([_P, _I, _I, _I, _I, _I, _I, _I, _I, _P], _I),
    "flue_wmunutau_c": ([_P, _I, _I, _I, _I, _I, _I, _I, _I, _I, _P], _I),
    "flue_cloverloopmunucoord_c": ([_P, _I, _I, _I, _I, _I, _I, _P], _I),
    "flue_loop5munucoord_c": ([_P, _I, _I, _I, _I, _I, _I, _P], _I),
    "flue_magnetic_c": ([_P, _I, _I, _I, _I, _P], _I),
    "flue_multiplymatmat_c": ([_P, _P, _P], _I),
    "flue_fixsu3matrix_c": ([_P], _I),
    "flue_uzerobar_c": ([_P, _I, _I, _I, _I, _P, _P], _I),
    "flue_scalargluonprop_c": ([_I, _I, _P, _D, _P], _I),
    "flue_magnetic_force_c": ([_P, _I, _I, _I, _I, _I, _I, _I, _P, _P], _I),
    "flue_release_host_cache": ([], None),
    "flue_ensemble_create": ([_P, _FP, _I, _I, _I, _I, _I], _I),
    "flue_ensemble_items": ([_P], _I),
    "flue_ensemble_run": ([_P, _P, _P], _I),
    "flue_ensemble_capture": ([_P, _P], _I),
    "flue_ensemble_replay": ([_P, _P], _I),
    "flue_ensemble_destroy": ([_P], _I),
}

_lock = threading.Lock()
_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the CUDA library (building it first if needed)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_build.LIB) or not _build.up_to_date():
                if not build_if_missing:
                    raise ImportError(f"flue_gb300 CUDA library missing: {_build.LIB}; run flue_gb300.build.build()")
                _build.build()
            L = ctypes.CDLL(_build.LIB)
            for name, (args, res) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.argtypes = args
                fn.restype = res
            _lib = L
    return _lib


def _strerror(status: int) -> str:
    try:
        return load().flue_strerror(status).decode()
    except Exception:  # pragma: no cover - used while formatting an error
        return "?"


def call(name: str, *args) -> int:
    """Call a C-ABI function and raise FlueError on a non-zero status."""
    L = load()
    rc = getattr(L, name)(*args)
    if rc != FLUE_OK:
        detail = L.flue_last_error_detail().decode(errors="replace")
        if rc in (FLUE_ERR_ARG, FLUE_ERR_SHAPE):
            raise ValueError(f"{name}: {_strerror(rc)}: {detail}")
        if rc in (FLUE_ERR_DTYPE, FLUE_ERR_LAYOUT):
            raise TypeError(f"{name}: {_strerror(rc)}: {detail}")
        raise FlueError(name, rc, detail)
    return rc


def exported_symbols():
    return sorted(SIGNATURES)
