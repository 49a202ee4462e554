"""ctypes binding of ``libgiao_gb300.so`` (the C ABI of include/giao_gb300.h).

There is no CPU fallback: every compute entry point runs on the GPU through
this library, and a missing library or device raises immediately.  Host-only
entry points (shell normalisation) work without a GPU.
"""

from __future__ import annotations

import ctypes
import threading
from pathlib import Path

import numpy as np

from .build import LIB

_d = ctypes.POINTER(ctypes.c_double)
_i = ctypes.POINTER(ctypes.c_int)
_i64 = ctypes.POINTER(ctypes.c_int64)
_u32 = ctypes.POINTER(ctypes.c_uint32)
_vp = ctypes.c_void_p


class BoysNumericalError(RuntimeError):
    """Complex Boys evaluation outside the verified domain (giao::BoysNumericalError)."""


class GxStats(ctypes.Structure):
    _fields_ = [
        ("requested", ctypes.c_int64),
        ("computed", ctypes.c_int64),
        ("screened", ctypes.c_int64),
        ("primitive_quartets", ctypes.c_int64),
        ("fp32_primitive_quartets", ctypes.c_int64),
        ("skipped_primitive_quartets", ctypes.c_int64),
        ("kernel_ms", ctypes.c_double),
        ("prepare_ms", ctypes.c_double),
        ("copy_ms", ctypes.c_double),
        ("call_ms", ctypes.c_double),
    ]


class GxQuartetBlock(ctypes.Structure):
    _fields_ = [
        ("shells", ctypes.c_uint32 * 4),
        ("shape", ctypes.c_int64 * 4),
        ("values", ctypes.POINTER(ctypes.c_double)),
        ("count", ctypes.c_int64),
    ]


# int (*gx_quartet_consumer)(const gx_quartet_block*, void*)
QUARTET_CONSUMER = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(GxQuartetBlock), ctypes.c_void_p)


class GxCholeskyOptions(ctypes.Structure):
    _fields_ = [
        ("threshold", ctypes.c_double),
        ("screening_threshold", ctypes.c_double),
        ("max_rank", ctypes.c_int64),
        ("pivot_batch_size", ctypes.c_int),
    ]


class GxCholeskyStats(ctypes.Structure):
    _fields_ = [
        ("rank", ctypes.c_int64),
        ("block_evaluations", ctypes.c_int64),
        ("column_entries", ctypes.c_int64),
        ("column_primitive_quartets", ctypes.c_int64),
        ("diagonal_primitive_quartets", ctypes.c_int64),
        ("column_cache_capacity", ctypes.c_int64),
        ("chained_steps", ctypes.c_int64),
        ("column_model_flops", ctypes.c_double),
        ("column_ms", ctypes.c_double),
        ("update_ms", ctypes.c_double),
        ("update_bytes", ctypes.c_double),
        ("update_flops", ctypes.c_double),
        ("column_pool_bytes", ctypes.c_double),
        ("seconds", ctypes.c_double),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class GxClassProfile(ctypes.Structure):
    _fields_ = [
        ("la", ctypes.c_int), ("lb", ctypes.c_int), ("lc", ctypes.c_int), ("ld", ctypes.c_int),
        ("tasks", ctypes.c_int64),
        ("primitive_quartets", ctypes.c_int64),
        ("fp64_quartets", ctypes.c_int64),
        ("fp32_quartets", ctypes.c_int64),
        ("model_flops_per_quartet", ctypes.c_double),
        ("ms", ctypes.c_float),
        ("per_group", ctypes.c_int),
        ("warps_per_block", ctypes.c_int),
        ("batch", ctypes.c_int),
        ("groups", ctypes.c_int64),
        ("kt", ctypes.c_int),
        ("ct", ctypes.c_int),
        ("min_blocks", ctypes.c_int),
        ("stream", ctypes.c_int),
    ]


class GxClassConfig(ctypes.Structure):
    _fields_ = [(name, ctypes.c_int) for name in ("per_group", "warps_per_block", "batch", "kt", "ct", "min_blocks",
                                                   "nostage", "stream", "nolane")]


# name -> (restype, argtypes); every symbol of include/giao_gb300.h
SIGNATURES = {
    "gx_context_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_vp)]),
    "gx_context_destroy": (None, [_vp]),
    "gx_last_error": (ctypes.c_char_p, []),
    "gx_version": (ctypes.c_char_p, []),
    "gx_primitive_normalization": (ctypes.c_double, [ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "gx_shell_normalize": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _d, _d, ctypes.c_int, _d]),
    "gx_basis_create": (ctypes.c_int, [_vp, ctypes.c_int, _d, _i, _i, _i, _d, _d, _i, ctypes.POINTER(_vp)]),
    "gx_basis_destroy": (None, [_vp]),
    "gx_basis_ao_count": (ctypes.c_int64, [_vp]),
    "gx_boys": (ctypes.c_int, [_vp, _d, ctypes.c_int64, ctypes.c_int, ctypes.c_int, _d, _i]),
    "gx_primitive_eri": (ctypes.c_int, [_vp, _d, _d, _i, _d, _i, _d, _d, _d]),
    "gx_eri_batch": (ctypes.c_int, [_vp, _vp, _d, _d, _u32, ctypes.c_int64, ctypes.c_int, ctypes.c_double,
                                    ctypes.c_double, _u32, _i64, _d, ctypes.c_int64, ctypes.POINTER(GxStats)]),
    "gx_eri_batch_device": (ctypes.c_int, [_vp, _vp, _d, _d, _u32, ctypes.c_int64, ctypes.c_int, ctypes.c_double,
                                           ctypes.c_double, _u32, _i64, _vp, ctypes.c_int64,
                                           ctypes.POINTER(GxStats)]),
    "gx_eri_for_each": (ctypes.c_int, [_vp, _vp, _d, _d, _u32, ctypes.c_int64, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_double, QUARTET_CONSUMER, _vp, ctypes.POINTER(GxStats)]),
    "gx_eri_center_derivatives": (ctypes.c_int, [_vp, _vp, _d, _d, _u32, ctypes.c_int64, _i64, _d, ctypes.c_int64,
                                                 ctypes.POINTER(ctypes.c_float)]),
    "gx_eri_center_derivatives_device": (ctypes.c_int, [_vp, _vp, _d, _d, _u32, ctypes.c_int64, _i64, _vp,
                                                        ctypes.c_int64, ctypes.POINTER(ctypes.c_float)]),
    "gx_eri_magnetic_derivatives": (ctypes.c_int, [_vp, _vp, _d, _d, _u32, ctypes.c_int64, _i64, _d,
                                                   ctypes.c_int64, ctypes.POINTER(ctypes.c_float)]),
    "gx_eri_mixed_derivatives": (ctypes.c_int, [_vp, _vp, _d, _d, _u32, ctypes.c_int64, _i64, _d, ctypes.c_int64]),
    "gx_eri_derivative_contraction": (ctypes.c_int, [_vp, _vp, _d, _d, _u32, ctypes.c_int64, _i64, ctypes.c_int,
                                                     ctypes.c_int, _d, ctypes.c_int, _d, _d, ctypes.c_int,
                                                     ctypes.c_int64, _d]),
    "gx_eri_derivative_schwarz": (ctypes.c_int, [_vp, _vp, _d, _d, _d, _d]),
    "gx_eri_plan_get_config": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(GxClassConfig)]),
    "gx_eri_plan_set_config": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(GxClassConfig)]),
    "gx_eri_shell": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _d, _d, _d]),
    "gx_eri_full": (ctypes.c_int, [_vp, _vp, _d, _d, ctypes.c_int, ctypes.c_double, ctypes.c_double, _d]),
    "gx_schwarz": (ctypes.c_int, [_vp, _vp, _d, _d, _d]),
    "gx_nuclear_attraction": (ctypes.c_int, [_vp, _vp, _d, _d, ctypes.c_int, _d, _d, _d]),
    "gx_cholesky_diagonal": (ctypes.c_int, [_vp, _vp, _i64, ctypes.c_int64, _d, _d, _d]),
    "gx_cholesky_columns": (ctypes.c_int, [_vp, _vp, _i64, ctypes.c_int64, _d, _d, _d]),
    "gx_cholesky": (ctypes.c_int, [_vp, _vp, _d, _d, ctypes.POINTER(GxCholeskyOptions), _d, _i64, _i64, _d]),
    "gx_cholesky_factor": (ctypes.c_int, [_vp, _vp, _d, _d, ctypes.POINTER(GxCholeskyOptions), ctypes.POINTER(_vp)]),
    "gx_cholesky_factors_info": (ctypes.c_int, [_vp, _i64, _i64, _d, _i]),
    "gx_cholesky_factors_copy": (ctypes.c_int, [_vp, _d, _i64]),
    "gx_cholesky_factors_device": (_vp, [_vp]),
    "gx_cholesky_factors_stats": (ctypes.c_int, [_vp, ctypes.POINTER(GxCholeskyStats)]),
    "gx_cholesky_factors_destroy": (None, [_vp]),
    "gx_cholesky_last_stats": (ctypes.c_int, [_vp, ctypes.POINTER(GxCholeskyStats)]),
    "gx_eri_batch_packed": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(_vp), _d, _d, ctypes.POINTER(_u32), _i64,
                                           ctypes.c_int, ctypes.c_double, ctypes.POINTER(_i64), ctypes.POINTER(_d),
                                           _i64, _d]),
    "gx_context_set_stable_launch": (ctypes.c_int, [_vp, ctypes.c_int]),
    "gx_context_set_copy_parts": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double]),
    "gx_context_set_stream": (ctypes.c_int, [_vp, _vp]),
    "gx_context_synchronize": (ctypes.c_int, [_vp]),
    "gx_eri_plan_create": (ctypes.c_int, [_vp, _vp, _u32, ctypes.c_int64, _i64, ctypes.POINTER(_vp)]),
    "gx_eri_plan_info": (ctypes.c_int, [_vp, _i64, _i64, _d, _i]),
    "gx_eri_plan_execute": (ctypes.c_int, [_vp, _d, _d, ctypes.c_int, ctypes.c_double, _vp]),
    "gx_eri_plan_destroy": (None, [_vp]),
    "gx_eri_plan_counts": (ctypes.c_int, [_vp, _i64, _i64, _d, _d]),
    "gx_eri_plan_class_count": (ctypes.c_int, [_vp]),
    "gx_eri_plan_graph_replays": (ctypes.c_int, [_vp]),
    "gx_eri_plan_profile": (ctypes.c_int, [_vp, _d, _d, ctypes.c_int, ctypes.c_double, _vp,
                                           ctypes.POINTER(GxClassProfile)]),
    "gx_eri_plan_autotune": (ctypes.c_int, [_vp, _d, _d, ctypes.c_int, ctypes.c_double, _vp, ctypes.c_int, _d, _d]),
    "gx_measure_fp64_peak": (ctypes.c_int, [_vp, _d]),
    "gx_measure_fp32_peak": (ctypes.c_int, [_vp, _d]),
    "gx_canonical_quartets": (ctypes.c_int64, [ctypes.c_int, _u32]),
    "gx_cholesky_step_noalloc": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int64, _vp, ctypes.c_int, ctypes.c_int,
                                                _vp, _vp, _vp, _vp]),
}

_lib: ctypes.CDLL | None = None
_lock = threading.RLock()


def library_path() -> Path:
    return LIB


def lib() -> ctypes.CDLL:
    """Load the library (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIB.exists():
                from .build import build

                build()
            handle = ctypes.CDLL(str(LIB))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
    return _lib


def last_error() -> str:
    msg = lib().gx_last_error()
    return msg.decode() if msg else ""


def check(rc: int) -> None:
    """Raise the reference's exception type for a gx_status code."""
    if rc == 0:
        return
    msg = last_error()
    if rc in (-1, -3):
        raise ValueError(msg)
    if rc == -2:
        raise IndexError(msg)
    if rc == -4:
        raise BoysNumericalError(msg)
    if rc == -6:
        raise MemoryError(msg)
    raise RuntimeError(msg)


class Context:
    """One CUDA device with its Boys table and pools (gx_context)."""

    def __init__(self, device: int = 0):
        handle = _vp()
        check(lib().gx_context_create(device, ctypes.byref(handle)))
        self.handle = handle
        self.device = device

    def close(self) -> None:
        """Release the device context.  Bases uploaded to it must not be used
        afterwards; contexts that are still referenced at interpreter exit are
        left to the process teardown (no destructor runs then)."""
        if getattr(self, "handle", None):
            lib().gx_context_destroy(self.handle)
            self.handle = None


_default: Context | None = None


def default_context() -> Context:
    """The process-wide context on CUDA device 0 (created on first use)."""
    global _default
    if _default is None:
        with _lock:
            if _default is None:
                _default = Context(0)
    return _default


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_d)


def iptr(a: np.ndarray):
    return a.ctypes.data_as(_i)


def i64ptr(a: np.ndarray):
    return a.ctypes.data_as(_i64)


def u32ptr(a: np.ndarray):
    return a.ctypes.data_as(_u32)
