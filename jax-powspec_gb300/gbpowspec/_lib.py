"""ctypes binding of libgbpowspec.so (the C ABI declared in include/gbpowspec.h).

There is no CPU fallback: if the library is missing every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import _build

GBP_OK = 0
GBP_ERR_INVALID = -1
GBP_ERR_CUDA = -2
GBP_ERR_CUFFT = -3
GBP_ERR_WORKSPACE = -4
GBP_ERR_UNSUPPORTED = -5
GBP_ERR_ALLOC = -6

MAS = {"ngp": 1, "cic": 2, "tsc": 3, "pcs": 4}
COMPAT_NONE, COMPAT_VEC, COMPAT_SCAN = 0, 1, 2
ELL0, ELL2, ELL4, KSUM = 1, 2, 4, 8


class GbpError(RuntimeError):
    """A libgbpowspec call returned a non-zero status."""

    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: {strerror(status)} (status {status})")


class DepositStats(C.Structure):
    """Mirror of gbp_deposit_stats."""

    _fields_ = [
        ("mass", C.c_double * 2),
        ("sum_w", C.c_double),
        ("sum_w2", C.c_double),
        ("n_kept", C.c_longlong),
        ("n_nonfinite", C.c_longlong),
        ("scale_exp", C.c_int),
        ("flags", C.c_int),
    ]


STATS_BYTES = C.sizeof(DepositStats)
STATS_REFILLED = 1          # gbp_deposit_stats.flags: the buckets outgrew their one-pass capacity
STATS_RESULT_BYTES = DepositStats.flags.offset   # the statistics proper (flags say how they were computed)


class Job(C.Structure):
    """Mirror of gbp_job (a mock described in device memory)."""

    _fields_ = [
        ("x", C.c_void_p),
        ("y", C.c_void_p),
        ("z", C.c_void_p),
        ("w", C.c_void_p),
        ("n", C.c_longlong),
        ("inv_cell", C.c_float),
        ("xmin", C.c_float),
        ("ymin", C.c_float),
        ("zmin", C.c_float),
        ("box_size", C.c_double),
    ]


JOB_BYTES = C.sizeof(Job)
LANE_GRAPH = 1


def lane_tiles_flag(tx: int, ty: int) -> int:
    """GBP_LANE_TILES(tx, ty): the column tile a lane's fused calls use (0, 0: the default)."""
    return ((int(tx) & 15) << 8) | ((int(ty) & 15) << 12)


class TraceRecord(C.Structure):
    """Mirror of gbp_trace_record."""

    _fields_ = [("kernel", C.c_char_p), ("ms", C.c_float)]


class LaneOut(C.Structure):
    """Mirror of gbp_lane_out (device pointers of the per-job output arrays)."""

    _fields_ = [("pk", C.c_void_p), ("kmean", C.c_void_p), ("nmodes", C.c_void_p), ("stats", C.c_void_p)]

_vp, _i, _i64, _f, _d, _sz = C.c_void_p, C.c_int, C.c_int64, C.c_float, C.c_double, C.c_size_t

# (name, restype, argtypes) for every exported entry point
SIGNATURES = [
    ("gbp_strerror", C.c_char_p, [_i]),
    ("gbp_version", _i, []),
    ("gbp_deposit_workspace_size", _i, [_i64, _i, _i, _i, _i, C.POINTER(_sz)]),
    ("gbp_deposit", _i, [_vp, _vp, _vp, _vp, _i64, _f, _f, _f, _f, _i, _i, _i, _i, _i,
                         _vp, _vp, _vp, _vp, _sz, _vp]),
    ("gbp_fft_plan_create", _i, [_i, _i, C.POINTER(_vp), C.POINTER(_sz)]),
    ("gbp_fft_plan_pitch", _i, [_vp, C.POINTER(_i)]),
    ("gbp_fft_plan_destroy", _i, [_vp]),
    ("gbp_fft_r2c", _i, [_vp, _vp, _vp, _vp, _sz, _vp]),
    ("gbp_bin_thresholds", _i, [_vp, _i, _i, _vp, C.POINTER(C.c_int32), C.POINTER(_i)]),
    ("gbp_bins_create", _i, [_vp, _i, _i, C.POINTER(_vp)]),
    ("gbp_bins_destroy", _i, [_vp]),
    ("gbp_bins_info", _i, [_vp, C.POINTER(_i), C.POINTER(_i), C.POINTER(C.c_int32)]),
    ("gbp_power_workspace_size", _i, [_vp, _i, _i, _i, C.POINTER(_sz)]),
    ("gbp_power", _i, [_vp, _i, _i, _vp, _i, _i, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    ("gbp_power_normalize", _i, [_vp, _vp, _vp, _i, _i, _d, _vp, _vp, _i, _vp, _vp, _vp]),
    ("gbp_power_noalloc", _i, [_vp, _i, _i, _vp, _i, _i, _vp, _vp, _vp, _vp, _vp]),
    ("gbp_deposit_job", _i, [_vp, _i64, _i, _i, _i, _vp, _vp, _vp, _sz, _vp]),
    ("gbp_power_normalize_job", _i, [_vp, _vp, _vp, _i, _i, _vp, _vp, _vp, _i, _vp, _vp, _vp]),
    ("gbp_lane_bytes", _i, [_i, _i, _i, _i, _vp, _i64, C.POINTER(_sz)]),
    ("gbp_lane_create", _i, [_i, _i, _i, _i, _i, _vp, _i64, _i, C.POINTER(_vp)]),
    ("gbp_lane_info", _i, [_vp, C.POINTER(_sz), C.POINTER(_i), C.POINTER(_i)]),
    ("gbp_lane_destroy", _i, [_vp]),
    ("gbp_lane_run", _i, [_vp, _vp, _i, _i, _i, _vp, _vp]),
    ("gbp_batch_run", _i, [_vp, _i, _vp, _i, _vp, _vp]),
    ("gbp_fft_power_workspace_size", _i, [_vp, _vp, _i, C.POINTER(_sz)]),
    ("gbp_fft_power", _i, [_vp, _vp, _vp, _vp, _i, _i, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    ("gbp_particles_power_workspace_size", _i, [_i64, _vp, _vp, _i, _i, C.POINTER(_sz)]),
    ("gbp_column_tile_variants", _i, [_i, C.POINTER(_i), C.POINTER(_i), _i, C.POINTER(_i)]),
    ("gbp_fft_plan_set_tiles", _i, [_vp, _i, _i]),
    ("gbp_fft_plan_tiles", _i, [_vp, C.POINTER(_i), C.POINTER(_i)]),
    ("gbp_particles_power", _i, [_vp, _vp, _vp, _vp, _i64, _f, _f, _f, _f, _vp, _vp, _i, _i, _vp, _vp, _vp, _vp,
                                 _vp, _vp, _sz, _vp]),
    ("gbp_particles_power_job", _i, [_vp, _i64, _vp, _vp, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    ("gbp_lognormal_workspace_size", _i, [_i, C.POINTER(_sz)]),
    ("gbp_lognormal", _i, [_i, _d, _d, _d, _i64, C.c_ulonglong, _vp, _vp, _vp, _vp, _sz, _vp]),
    ("gbp_lognormal_field", _i, [_i, _d, _d, C.c_ulonglong, _vp, _vp, _vp, _sz, _vp]),
    ("gbp_philox4x32_10", _i, [_vp, _vp, _vp]),
    ("gbp_xi_workspace_size", _i, [_vp, _vp, C.POINTER(_sz)]),
    ("gbp_xi", _i, [_vp, _vp, _vp, _vp, _vp, _i, _i, _vp, _vp, _vp, _sz, _vp]),
    ("gbp_bispec_workspace_size", _i, [_vp, _vp, C.POINTER(_sz)]),
    ("gbp_bispec", _i, [_vp, _vp, _vp, _vp, _i, _vp, _i, _d, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    ("gbp_power_backward_workspace_size", _i, [_vp, C.POINTER(_sz)]),
    ("gbp_power_backward", _i, [_vp, _vp, _vp, _i, _vp, _vp, _vp, _d, _vp, _vp, _sz, _vp]),
    ("gbp_deposit_backward", _i, [_vp, _vp, _vp, _vp, _i64, _f, _f, _f, _f, _i, _i, _i, _vp, _vp, _vp, _vp, _vp,
                                  _vp]),
    ("gbp_trace_enable", _i, [_i]),
    ("gbp_trace_collect", _i, [_vp, _i, C.POINTER(_i)]),
]

_lock = threading.Lock()
_LIB: C.CDLL | None = None


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load (building first if needed and allowed) and declare the library."""
    global _LIB
    with _lock:
        if _LIB is not None:
            return _LIB
        path = lib_path()
        if not os.path.exists(path) or not _build.up_to_date():
            if not build_if_missing:
                raise RuntimeError(f"{path} is missing: build it with `python -m gbpowspec._build`")
            _build.build()
        lib = C.CDLL(path)
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
        return lib


def strerror(status: int) -> str:
    try:
        return load().gbp_strerror(status).decode()
    except Exception:  # pragma: no cover - only when the library itself is unusable
        return "unknown"


def check(status: int, what: str) -> None:
    if status != GBP_OK:
        raise GbpError(status, what)
