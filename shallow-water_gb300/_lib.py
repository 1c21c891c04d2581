"""ctypes binding of the C ABI in include/swe_gb300.h (libswe_gb300.so, built in-tree).

Loading never falls back to anything: if the shared library is missing or does not
export the ABI, :func:`lib` raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libswe_gb300.so")

SWE_OK = 0
SWE_ERR_BAD_ARG = 1
SWE_ERR_CUDA = 2
SWE_ERR_NONFINITE = 3
SWE_ERR_CFL = 4
SWE_ERR_TIMEOUT = 5
SWE_ERR_NO_DEVICE = 6
SWE_ERR_UNSUPPORTED = 7
SWE_ERR_IO = 8

SWE_BC_REFLECTING = 0
SWE_BC_TRANSMISSIVE = 1
SWE_PRECISION_FP64 = 0
SWE_PRECISION_FP32_MIXED = 1
SWE_SCHEME_FUSED = 0
SWE_SCHEME_MODULAR = 1
RECONSTRUCTIONS = {"PiecewiseConst": 0, "MUSCL": 1}
RIEMANN_SOLVERS = {"HLL": 0, "Rusanov": 1, "ROE": 2}

# Every symbol include/swe_gb300.h declares.
EXPORTS = (
    "swe_params_default", "swe_create", "swe_destroy", "swe_upload", "swe_download",
    "swe_step", "swe_step_host", "swe_max_wave_speed", "swe_stable_dt", "swe_dt_log", "swe_last_error",
    "swe_status_string", "swe_kernel_launches", "swe_last_step_ms", "swe_totals",
    "swe_ens_create", "swe_ens_destroy", "swe_ens_upload", "swe_ens_download", "swe_ens_step",
    "swe_ens_times", "swe_ens_last_dt", "swe_ens_last_step_ms", "swe_ens_kernel_launches",
    "swe_ens_set_schedule", "swe_ens_get_schedule", "swe_ens_tune", "swe_ens_last_error",
    "swe_totals_noalloc", "swe_adjoint_gauge", "swe_selftest_soft_f64", "swe_stage",
    "swe_halo", "swe_sanity",
    "swe_snapshot_open", "swe_snapshot_bathymetry", "swe_snapshot_metadata",
    "swe_snapshot_write_host", "swe_snapshot_write", "swe_snapshot_flush",
    "swe_snapshot_records", "swe_snapshot_stats", "swe_snapshot_close", "swe_snapshot_destroy",
    "swe_snapshot_last_error", "swe_sanity_log_open", "swe_sanity_log_write",
    "swe_sanity_log_close", "swe_sanity_log_destroy", "swe_sanity_log_last_error",
    "swe_params_size", "swe_snapshot_params_size", "swe_selftest_wait_timeout",
    "swe_test_preset_timeout", "swe_ens_test_preset_timeout",
    "swe_slabs_create", "swe_slabs_destroy", "swe_slabs_upload", "swe_slabs_download",
    "swe_slabs_step", "swe_slabs_last_step_ms", "swe_slabs_kernel_launches",
    "swe_slabs_last_error",
)
TOTALS_NOALLOC_MAX_BLOCKS = 1024
ADJ_TAPE_ALL = -1  # n_snapshots value of swe_adjoint_gauge's tape mode
ADJ_SEGMENTS = -2  # n_snapshots value of its segmented schedule (snapshots every sqrt(n) steps)

SHAPES = {"8x32": 0, "8x16": 1, "4x64": 2, "16x32": 3, "8x64": 4, "cols": 5, "strip": 6}


class SweParams(ctypes.Structure):
    _fields_ = [
        ("Nx", ctypes.c_int),
        ("Ny", ctypes.c_int),
        ("nG", ctypes.c_int),
        ("Lx", ctypes.c_double),
        ("Ly", ctypes.c_double),
        ("g", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("bc", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("device", ctypes.c_int),
        ("x_halo_lo", ctypes.c_int),
        ("x_halo_hi", ctypes.c_int),
        ("reserved", ctypes.c_int),
        ("dx", ctypes.c_double),
        ("dy", ctypes.c_double),
        ("scheme", ctypes.c_int),
        ("reconstruction", ctypes.c_int),
        ("riemann", ctypes.c_int),
        ("bathymetry", ctypes.c_int),
    ]


class SnapshotParams(ctypes.Structure):
    _fields_ = [
        ("Nx", ctypes.c_int),
        ("Ny", ctypes.c_int),
        ("dx", ctypes.c_double),
        ("dy", ctypes.c_double),
        ("unit_x", ctypes.c_char_p),
        ("unit_y", ctypes.c_char_p),
        ("unit_h", ctypes.c_char_p),
        ("unit_time", ctypes.c_char_p),
        ("save_every", ctypes.c_int),
        ("format", ctypes.c_int),
    ]


_lib = None


def lib(path: str = LIB_PATH):
    """Loads libswe_gb300.so and declares the ABI; raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} not found: build it first (python shallow-water_gb300/build.py); "
            "there is no CPU fallback")
    L = ctypes.CDLL(path)
    dp = ctypes.POINTER(ctypes.c_double)
    vp = ctypes.c_void_p
    L.swe_params_size.argtypes = []
    L.swe_params_size.restype = ctypes.c_size_t
    L.swe_snapshot_params_size.argtypes = []
    L.swe_snapshot_params_size.restype = ctypes.c_size_t
    if (L.swe_params_size() != ctypes.sizeof(SweParams) or
            L.swe_snapshot_params_size() != ctypes.sizeof(SnapshotParams)):
        raise RuntimeError(f"{path}: struct layout differs from this binding (rebuild it)")
    L.swe_params_default.argtypes = [ctypes.POINTER(SweParams)]
    L.swe_params_default.restype = None
    L.swe_create.argtypes = [ctypes.POINTER(SweParams), ctypes.POINTER(vp)]
    L.swe_create.restype = ctypes.c_int
    L.swe_destroy.argtypes = [vp]
    L.swe_destroy.restype = None
    L.swe_upload.argtypes = [vp, dp, dp, dp, dp]
    L.swe_upload.restype = ctypes.c_int
    L.swe_download.argtypes = [vp, dp, dp, dp]
    L.swe_download.restype = ctypes.c_int
    L.swe_step.argtypes = [vp, ctypes.c_int, ctypes.c_double, dp]
    L.swe_step.restype = ctypes.c_int
    L.swe_step_host.argtypes = [vp, dp, dp, dp, dp, dp, dp, dp, ctypes.c_int, ctypes.c_double,
                                dp]
    L.swe_step_host.restype = ctypes.c_int
    L.swe_max_wave_speed.argtypes = [vp, dp]
    L.swe_max_wave_speed.restype = ctypes.c_int
    L.swe_stable_dt.argtypes = [vp, dp]
    L.swe_stable_dt.restype = ctypes.c_int
    L.swe_dt_log.argtypes = [vp, dp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.swe_dt_log.restype = ctypes.c_int
    L.swe_last_error.argtypes = [vp]
    L.swe_last_error.restype = ctypes.c_char_p
    L.swe_status_string.argtypes = [ctypes.c_int]
    L.swe_status_string.restype = ctypes.c_char_p
    L.swe_kernel_launches.argtypes = [vp]
    L.swe_kernel_launches.restype = ctypes.c_longlong
    L.swe_totals.argtypes = [vp, dp, dp, dp]
    L.swe_totals.restype = ctypes.c_int
    L.swe_last_step_ms.argtypes = [vp, dp]
    L.swe_last_step_ms.restype = ctypes.c_int
    ip = ctypes.POINTER(ctypes.c_int)
    L.swe_ens_create.argtypes = [ctypes.POINTER(SweParams), ctypes.c_int, ip, ip, dp, dp,
                                 ctypes.POINTER(vp)]
    L.swe_ens_create.restype = ctypes.c_int
    L.swe_ens_destroy.argtypes = [vp]
    L.swe_ens_destroy.restype = None
    L.swe_ens_upload.argtypes = [vp, ctypes.c_int, dp, dp, dp, dp]
    L.swe_ens_upload.restype = ctypes.c_int
    L.swe_ens_download.argtypes = [vp, ctypes.c_int, dp, dp, dp]
    L.swe_ens_download.restype = ctypes.c_int
    L.swe_ens_step.argtypes = [vp, ctypes.c_int, ctypes.c_double]
    L.swe_ens_step.restype = ctypes.c_int
    L.swe_ens_times.argtypes = [vp, dp]
    L.swe_ens_times.restype = ctypes.c_int
    L.swe_ens_last_dt.argtypes = [vp, dp]
    L.swe_ens_last_dt.restype = ctypes.c_int
    L.swe_ens_last_step_ms.argtypes = [vp, dp]
    L.swe_ens_last_step_ms.restype = ctypes.c_int
    L.swe_ens_kernel_launches.argtypes = [vp]
    L.swe_ens_kernel_launches.restype = ctypes.c_longlong
    L.swe_ens_set_schedule.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.swe_ens_set_schedule.restype = ctypes.c_int
    L.swe_ens_get_schedule.argtypes = [vp, ip, ip, ip]
    L.swe_ens_get_schedule.restype = ctypes.c_int
    L.swe_ens_tune.argtypes = [vp, ctypes.c_int, dp]
    L.swe_ens_tune.restype = ctypes.c_int
    L.swe_totals_noalloc.argtypes = [vp, vp, vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_longlong, ctypes.c_double, ctypes.c_int, vp, vp]
    L.swe_totals_noalloc.restype = ctypes.c_int
    L.swe_adjoint_gauge.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.c_int, ip, ip, dp,
                                    ctypes.c_int, dp, dp, dp, dp, dp, dp]
    L.swe_adjoint_gauge.restype = ctypes.c_int
    L.swe_sanity.argtypes = [vp, dp, dp, ctypes.POINTER(ctypes.c_longlong), dp]
    L.swe_sanity.restype = ctypes.c_int
    L.swe_stage.argtypes = [vp, ctypes.c_int, ctypes.c_double]
    L.swe_stage.restype = ctypes.c_int
    L.swe_halo.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp]
    L.swe_halo.restype = ctypes.c_int
    L.swe_selftest_soft_f64.argtypes = [ctypes.c_longlong, ctypes.c_ulonglong,
                                        ctypes.POINTER(ctypes.c_longlong)]
    L.swe_selftest_soft_f64.restype = ctypes.c_int
    L.swe_selftest_wait_timeout.argtypes = [ctypes.c_int, ctypes.c_double,
                                            ctypes.POINTER(ctypes.c_longlong), dp]
    L.swe_selftest_wait_timeout.restype = ctypes.c_int
    L.swe_test_preset_timeout.argtypes = [vp]
    L.swe_test_preset_timeout.restype = ctypes.c_int
    L.swe_ens_test_preset_timeout.argtypes = [vp]
    L.swe_ens_test_preset_timeout.restype = ctypes.c_int
    L.swe_ens_last_error.argtypes = [vp]
    L.swe_ens_last_error.restype = ctypes.c_char_p
    L.swe_slabs_create.argtypes = [ctypes.POINTER(SweParams), ctypes.c_int, ip,
                                   ctypes.POINTER(vp)]
    L.swe_slabs_create.restype = ctypes.c_int
    L.swe_slabs_destroy.argtypes = [vp]
    L.swe_slabs_destroy.restype = None
    L.swe_slabs_upload.argtypes = [vp, dp, dp, dp, dp]
    L.swe_slabs_upload.restype = ctypes.c_int
    L.swe_slabs_download.argtypes = [vp, dp, dp, dp]
    L.swe_slabs_download.restype = ctypes.c_int
    L.swe_slabs_step.argtypes = [vp, ctypes.c_int, ctypes.c_double, dp]
    L.swe_slabs_step.restype = ctypes.c_int
    L.swe_slabs_last_step_ms.argtypes = [vp, dp]
    L.swe_slabs_last_step_ms.restype = ctypes.c_int
    L.swe_slabs_kernel_launches.argtypes = [vp]
    L.swe_slabs_kernel_launches.restype = ctypes.c_longlong
    L.swe_slabs_last_error.argtypes = [vp]
    L.swe_slabs_last_error.restype = ctypes.c_char_p
    cp = ctypes.c_char_p
    L.swe_snapshot_open.argtypes = [cp, ctypes.POINTER(SnapshotParams), ctypes.POINTER(vp)]
    L.swe_snapshot_open.restype = ctypes.c_int
    L.swe_snapshot_bathymetry.argtypes = [vp, dp]
    L.swe_snapshot_bathymetry.restype = ctypes.c_int
    L.swe_snapshot_metadata.argtypes = [vp, ctypes.c_double, cp, cp, cp, cp, cp, cp]
    L.swe_snapshot_metadata.restype = ctypes.c_int
    L.swe_snapshot_write_host.argtypes = [vp, ctypes.c_double, dp, dp, dp]
    L.swe_snapshot_write_host.restype = ctypes.c_int
    L.swe_snapshot_write.argtypes = [vp, vp, ctypes.c_double]
    L.swe_snapshot_write.restype = ctypes.c_int
    L.swe_snapshot_flush.argtypes = [vp]
    L.swe_snapshot_flush.restype = ctypes.c_int
    L.swe_snapshot_records.argtypes = [vp]
    L.swe_snapshot_records.restype = ctypes.c_longlong
    L.swe_snapshot_stats.argtypes = [vp, dp, dp, ctypes.POINTER(ctypes.c_longlong)]
    L.swe_snapshot_stats.restype = ctypes.c_int
    L.swe_snapshot_close.argtypes = [vp]
    L.swe_snapshot_close.restype = ctypes.c_int
    L.swe_snapshot_destroy.argtypes = [vp]
    L.swe_snapshot_destroy.restype = None
    L.swe_snapshot_last_error.argtypes = [vp]
    L.swe_snapshot_last_error.restype = cp
    L.swe_sanity_log_open.argtypes = [cp, cp, cp, ctypes.c_int, ctypes.c_double, cp, cp, cp,
                                      cp, cp, cp, ctypes.POINTER(vp)]
    L.swe_sanity_log_open.restype = ctypes.c_int
    L.swe_sanity_log_write.argtypes = [vp, ctypes.c_ulonglong, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double]
    L.swe_sanity_log_write.restype = ctypes.c_int
    L.swe_sanity_log_close.argtypes = [vp]
    L.swe_sanity_log_close.restype = ctypes.c_int
    L.swe_sanity_log_destroy.argtypes = [vp]
    L.swe_sanity_log_destroy.restype = None
    L.swe_sanity_log_last_error.argtypes = [vp]
    L.swe_sanity_log_last_error.restype = cp
    _lib = L
    return L
