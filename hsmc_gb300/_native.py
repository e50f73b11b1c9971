"""ctypes binding of the C ABI in ``include/hsmc_gpu.h``.

The shared library is built in-tree (``hsmc_gb300/libhsmc_gpu.so``) by
``hsmc_gb300.build``.  Loading fails loudly when it is missing: there is no
CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "libhsmc_gpu.so")
HEADER = os.path.join(ROOT, "include", "hsmc_gpu.h")

HSMC_OK = 0
STATUS_NAMES = {
    0: "HSMC_OK",
    1: "HSMC_ERR_INVALID_ARG",
    2: "HSMC_ERR_CUDA",
    3: "HSMC_ERR_NO_DEVICE",
    4: "HSMC_ERR_CELL_OVERFLOW",
    5: "HSMC_ERR_CELL_TOO_SMALL",
    6: "HSMC_ERR_BAD_BIN",
    7: "HSMC_ERR_TIMEOUT",
    8: "HSMC_ERR_OUT_OF_BOX",
    9: "HSMC_ERR_OVERLAP",
    10: "HSMC_ERR_CAVITY_RANGE",
}


class HsmcParams(C.Structure):
    _fields_ = [
        ("n_particles", C.c_int),
        ("lattice_type", C.c_int),
        ("cells", C.c_int * 3),
        ("rho", C.c_double),
        ("box", C.c_double * 3),
        ("dr_max", C.c_double),
        ("dv_max", C.c_double),
        ("pressure", C.c_double),
        ("seed", C.c_uint64),
        ("cell_capacity", C.c_int),
        ("lanes_per_cell", C.c_int),
        ("min_cell_edge", C.c_double),
        ("cavity_pcav", C.c_double),
        ("cavity_maxdr", C.c_double),
        ("cavity_mindr", C.c_double),
        ("reserved", C.c_int * 4),
    ]


def declared_symbols() -> list[str]:
    """Every entry point include/hsmc_gpu.h declares."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hsmc_[a-z0-9_]+)\s*\(", text)))


_lib = None

_vp = C.c_void_p
_P = C.POINTER


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing; build it with hsmc_gb300.build.build() "
                          "(there is no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    L.hsmc_gpu_create.argtypes = [_P(HsmcParams), _P(_vp)]
    L.hsmc_gpu_destroy.argtypes = [_vp]
    L.hsmc_gpu_destroy.restype = None
    L.hsmc_gpu_upload_config.argtypes = [_vp, _vp, C.c_int]
    L.hsmc_gpu_download_config.argtypes = [_vp, _vp, C.c_int]
    L.hsmc_gpu_set_step.argtypes = [_vp, C.c_double, C.c_double]
    L.hsmc_gpu_sweeps.argtypes = [_vp, C.c_int, _vp]
    L.hsmc_gpu_npt_sweeps.argtypes = [_vp, C.c_int, _vp]
    L.hsmc_gpu_get_box.argtypes = [_vp, _vp]
    L.hsmc_gpu_rdf.argtypes = [_vp, C.c_double, C.c_double, C.c_int, _vp]
    L.hsmc_gpu_pressv.argtypes = [_vp, C.c_double, C.c_double, C.c_int, _vp]
    L.hsmc_gpu_presst.argtypes = [_vp, _vp, C.c_int, _vp]
    L.hsmc_gpu_scan_overlap.argtypes = [_vp, C.c_double, _P(C.c_int)]
    L.hsmc_gpu_widom.argtypes = [_vp, C.c_int64, _P(C.c_uint64)]
    L.hsmc_gpu_ql.argtypes = [_vp, C.c_int, C.c_double, _P(C.c_double), _vp]
    L.hsmc_gpu_rng_state.argtypes = [_vp, _vp]
    L.hsmc_gpu_rng_set_state.argtypes = [_vp, _vp]
    L.hsmc_gpu_strerror.argtypes = [C.c_int]
    L.hsmc_gpu_strerror.restype = C.c_char_p
    L.hsmc_gpu_overlap_replay.argtypes = [_vp, _vp, _vp, C.c_int, _vp]
    L.hsmc_gpu_widom_replay.argtypes = [_vp, _vp, C.c_int, _vp]
    L.hsmc_gpu_sweeps_traced.argtypes = [_vp, C.c_int, _vp, C.c_int64, _P(C.c_int64), _vp]
    L.hsmc_gpu_grid_info.argtypes = [_vp, _vp, _vp, _vp, _P(C.c_int)]
    L.hsmc_gpu_set_profiling.argtypes = [_vp, C.c_int]
    L.hsmc_gpu_autotune.argtypes = [_vp, C.c_int, _P(C.c_int)]
    L.hsmc_gpu_set_schedule.argtypes = [_vp, C.c_int, C.c_int]
    L.hsmc_gpu_get_schedule.argtypes = [_vp, _P(C.c_int), _P(C.c_int)]
    L.hsmc_gpu_hold_region.argtypes = [_vp, C.c_int]
    L.hsmc_gpu_cluster_moves.argtypes = [_vp, C.c_int, _vp, _vp]
    L.hsmc_gpu_cavity_psi.argtypes = [_vp, _vp, C.c_int, _vp]
    L.hsmc_gpu_cavity_trace.argtypes = [_vp, C.c_int64]
    L.hsmc_gpu_cavity_trace_read.argtypes = [_vp, _vp, C.c_int64, _P(C.c_int64)]
    L.hsmc_gpu_cluster_move_at.argtypes = [_vp, _vp, C.c_int, C.c_int, _P(C.c_int64)]
    L.hsmc_gpu_last_timing.argtypes = [_vp, _P(C.c_double), _P(C.c_double), _P(C.c_int)]
    L.hsmc_gpu_optimize.argtypes = [_vp, C.c_int, C.c_int, C.c_double, C.c_double, _vp]
    _lib = L
    return L
