"""ctypes binding of libgmgs.so (the C ABI declared in include/gmgs.h).

The library is required: importing the solver without it raises
GMGSLibraryMissing; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

# GMGS_LIB selects another build of the library, e.g. the checked build
# (gmgs-3d_gb300/build.py --debug writes libgmgs_checked.so)
LIB_PATH = Path(os.environ.get("GMGS_LIB") or Path(__file__).resolve().parent / "libgmgs.so")

# status codes (enum gmgs_status)
OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_RESOLUTION = 2
ERR_NO_SOLID = 3
ERR_NO_LOADS = 4
ERR_NO_FIXINGS = 5
ERR_NOT_SPD = 6
ERR_MAX_ITERATIONS = 7
ERR_NONFINITE = 8
ERR_NO_SOLUTION = 9
ERR_CUDA = 10
ERR_OUT_OF_MEMORY = 11
ERR_STATE = 12
ERR_MESH = 13

FP64 = 0
MIXED = 1

DOT_NOALLOC_MAX_N = 536870912   # GMGS_DOT_NOALLOC_MAX_N

# every function the header declares, with (restype, argtypes)
_p = C.c_void_p
_i32 = C.c_int32
_i64 = C.c_int64
_d = C.c_double
_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)


class Params(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_it", C.c_int32), ("omega", C.c_double),
                ("youngs_modulus", C.c_double), ("poisson_ratio", C.c_double),
                ("coarsest_resolution_control", C.c_int64), ("num_levels", C.c_int32),
                ("precision", C.c_int32), ("verbose", C.c_int32)]


SIGNATURES = {
    "gmgs_default_params": (None, [C.POINTER(Params)]),
    "gmgs_create": (C.c_int, [_i32p, _i32, _i32, _i32, _dp, C.POINTER(Params), C.POINTER(_p)]),
    "gmgs_set_bc": (C.c_int, [_p, _i32p, _i64, _dp, _i64]),
    "gmgs_set_density": (C.c_int, [_p, _dp, _d]),
    "gmgs_solve": (C.c_int, [_p, _dp, _i32p, _dp, _dp]),
    "gmgs_solve_dev": (C.c_int, [_p, _p, _i32p, _dp, _dp]),
    "gmgs_stress": (C.c_int, [_p, _dp, _fp]),
    "gmgs_stress_dev": (C.c_int, [_p, _p, _p]),
    "gmgs_grad": (C.c_int, [_p, _dp, _dp]),
    "gmgs_grad_dev": (C.c_int, [_p, _p, _p]),
    "gmgs_apply_operator": (C.c_int, [_p, _i32, _dp, _dp]),
    "gmgs_apply_preconditioner": (C.c_int, [_p, _dp, _dp]),
    "gmgs_apply_operator_dev": (C.c_int, [_p, _i32, _p, _p]),
    "gmgs_apply_preconditioner_dev": (C.c_int, [_p, _p, _p]),
    "gmgs_dot_dev": (C.c_int, [_p, _p, _p, _i64, _dp]),
    "gmgs_dot_dev_noalloc": (C.c_int, [_p, _p, _i64, _p, _p]),
    "gmgs_num_levels": (C.c_int, [_p, _i32p]),
    "gmgs_num_nodes": (C.c_int, [_p, _i32, _i64p]),
    "gmgs_num_elements": (C.c_int, [_p, _i32, _i64p]),
    "gmgs_padded_dims": (C.c_int, [_p, _i32p]),
    "gmgs_set_stream": (C.c_int, [_p, _p]),
    "gmgs_set_tolerance": (C.c_int, [_p, _d, _i32]),
    "gmgs_device_bytes": (C.c_int, [_p, _i64p]),
    "gmgs_launch_count": (C.c_int, [_p, _i64p]),
    "gmgs_voxelize_mesh": (C.c_int, [_dp, _i64, _i32p, _i64, _i32, _i32p, _i32p]),
    "gmgs_memory_stats": (C.c_int, [_i64p, _i64p, _i32]),
    "gmgs_phase_times": (C.c_int, [_p, _dp]),
    "gmgs_set_profiling": (C.c_int, [_p, _i32]),
    "gmgs_kernel_time": (C.c_int, [_p, _i32, _i64p, _dp, _dp]),
    "gmgs_last_error": (C.c_char_p, [_p]),
    "gmgs_status_string": (C.c_char_p, [C.c_int]),
    "gmgs_destroy": (None, [_p]),
}


class GMGSLibraryMissing(RuntimeError):
    pass


_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load libgmgs.so (built by gmgs-3d_gb300/build.py) and declare its ABI."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise GMGSLibraryMissing(
            f"{p} not found: build it with `python gmgs-3d_gb300/build.py` (the solver has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib
