"""ctypes binding of libturtle_gb300.so (the C ABI in include/turtle_gb300.h).

The library is built in-tree by turtlesort_gb300/build.py.  There is no
fallback: if the shared library is missing, loading fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libturtle_gb300.so"

# turtle_dtype
INT8, UINT8, INT16, UINT16, INT32, UINT32, INT64, UINT64, FLOAT32, FLOAT64 = range(10)

STATUS = {
    0: "TURTLE_OK",
    1: "TURTLE_ERR_INVALID_ARGUMENT",
    2: "TURTLE_ERR_TOO_LARGE",
    3: "TURTLE_ERR_CUDA",
    4: "TURTLE_ERR_OUT_OF_MEMORY",
    5: "TURTLE_ERR_TIMEOUT",
    6: "TURTLE_ERR_CAPACITY",
    7: "TURTLE_ERR_STATE",
    8: "TURTLE_ERR_ALIGNMENT",
    9: "TURTLE_ERR_NO_DEVICE",
    10: "TURTLE_ERR_BUDGET",
}

# (name, restype, argtypes) for every entry point of include/turtle_gb300.h
_P = C.c_void_p
_I64 = C.c_int64
_I = C.c_int
SIGNATURES = [
    ("turtle_create", _I, [_I, _I64, _I, _I, _I, C.POINTER(_P)]),
    ("turtle_destroy", _I, [_P]),
    ("turtle_compression_ok", _I, [_P]),
    ("turtle_start", _I, [_P, _P, _P, _I64]),
    ("turtle_sync", _I, [_P, C.POINTER(C.c_double)]),
    ("turtle_multisort", _I, [_P, _P, _I64, _I64, _I, C.POINTER(C.c_double)]),
    ("turtle_multisort_idx", _I, [_P, _P, _P, _I64, _I64, _I, C.POINTER(C.c_double)]),
    ("turtle_sort_device", _I, [_P, _P, _P, _I64, _P]),
    ("turtle_sort_batched_device", _I, [_P, _P, _P, _P, _I64, _I64, _P]),
    ("turtle_multisort_device", _I, [_P, _P, _P, _I64, _I64, _P]),
    ("turtle_stream_status", _I, [_P, _P]),
    ("turtle_launch_count", _I64, [_P]),
    ("turtle_last_levels", _I, [_P]),
    ("turtle_last_form", _I, [_P]),
    ("turtle_max_elements", _I64, [_I, _I]),
    ("turtle_smem_capacity", _I64, [_I, _I]),
    ("turtle_status_string", C.c_char_p, [_I]),
    ("turtle_last_cuda_error", C.c_char_p, [_P]),
    ("turtle_debug_fail_allocations", None, [_I]),
    ("turtle_debug_fail_allocation_at", None, [_I]),
    ("turtle_version", C.c_char_p, []),
    ("turtle_debug_timeline", _I, [_P, _P, _P, _I]),
    ("turtle_sort_device_noalloc", _I, [_I, _P, _P, _I64, _P]),
    ("turtle_noalloc_max_elements", _I64, []),
    ("turtle_set_pivot_rule", _I, [_P, _I]),
    ("turtle_debug_time_kernels", _I, [_P, _I]),
    ("turtle_debug_kernel_times", _I, [_P, _I, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("turtle_debug_pass_times", _I, [_P, _I, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("turtle_debug_error_site", _I, [_P, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I)]),
    ("turtle_debug_yield_threshold", _I, [_P, C.c_int32]),
    ("turtle_debug_barrier_polls", _I, [_P, _I64]),
    ("turtle_debug_radix_stall", _I, [_P, _I64]),
    ("turtle_set_tuning", _I, [_P, _I]),
    ("turtle_set_config", _I, [_P, _I, _I, _I, _I, _I]),
    ("turtle_tuning_lookup", _I, [_I, _I, _I64, _P]),
    ("turtle_tuning_multisort_geometry", _I, [_I, _I, _I64]),
    ("turtle_tuning_source", C.c_char_p, []),
    ("turtle_leaf_geometry", _I, [_I, _I, _P]),
    ("turtle_debug_multisort_geometry", _I, [_I, _P, _P, _I64, _I64, _I, _P]),
    ("turtle_server_create", _I, [_I, _I64, _I, _I64, C.POINTER(_P)]),
    ("turtle_server_submit", _I, [_P, _I, _P, _P, _I64, C.POINTER(C.c_uint64)]),
    ("turtle_server_poll", _I, [_P, C.c_uint64, C.POINTER(_I)]),
    ("turtle_server_wait", _I, [_P, C.c_uint64, C.POINTER(C.c_double)]),
    ("turtle_server_drain", _I, [_P]),
    ("turtle_server_get_stats", _I, [_P, _P]),
    ("turtle_server_destroy", _I, [_P]),
]


class ServerStats(C.Structure):
    """turtle_server_stats of include/turtle_gb300.h."""

    _fields_ = [
        ("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64),
        ("batches", C.c_int64), ("keys", C.c_int64),
        ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("mean_ms", C.c_double),
        ("max_ms", C.c_double), ("span_s", C.c_double), ("keys_per_s", C.c_double),
        ("in_use_bytes", C.c_int64),
    ]

_lib = None


class TurtleError(RuntimeError):
    """A non-zero turtle_status returned by the native library."""

    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        name = STATUS.get(status, str(status))
        super().__init__(f"{where}: {name}" + (f" ({detail})" if detail else ""))


def load() -> C.CDLL:
    """Load the in-tree shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -m turtlesort_gb300.build` "
            "(the CUDA extension is required; there is no CPU fallback)")
    lib = C.CDLL(os.fspath(LIB_PATH))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
