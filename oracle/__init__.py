"""CPU oracle for the TurtleSort GB300 path -- TEST INFRASTRUCTURE ONLY.

Loads oracle/_build/liboracle.so (built from oracle/turtle_oracle.cpp by
oracle/Makefile).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline legs may use it; the product package never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

_DT = {
    np.dtype(np.int8): 0, np.dtype(np.uint8): 1, np.dtype(np.int16): 2, np.dtype(np.uint16): 3,
    np.dtype(np.int32): 4, np.dtype(np.uint32): 5, np.dtype(np.int64): 6, np.dtype(np.uint64): 7,
}
_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", os.fspath(HERE)], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(os.fspath(LIB))
        P, I64, I = C.c_void_p, C.c_int64, C.c_int
        L.oracle_turtle_sort.argtypes = [I, P, P, I64, I64, I]
        L.oracle_stable_sort.argtypes = [I, P, P, I64]
        L.oracle_multisort_heap.argtypes = [I, P, I64, I64, I]
        L.oracle_segmented_sort.argtypes = [I, P, P, P, I64, I]
        L.cpu_sort_pairs.argtypes = [I, P, P, I64, I, I]
        L.cpu_sort_pairs.restype = C.c_double
        L.oracle_hardware_threads.restype = I
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def total_order_image(x: np.ndarray) -> np.ndarray:
    """Float keys -> unsigned images whose integer order is IEEE-754 totalOrder
    (-NaN < -inf < ... < -0 < +0 < ... < +inf < +NaN): negative values have
    every bit flipped, the others get the sign bit set."""
    u = x.view(np.uint32 if x.dtype == np.float32 else np.uint64)
    sign = u.dtype.type(1) << u.dtype.type(8 * u.itemsize - 1)
    return np.where((u & sign) != 0, ~u, u | sign).astype(u.dtype)


def from_total_order_image(u: np.ndarray, dtype) -> np.ndarray:
    sign = u.dtype.type(1) << u.dtype.type(8 * u.itemsize - 1)
    return np.where((u & sign) != 0, u ^ sign, ~u).astype(u.dtype).view(dtype)


def turtle_sort(keys: np.ndarray, idx: np.ndarray | None = None, leaf_max: int = 8192,
                threads: int = 1):
    """Restated reference 3-pivot quicksort (stable tie order); returns copies.
    Float keys (the reference's float/double instantiations,
    turtle-sort.cu:1136-1174) are sorted as their totalOrder images."""
    if keys.dtype in (np.float32, np.float64):
        k, i = turtle_sort(total_order_image(np.ascontiguousarray(keys)), idx, leaf_max, threads)
        return from_total_order_image(k, keys.dtype), i
    k = np.ascontiguousarray(keys).copy()
    i = None if idx is None else np.ascontiguousarray(idx, dtype=np.int32).copy()
    rc = lib().oracle_turtle_sort(_DT[k.dtype], _p(k), _p(i), k.size, leaf_max, threads)
    assert rc == 0
    return k, i


def stable_sort(keys: np.ndarray, idx: np.ndarray | None = None):
    k = np.ascontiguousarray(keys).copy()
    i = None if idx is None else np.ascontiguousarray(idx, dtype=np.int32).copy()
    rc = lib().oracle_stable_sort(_DT[k.dtype], _p(k), _p(i), k.size)
    assert rc == 0
    return k, i


def multisort_heap(keys: np.ndarray, arr_size: int, num_arrays: int, threads: int = 1):
    k = np.ascontiguousarray(keys).copy()
    rc = lib().oracle_multisort_heap(_DT[k.dtype], _p(k), arr_size, num_arrays, threads)
    assert rc == 0
    return k


def segmented_sort(keys: np.ndarray, offsets: np.ndarray, idx: np.ndarray | None = None,
                   threads: int = 1):
    k = np.ascontiguousarray(keys).copy()
    i = None if idx is None else np.ascontiguousarray(idx, dtype=np.int32).copy()
    o = np.ascontiguousarray(offsets, dtype=np.int64)
    rc = lib().oracle_segmented_sort(_DT[k.dtype], _p(k), _p(i), _p(o), o.size - 1, threads)
    assert rc == 0
    return k, i


def cpu_sort_seconds(keys: np.ndarray, idx: np.ndarray | None, mode: int, threads: int = 1):
    """Times a CPU baseline sort in place.  mode 0: std::sort (1 thread);
    1: std::sort(par_unseq); 2: __gnu_parallel::sort on `threads` threads."""
    return lib().cpu_sort_pairs(_DT[keys.dtype], _p(keys), _p(idx), keys.size, mode, threads)


def hardware_threads() -> int:
    return int(lib().oracle_hardware_threads())
