"""GB300-native TurtleSort sort path.

Python mirror of the reference host API (turtle-sort.cuh:31-283) over the
C ABI of libturtle_gb300.so.  The class and method names follow the reference
so that code and tests read like the reference's own programs::

    sorter = TurtleSort(np.int32, max_elements=n, compress=False)
    sorter.StartSorting(values, index)   # asynchronous, like the reference
    seconds = sorter.Sync()              # values/index sorted in place
    seconds = sorter.MultiSort(arr_size, num_arrays, host_array)

Device-resident forms (no reference counterpart) take raw device pointers
(e.g. ``tensor.data_ptr()``) and a CUDA stream handle.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _native
from ._native import TurtleError

__all__ = ["TurtleSort", "TurtleServer", "TurtleError", "dtype_code", "smem_capacity",
           "load_library", "tuning_lookup", "leaf_geometry", "tuning_source"]

_DTYPES = {
    np.dtype(np.int8): _native.INT8,
    np.dtype(np.uint8): _native.UINT8,
    np.dtype(np.int16): _native.INT16,
    np.dtype(np.uint16): _native.UINT16,
    np.dtype(np.int32): _native.INT32,
    np.dtype(np.uint32): _native.UINT32,
    np.dtype(np.int64): _native.INT64,
    np.dtype(np.uint64): _native.UINT64,
    np.dtype(np.float32): _native.FLOAT32,  # IEEE-754 totalOrder (NaNs by sign at the ends)
    np.dtype(np.float64): _native.FLOAT64,
}


def load_library():
    return _native.load()


def dtype_code(dtype) -> int:
    dt = np.dtype(dtype)
    if dt not in _DTYPES:
        raise TypeError(f"unsupported key dtype {dt} (int8..uint64, float32, float64)")
    return _DTYPES[dt]


def smem_capacity(dtype, track_index: bool = True) -> int:
    """Longest array the one-CTA shared-memory sort handles for this dtype."""
    return int(load_library().turtle_smem_capacity(dtype_code(dtype), int(track_index)))


CUDA_STREAM_LEGACY = 1  # cudaStreamLegacy: the legacy default stream


def _stream(stream) -> Optional[C.c_void_p]:
    """None -> the sorter's own stream (NULL in the C ABI); 0 -> the legacy
    default stream (torch's default stream handle is 0); else the handle."""
    if stream is None:
        return None
    return C.c_void_p(CUDA_STREAM_LEGACY if int(stream) == 0 else int(stream))


_SITES = {1: "grid barrier wait", 3: "bulk-copy wait", 4: "work list full"}


def _check(st: int, where: str, handle=None) -> None:
    if st != 0:
        detail = ""
        if handle is not None:
            lib = load_library()
            raw = lib.turtle_last_cuda_error(handle)
            detail = raw.decode() if raw else ""
            if st in (5, 6):  # device-side: say which wait or list
                site, block, info = C.c_int(), C.c_int(), C.c_int()
                lib.turtle_debug_error_site(handle, C.byref(site), C.byref(block), C.byref(info))
                detail = (f"{_SITES.get(site.value, site.value)} in block {block.value}, "
                          f"info {info.value}")
        raise TurtleError(st, where, detail)


class TurtleSort:
    """Mirror of Turtle::TurtleSort<Type, TrackIndex> (turtle-sort.cuh:31-283).

    ``dtype`` is the key type (the reference's template parameter), ``track_index``
    the TrackIndex template flag, ``max_elements``/``compress`` the constructor
    arguments (turtle-sort.cuh:63).
    """

    def __init__(self, dtype, max_elements: int, compress: bool = False,
                 track_index: bool = True, device: int = -1):
        self._lib = load_library()
        self.dtype = np.dtype(dtype)
        self._code = dtype_code(self.dtype)
        self.max_elements = int(max_elements)
        self.track_index = bool(track_index)
        h = C.c_void_p()
        _check(self._lib.turtle_create(self._code, self.max_elements, int(track_index),
                                       int(compress), int(device), C.byref(h)),
               "TurtleSort()")
        self._h = h
        self._pending = None

    # -- lifetime --
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.turtle_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- reference API --
    def MemoryCompressionSuccessful(self) -> bool:
        return bool(self._lib.turtle_compression_ok(self._h))

    def StartSorting(self, values: np.ndarray, index: Optional[np.ndarray] = None) -> None:
        """Starts sorting ``values`` (and reorders ``index`` alongside); returns
        immediately.  Both arrays are updated in place by :meth:`Sync`."""
        if values.dtype != self.dtype or not values.flags.c_contiguous:
            raise TypeError(f"values must be a contiguous {self.dtype} array")
        if not self.track_index:
            index = None  # TrackIndex=false ignores the index (turtle-sort.cuh:176-179)
        if index is not None:
            if index.dtype != np.int32 or not index.flags.c_contiguous:
                raise TypeError("index must be a contiguous int32 array")
            if index.shape[0] != values.shape[0]:
                raise ValueError("values and index must have the same size")
        n = int(values.shape[0])
        st = self._lib.turtle_start(self._h, values.ctypes.data_as(C.c_void_p),
                                    index.ctypes.data_as(C.c_void_p) if index is not None else None,
                                    n)
        _check(st, "StartSorting", self._h)
        self._pending = (values, index)  # keep the buffers alive until Sync

    def Sync(self) -> float:
        """Waits for the sort, writes results back; returns elapsed seconds."""
        secs = C.c_double(0.0)
        st = self._lib.turtle_sync(self._h, C.byref(secs))
        self._pending = None
        _check(st, "Sync", self._h)
        return float(secs.value)

    def MultiSort(self, arr_size: int, num_arrays: int, host: np.ndarray,
                  block_size: int = 32, index: Optional[np.ndarray] = None) -> float:
        """Sorts ``num_arrays`` contiguous arrays of ``arr_size`` keys in place
        (MultiSort<Type, arrSize, blockSize>, turtle-sort.cuh:265-276).  With
        ``index`` (int32, one per key; a sorter made with track_index) the ids
        are permuted with the keys, stably within each array."""
        if host.dtype != self.dtype or not host.flags.c_contiguous:
            raise TypeError(f"host must be a contiguous {self.dtype} array")
        if host.size < arr_size * num_arrays:
            raise ValueError("host array smaller than num_arrays * arr_size")
        if index is not None and (index.dtype != np.int32 or not index.flags.c_contiguous or
                                  index.size < arr_size * num_arrays):
            raise ValueError("index must be a contiguous int32 array with one id per key")
        secs = C.c_double(0.0)
        st = self._lib.turtle_multisort_idx(
            self._h, host.ctypes.data_as(C.c_void_p),
            index.ctypes.data_as(C.c_void_p) if index is not None else None, int(arr_size),
            int(num_arrays), int(block_size), C.byref(secs))
        _check(st, "MultiSort", self._h)
        return float(secs.value)

    # -- device-resident forms --
    def sort_device(self, keys_ptr: int, idx_ptr: Optional[int], n: int, stream=None) -> None:
        """Sorts on ``stream`` (a CUDA stream handle; 0 = legacy default stream,
        None = the sorter's own stream).  Asynchronous."""
        st = self._lib.turtle_sort_device(self._h, C.c_void_p(keys_ptr),
                                          C.c_void_p(idx_ptr) if idx_ptr else None, int(n),
                                          _stream(stream))
        _check(st, "sort_device", self._h)

    def sort_batched_device(self, keys_ptr: int, idx_ptr: Optional[int], offsets_ptr: int,
                            num: int, total: int, stream=None) -> None:
        st = self._lib.turtle_sort_batched_device(
            self._h, C.c_void_p(keys_ptr), C.c_void_p(idx_ptr) if idx_ptr else None,
            C.c_void_p(offsets_ptr), int(num), int(total), _stream(stream))
        _check(st, "sort_batched_device", self._h)

    def multisort_device(self, keys_ptr: int, idx_ptr: Optional[int], arr_size: int,
                         num_arrays: int, stream=None) -> None:
        st = self._lib.turtle_multisort_device(
            self._h, C.c_void_p(keys_ptr), C.c_void_p(idx_ptr) if idx_ptr else None,
            int(arr_size), int(num_arrays), _stream(stream))
        _check(st, "multisort_device", self._h)

    def status(self, stream=None) -> None:
        """Waits for ``stream`` (None = the sorter's own stream) and raises if
        the device reported an error."""
        st = self._lib.turtle_stream_status(self._h, _stream(stream))
        _check(st, "device status", self._h)

    @property
    def launches(self) -> int:
        return int(self._lib.turtle_launch_count(self._h))

    def timeline(self):
        """(ns, info) arrays of the last persistent sort's phase timeline."""
        ns = np.zeros(256, dtype=np.uint64)
        info = np.zeros(256, dtype=np.int32)
        n = self._lib.turtle_debug_timeline(self._h, ns.ctypes.data_as(C.c_void_p),
                                            info.ctypes.data_as(C.c_void_p), 256)
        return ns[:n], info[:n]

    @property
    def last_levels(self) -> int:
        return int(self._lib.turtle_last_levels(self._h))

    @property
    def last_form(self) -> str:
        """Form of the last enqueued sort: 'radix', 'two_level', 'sampled' or
        'reference'."""
        return {0: "reference", 1: "sampled", 2: "two_level", 4: "radix"}.get(
            int(self._lib.turtle_last_form(self._h)), "none")

    def set_pivot_rule(self, rule: str) -> None:
        """'auto' (default: the tuned table's form), 'sampled' (quartiles of
        31 evenly spaced keys), 'reference' (the reference's median of
        start/middle/stop keys), 'two_level' (passes of two levels, 31
        classes) or 'radix' (LSD passes over 8-bit digits; plain sorts, batched
        sorts keep a pivot form); same output."""
        code = {"reference": 0, "sampled": 1, "two_level": 2, "auto": 3, "radix": 4}[rule]
        _check(self._lib.turtle_set_pivot_rule(self._h, code), "set_pivot_rule", self._h)

    def error_site(self):
        """(device status, site, block, info) of the last sort's device-side error."""
        site, block, info = C.c_int(), C.c_int(), C.c_int()
        st = self._lib.turtle_debug_error_site(self._h, C.byref(site), C.byref(block),
                                               C.byref(info))
        return int(st), int(site.value), int(block.value), int(info.value)

    def time_kernels(self, enable: bool = True) -> None:
        """Record CUDA events around the partition and leaf kernels of every
        later sort (see kernel_times)."""
        _check(self._lib.turtle_debug_time_kernels(self._h, int(enable)), "time_kernels", self._h)

    def yield_threshold(self, leaves: int) -> None:
        """Testing: yield to the leaf phase whenever more than ``leaves`` leaves
        are pending (0 = only when the lists could overflow)."""
        _check(self._lib.turtle_debug_yield_threshold(self._h, int(leaves)), "yield_threshold",
               self._h)

    # -- launch configuration (the output never depends on it) --
    def set_tuning(self, enable: bool = True) -> None:
        """Use the tuned configuration table (default) or the compile-time
        defaults."""
        _check(self._lib.turtle_set_tuning(self._h, int(enable)), "set_tuning", self._h)

    def set_config(self, form: str, tile_shift: int, geometry: int, leaf_cut: int,
                   grid_div: int = 1) -> None:
        """Pin a launch configuration: form 'sampled' (one-level passes),
        'two_level' or 'radix' (LSD digit passes: the other values then apply
        only to batched sorts), tile of 1 << tile_shift keys, shared-memory
        geometry 0..3, leaf cut, partition grid divisor 1/2/4."""
        code = {"sampled": 1, "two_level": 2, "radix": 4}[form]
        _check(self._lib.turtle_set_config(self._h, code, int(tile_shift), int(geometry),
                                           int(leaf_cut), int(grid_div)), "set_config", self._h)

    def clear_config(self) -> None:
        """Back to the tuned table after set_config."""
        _check(self._lib.turtle_set_config(self._h, -1, 0, 0, 0, 0), "clear_config", self._h)

    def barrier_polls(self, polls: int) -> None:
        """Testing: give up a grid-barrier wait after ``polls`` polls (the
        sort then reports TURTLE_ERR_TIMEOUT); 0 restores the default."""
        _check(self._lib.turtle_debug_barrier_polls(self._h, int(polls)), "barrier_polls",
               self._h)

    def radix_stall(self, tile: int) -> None:
        """Testing: tile ``tile`` of every later radix digit pass never
        publishes its look-back words, so the sort runs into the poll limit and
        reports TURTLE_ERR_TIMEOUT; a negative tile turns this off."""
        _check(self._lib.turtle_debug_radix_stall(self._h, int(tile)), "radix_stall", self._h)

    def kernel_times(self, last: int):
        """(sorts, partition_ms, leaf_ms) summed over the last `last` timed sorts."""
        pm, lm = C.c_double(), C.c_double()
        n = self._lib.turtle_debug_kernel_times(self._h, int(last), C.byref(pm), C.byref(lm))
        return int(n), float(pm.value), float(lm.value)

    def pass_times(self, last: int):
        """(sorts, setup_ms, pass_ms) summed over the last `last` timed sorts:
        the partition time split where the partition kernel (radix form: the
        first digit pass) starts."""
        su, pm = C.c_double(), C.c_double()
        n = self._lib.turtle_debug_pass_times(self._h, int(last), C.byref(su), C.byref(pm))
        return int(n), float(su.value), float(pm.value)


def tuning_lookup(dtype, track_index: bool, n: int) -> dict:
    """The tuned configuration the table gives a sort of n keys."""
    out = (C.c_int32 * 6)()
    _check(load_library().turtle_tuning_lookup(dtype_code(dtype), int(track_index), int(n), out),
           "tuning_lookup")
    return {"form": out[0], "tile_shift": out[1], "geometry": out[2], "leaf_cut": out[3],
            "grid_div": out[4], "radix": out[5]}


def leaf_geometry(dtype, g: int) -> dict:
    """Shared-memory sort geometry g: CTA threads, keys per thread, capacity,
    size classes."""
    out = (C.c_int32 * 4)()
    if not load_library().turtle_leaf_geometry(dtype_code(dtype), int(g), out):
        raise ValueError(f"no geometry {g}")
    return {"threads": out[0], "items": out[1], "capacity": out[2], "classes": out[3]}


def tuning_source() -> str:
    return load_library().turtle_tuning_source().decode()


class TurtleServer:
    """Continuous-batching sort server over the C ABI (turtle_server_*).

    No reference counterpart: a serving process on the reference issues one
    StartSorting/Sync pair per request (turtle-sort.cuh:124-258).  Requests are
    numpy arrays sorted in place; submit() returns a ticket, wait() blocks on
    it.  Arrays should live in pinned memory for full copy speed (any host
    memory works) and must stay alive until wait() returns.
    """

    def __init__(self, hbm_budget_bytes: int, device: int = -1, max_batch_requests: int = 0,
                 max_batch_keys: int = 0):
        self._lib = load_library()
        h = C.c_void_p()
        st = self._lib.turtle_server_create(int(device), int(hbm_budget_bytes),
                                            int(max_batch_requests), int(max_batch_keys),
                                            C.byref(h))
        _check(st, "turtle_server_create")
        self._h = h
        self._keep = {}

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.turtle_server_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, values: np.ndarray, index: Optional[np.ndarray] = None) -> int:
        if not values.flags.c_contiguous:
            raise ValueError("values must be C-contiguous")
        if index is not None:
            if index.dtype != np.int32 or index.shape != values.shape or not index.flags.c_contiguous:
                raise ValueError("index must be a C-contiguous int32 array of the values' shape")
        t = C.c_uint64()
        st = self._lib.turtle_server_submit(
            self._h, dtype_code(values.dtype), values.ctypes.data_as(C.c_void_p),
            index.ctypes.data_as(C.c_void_p) if index is not None else None, int(values.size),
            C.byref(t))
        _check(st, "turtle_server_submit")
        self._keep[t.value] = (values, index)
        return int(t.value)

    def poll(self, ticket: int) -> bool:
        d = C.c_int()
        _check(self._lib.turtle_server_poll(self._h, C.c_uint64(ticket), C.byref(d)),
               "turtle_server_poll")
        return bool(d.value)

    def wait(self, ticket: int) -> float:
        """Blocks until the request is sorted; returns its latency in seconds."""
        lat = C.c_double()
        st = self._lib.turtle_server_wait(self._h, C.c_uint64(ticket), C.byref(lat))
        self._keep.pop(ticket, None)
        _check(st, "turtle_server_wait")
        return float(lat.value)

    def drain(self) -> None:
        _check(self._lib.turtle_server_drain(self._h), "turtle_server_drain")

    def stats(self) -> dict:
        s = _native.ServerStats()
        _check(self._lib.turtle_server_get_stats(self._h, C.byref(s)), "turtle_server_get_stats")
        return {name: getattr(s, name) for name, _ in s._fields_}
