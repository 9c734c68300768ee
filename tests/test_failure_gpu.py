"""Failure paths of the sort path, exercised without faulting the GPU.

* A bounded device-side wait that runs out: a test-only poll limit makes the
  persistent kernel's grid-barrier wait give up at once; the sort must report
  TURTLE_ERR_TIMEOUT (the reference aborts the process on any CUDA error,
  turtle-globals.cuh:18-30), and the next sort on the same sorter must be
  exact.  Only the grid-barrier wait is shortened: a CTA has no bulk copy in
  flight while it waits there.  The radix form's look-back wait is made to
  run out by a tile that never publishes its words (a flag nothing sets).
* Device-buffer allocation failures injected on the host: the constructor
  fails with TURTLE_ERR_OUT_OF_MEMORY at each of its buffers in turn and
  leaves no device memory behind (turtle-buffer.cuh:43-57 is the reference's
  allocation path).
* Compressible buffers (TurtleSort(n, optInCompression=true),
  turtle-sort.cuh:63-113): the sort is exact whether or not the driver
  grants generic compression, and what it granted is reported.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import turtlesort_gb300 as ts
from turtlesort_gb300 import TurtleError, TurtleSort
from turtlesort_gb300 import datagen as dg

pytestmark = pytest.mark.gpu

TIMEOUT = 5
OUT_OF_MEMORY = 4


def _stable(keys, idx):
    order = np.argsort(keys, kind="stable")
    return keys[order], idx[order]


@pytest.mark.parametrize("rule", ["sampled", "two_level"])
def test_grid_barrier_timeout_then_recovers(gpu, rule):
    n = 1 << 21
    s = TurtleSort(np.int32, n, track_index=True)
    try:
        s.set_pivot_rule(rule)
        keys = dg.uniform(np.int32, n, 4242)
        idx = np.arange(n, dtype=np.int32)
        s.barrier_polls(1)
        k, i = keys.copy(), idx.copy()
        s.StartSorting(k, i)
        with pytest.raises(TurtleError) as ei:
            s.Sync()
        assert ei.value.status == TIMEOUT
        status, site, _block, _info = s.error_site()
        assert status == TIMEOUT and site == 1  # the grid-barrier wait gave up
        # the context is usable and the sorter sorts exactly again
        s.barrier_polls(0)
        ek, eidx = _stable(keys, idx)
        for _ in range(2):
            k, i = keys.copy(), idx.copy()
            s.StartSorting(k, i)
            s.Sync()
            assert np.array_equal(k, ek) and np.array_equal(i, eidx)
    finally:
        s.close()


def test_device_form_reports_timeout(gpu):
    torch = pytest.importorskip("torch")
    n = 300_001
    s = TurtleSort(np.uint64, n, track_index=False)
    try:
        keys = dg.uniform(np.uint64, n, 99)
        d = torch.from_numpy(keys.view(np.int64).copy()).cuda()
        torch.cuda.synchronize()
        s.set_pivot_rule("two_level")  # the grid-barrier wait of the partition kernel
        s.barrier_polls(1)
        s.sort_device(d.data_ptr(), None, n, None)
        with pytest.raises(TurtleError) as ei:
            s.status(None)
        assert ei.value.status == TIMEOUT
        s.barrier_polls(0)
        d.copy_(torch.from_numpy(keys.view(np.int64).copy()))
        torch.cuda.synchronize()
        s.sort_device(d.data_ptr(), None, n, None)
        s.status(None)
        assert np.array_equal(d.cpu().numpy().view(np.uint64), np.sort(keys))
    finally:
        s.close()


@pytest.mark.parametrize("stall", [0, 7, 250])
def test_radix_lookback_timeout_then_recovers(gpu, stall):
    n = (1 << 20) + 17  # 257 tiles of 4096 keys
    s = TurtleSort(np.int32, n, track_index=True)
    try:
        s.set_pivot_rule("radix")
        keys = dg.uniform(np.int32, n, 777)
        idx = np.arange(n, dtype=np.int32)
        s.barrier_polls(20000)
        s.radix_stall(stall)
        k, i = keys.copy(), idx.copy()
        s.StartSorting(k, i)
        with pytest.raises(TurtleError) as ei:
            s.Sync()
        assert ei.value.status == TIMEOUT
        status, site, _block, info = s.error_site()
        assert status == TIMEOUT and site == 5 and info > stall  # a later tile gave up
        # no wait was unbounded: the sorter sorts exactly again
        s.radix_stall(-1)
        s.barrier_polls(0)
        ek, eidx = _stable(keys, idx)
        for _ in range(2):
            k, i = keys.copy(), idx.copy()
            s.StartSorting(k, i)
            s.Sync()
            assert s.last_form == "radix"
            assert np.array_equal(k, ek) and np.array_equal(i, eidx)
    finally:
        s.close()


def test_allocation_failure_leaves_nothing_behind(gpu):
    torch = pytest.importorskip("torch")
    lib = ts.load_library()
    n = 1 << 24  # 64 MiB per key buffer: a leak would show in the free memory
    TurtleSort(np.int32, n, track_index=True).close()  # modules loaded before measuring
    torch.cuda.synchronize()
    # keysA, keysB, idxA, idxB, work lists: fail each one in turn
    for k in range(1, 6):
        free0 = torch.cuda.mem_get_info()[0]
        lib.turtle_debug_fail_allocation_at(k)
        h = C.c_void_p()
        st = lib.turtle_create(ts.dtype_code(np.int32), n, 1, 0, -1, C.byref(h))
        lib.turtle_debug_fail_allocation_at(0)
        assert st == OUT_OF_MEMORY, f"allocation {k}: status {st}"
        assert not h.value
        free1 = torch.cuda.mem_get_info()[0]
        assert abs(free1 - free0) <= (4 << 20), f"allocation {k}: {free0 - free1} bytes kept"
    # the blanket form: every allocation of the next constructor fails
    lib.turtle_debug_fail_allocations(1)
    with pytest.raises(TurtleError) as ei:
        TurtleSort(np.int64, n, track_index=False)
    lib.turtle_debug_fail_allocations(0)
    assert ei.value.status == OUT_OF_MEMORY
    # and a sorter built afterwards works
    s = TurtleSort(np.int32, n, track_index=True)
    try:
        keys = dg.uniform(np.int32, 100_000, 7)
        idx = np.arange(keys.size, dtype=np.int32)
        k, i = keys.copy(), idx.copy()
        s.StartSorting(k, i)
        s.Sync()
        ek, eidx = _stable(keys, idx)
        assert np.array_equal(k, ek) and np.array_equal(i, eidx)
    finally:
        s.close()


@pytest.mark.parametrize("dtype", [np.int32, np.uint8, np.int64])
def test_compressed_buffers_sort_exactly(gpu, dtype, record_property):
    n = 3_000_000
    s = TurtleSort(dtype, n, compress=True, track_index=True)
    try:
        granted = s.MemoryCompressionSuccessful()
        record_property("compression_granted", bool(granted))
        print(f"\ncompressible buffers for {np.dtype(dtype).name}: granted={granted}")
        for dist, seed in [("uniform", 1), ("dups", 2)]:
            keys = (dg.uniform(dtype, n, seed) if dist == "uniform"
                    else dg.uniform(dtype, n, seed, 0, 15))
            idx = np.arange(n, dtype=np.int32)
            k, i = keys.copy(), idx.copy()
            s.StartSorting(k, i)
            s.Sync()
            ek, eidx = _stable(keys, idx)
            assert np.array_equal(k, ek) and np.array_equal(i, eidx)
    finally:
        s.close()
