"""The allocation-free sort entry point, called through the C ABI.

turtle_sort_device_noalloc exists for callers that may not allocate device
memory when they sort (hosts that own a fixed device-memory pool, plugins
handed device pointers but no allocator, real-time loops that must not block
on the allocator): its scratch space is an array compiled into the library.
These tests check that its output equals the regular entry point's
(turtle_sort_device through a sorter) exactly -- keys and ids are integers, so
the tolerance is zero -- on two calls in a row (the scratch array keeps the
previous call's contents), and that oversized calls are rejected.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes when run alone.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import turtlesort_gb300 as ts
from turtlesort_gb300 import datagen as dg

pytestmark = pytest.mark.gpu


def _noalloc(lib, dtype, keys_t, idx_t, n, stream):
    return lib.turtle_sort_device_noalloc(ts.dtype_code(dtype), C.c_void_p(keys_t.data_ptr()),
                                          C.c_void_p(idx_t.data_ptr()) if idx_t is not None else None,
                                          int(n), C.c_void_p(stream) if stream else None)


@pytest.mark.parametrize("dtype", [np.int32, np.uint64, np.int8])
def test_noalloc_matches_regular_entry_point(dtype):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = ts.load_library()
    nmax = int(lib.turtle_noalloc_max_elements())
    assert nmax == 1 << 20
    stream = torch.cuda.current_stream().cuda_stream
    sorter = ts.TurtleSort(dtype, nmax, track_index=True)
    try:
        # two calls in a row with different inputs and sizes
        for call, (n, seed) in enumerate([(nmax, 11), (77_777, 12)]):
            keys = dg.uniform(dtype, n, seed)
            idx = dg.uniform(np.int32, n, seed + 100)
            k1 = torch.from_numpy(keys.copy()).cuda()
            i1 = torch.from_numpy(idx.copy()).cuda()
            k2 = k1.clone()
            i2 = i1.clone()
            torch.cuda.synchronize()
            sorter.sort_device(k1.data_ptr(), i1.data_ptr(), n, stream)
            sorter.status(stream)
            st = _noalloc(lib, dtype, k2, i2, n, stream)
            assert st == 0, f"call {call}: status {st}"
            assert torch.equal(k1, k2), f"call {call}: keys differ"
            assert torch.equal(i1, i2), f"call {call}: ids differ"
            # and both equal the stable order of the input
            order = np.argsort(keys, kind="stable")
            assert np.array_equal(k2.cpu().numpy(), keys[order])
            assert np.array_equal(i2.cpu().numpy(), idx[order])
    finally:
        sorter.close()


def test_noalloc_keys_only_and_limits():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = ts.load_library()
    nmax = int(lib.turtle_noalloc_max_elements())
    keys = dg.uniform(np.uint16, 300_001, 5)
    k = torch.from_numpy(keys.view(np.int16).copy()).cuda()
    assert _noalloc(lib, np.uint16, k, None, keys.size, 0) == 0
    got = k.cpu().numpy().view(np.uint16)
    assert np.array_equal(got, np.sort(keys))
    big = torch.zeros(nmax + 1, dtype=torch.int32, device="cuda")
    assert _noalloc(lib, np.int32, big, None, nmax + 1, 0) == 2  # TURTLE_ERR_TOO_LARGE
