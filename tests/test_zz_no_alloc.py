"""The allocation-free sort entry point, called through the C ABI.

turtle_sort_device_noalloc exists for callers that may not allocate device
memory when they sort (hosts that own a fixed device-memory pool, plugins
handed device pointers but no allocator, real-time loops that must not block
on the allocator): its scratch space is an array compiled into the library.
These tests check that its output equals the regular entry point's
(turtle_sort_device through a sorter) exactly -- keys and ids are integers
(float keys are compared as bit patterns), so the tolerance is zero -- on two
calls in a row (the scratch array keeps the previous call's contents), that
calls after the first leave the device's free memory unchanged, and that
oversized calls are rejected.

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


def _specials(dtype, n, seed):
    """Floats with NaNs of both signs, -0.0, +0.0 and both infinities mixed
    into normal values."""
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(n).astype(dtype)
    pool = np.array([np.nan, -np.nan, np.inf, -np.inf, 0.0, -0.0], dtype=dtype)
    pick = rng.random(n) < 0.2
    x[pick] = pool[rng.integers(0, pool.size, int(pick.sum()))]
    return x


def _noalloc(lib, dtype, keys_t, idx_t, n, stream):
    return lib.turtle_sort_device_noalloc(ts.dtype_code(dtype), C.c_void_p(keys_t.data_ptr()),
                                          C.c_void_p(idx_t.data_ptr()) if idx_t is not None else None,
                                          int(n), C.c_void_p(stream) if stream else None)


@pytest.mark.parametrize("dtype", [np.int32, np.uint64, np.int8, np.float32, np.float64])
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
        # calls in a row with different inputs and sizes
        is_float = np.dtype(dtype).kind == "f"
        bits_t = np.uint32 if dtype == np.float32 else np.uint64
        # torch has no uint64 tensors: unsigned 64-bit keys travel as int64 bits
        host_t = np.int64 if dtype == np.uint64 else dtype
        for call, (n, seed) in enumerate([(nmax, 11), (77_777, 12), (nmax - 5, 13)]):
            keys = _specials(dtype, n, seed) if is_float else dg.uniform(dtype, n, seed)
            idx = dg.uniform(np.int32, n, seed + 100)
            k1 = torch.from_numpy(keys.view(host_t).copy()).cuda()
            i1 = torch.from_numpy(idx.copy()).cuda()
            k2 = k1.clone()
            i2 = i1.clone()
            torch.cuda.synchronize()
            sorter.sort_device(k1.data_ptr(), i1.data_ptr(), n, stream)
            sorter.status(stream)
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
            st = _noalloc(lib, dtype, k2, i2, n, stream)
            assert st == 0, f"call {call}: status {st}"
            torch.cuda.synchronize()
            free_after = torch.cuda.mem_get_info()[0]
            # the first call on the device may load the module that holds the
            # scratch array; every later call must leave free memory unchanged
            if call > 0:
                assert free_after == free_before, f"call {call}: free memory changed"
            got_k = k2.cpu().numpy().view(dtype)
            ref_k = k1.cpu().numpy().view(dtype)
            if is_float:  # bit patterns: NaN payloads and -0.0 must match too
                assert np.array_equal(got_k.view(bits_t), ref_k.view(bits_t)), \
                    f"call {call}: keys differ"
            else:
                assert np.array_equal(got_k, ref_k), f"call {call}: keys differ"
            assert torch.equal(i1, i2), f"call {call}: ids differ"
            # and both equal the stable order of the input (IEEE-754 totalOrder
            # for floats: the order of the sign-adjusted bit patterns)
            if is_float:
                u = keys.view(bits_t)
                sign = bits_t(1) << bits_t(8 * u.itemsize - 1)
                order = np.argsort(np.where((u & sign) != 0, ~u, u | sign), kind="stable")
                assert np.array_equal(got_k.view(bits_t), u[order])
            else:
                order = np.argsort(keys, kind="stable")
                assert np.array_equal(got_k, keys[order])
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
