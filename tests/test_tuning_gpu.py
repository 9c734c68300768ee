"""Every launch configuration the tuner can pick sorts exactly (GPU).

The configuration (pass form, partition tile, shared-memory geometry, leaf
cut, partition grid) changes only how the work is split, never the output:
each one must give the stable sort.  Also every table entry at its band size,
and MultiSort under every shared-memory geometry that holds the arrays.
"""
from __future__ import annotations

import ctypes as C
import itertools

import numpy as np
import pytest

import turtlesort_gb300 as ts
from test_tuning_cpu import parse_table
from turtlesort_gb300 import TurtleSort
from turtlesort_gb300 import datagen as dg

pytestmark = pytest.mark.gpu


def _stable(keys, idx):
    order = np.argsort(keys, kind="stable")
    return keys[order], idx[order]


@pytest.mark.parametrize("dtype", [np.int32, np.uint64, np.uint8])
def test_every_configuration_sorts_exactly(gpu, dtype):
    n = 1_500_007
    keys = dg.uniform(dtype, n, 321) if dtype != np.uint8 else dg.uniform(dtype, n, 321, 0, 40)
    idx = np.arange(n, dtype=np.int32)
    ek, ei = _stable(keys, idx)
    with TurtleSort(dtype, n, track_index=True) as s:
        for form, tile, g, half, gd in itertools.product(("sampled", "two_level"), (10, 11, 12),
                                                         range(4), (False, True), (1, 2)):
            cap = ts.leaf_geometry(dtype, g)["capacity"]
            cut = cap // 2 if half else cap
            if cut < 1024:
                continue
            s.set_config(form, tile, g, cut, gd)
            k, i = keys.copy(), idx.copy()
            s.StartSorting(k, i)
            s.Sync()
            cfg = (form, tile, g, cut, gd)
            assert np.array_equal(k, ek), f"keys differ under {cfg}"
            assert np.array_equal(i, ei), f"ids differ under {cfg}"
        s.clear_config()


def test_table_entries_sort_exactly(gpu):
    sorts, _ = parse_table()
    dtypes = {1: np.uint8, 2: np.uint16, 4: np.int32, 8: np.int64}
    seen = set()
    for w, ids, max_n, *cfg in sorts:
        n = min(max_n, 1 << 22)
        if (w, ids, n, tuple(cfg)) in seen:
            continue
        seen.add((w, ids, n, tuple(cfg)))
        dtype = dtypes[w]
        keys = dg.uniform(dtype, n, 77 + n)
        idx = np.arange(n, dtype=np.int32) if ids else None
        with TurtleSort(dtype, n, track_index=bool(ids)) as s:
            k = keys.copy()
            i = idx.copy() if ids else None
            s.StartSorting(k, i)
            s.Sync()
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(k, keys[order]), (w, ids, n, cfg)
        if ids:
            assert np.array_equal(i, idx[order]), (w, ids, n, cfg)


@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.uint16])
@pytest.mark.parametrize("arr", [7, 100, 1000, 4096, 9000])
def test_multisort_every_geometry(gpu, dtype, arr):
    torch = pytest.importorskip("torch")
    lib = ts.load_library()
    num = 333
    keys = dg.uniform(dtype, num * arr, 5 + arr)
    for g in range(4):
        cap = ts.leaf_geometry(dtype, g)["capacity"]
        d = torch.from_numpy(keys.copy()).cuda()
        ids = torch.arange(num * arr, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        st = lib.turtle_debug_multisort_geometry(ts.dtype_code(dtype), C.c_void_p(d.data_ptr()),
                                                 C.c_void_p(ids.data_ptr()), arr, num, g, None)
        torch.cuda.synchronize()
        if arr > cap:
            assert st == 2  # TURTLE_ERR_TOO_LARGE
            continue
        assert st == 0
        rows = keys.reshape(num, arr)
        order = np.argsort(rows, axis=1, kind="stable")
        exp_k = np.take_along_axis(rows, order, axis=1).reshape(-1)
        exp_i = (order + (np.arange(num) * arr)[:, None]).astype(np.int32).reshape(-1)
        assert np.array_equal(d.cpu().numpy(), exp_k), f"geometry {g}"
        assert np.array_equal(ids.cpu().numpy(), exp_i), f"geometry {g}"


@pytest.mark.parametrize("dtype", [np.int32, np.int16, np.uint8, np.int64, np.float32])
def test_largest_leaves_with_ids(gpu, dtype):
    """Arrays that fill the largest shared-memory geometry are sorted as one
    leaf: positions up to the geometry's capacity must survive the packing of
    narrow-range keys (and of full-range keys)."""
    cap = ts.leaf_geometry(dtype, 2)["capacity"]
    with TurtleSort(dtype, cap, track_index=True) as s:
        s.set_config("two_level", 11, 2, cap, 1)
        for n in (cap, cap - 1, cap // 2 + 1, 1000):
            for span in (7, 1000, None):
                if np.dtype(dtype).kind == "f":
                    keys = (dg.uniform(np.int32, n, n + 3, 0, span or 2**30)
                            .astype(np.float64) * 0.25).astype(dtype)
                else:
                    keys = (dg.uniform(dtype, n, n + 3, 0, span) if span
                            else dg.uniform(dtype, n, n + 3))
                idx = np.arange(n, dtype=np.int32)
                k, i = keys.copy(), idx.copy()
                s.StartSorting(k, i)
                s.Sync()
                ek, ei = _stable(keys, idx)
                assert np.array_equal(k, ek), (n, span)
                assert np.array_equal(i, ei), (n, span)


@pytest.mark.parametrize("form", ["sampled", "two_level"])
def test_big_leaves_at_scale(gpu, form):
    """The configuration that first exposed the position-width limit: 2^24
    keys, 1024-key tiles, the 1024-thread geometry with 16384-key leaves."""
    n = 1 << 24
    keys = dg.uniform(np.int32, n, 4711)
    idx = np.arange(n, dtype=np.int32)
    with TurtleSort(np.int32, n, track_index=True) as s:
        s.set_config(form, 10, 2, ts.leaf_geometry(np.int32, 2)["capacity"], 1)
        k, i = keys.copy(), idx.copy()
        s.StartSorting(k, i)
        s.Sync()
    assert np.all(k[1:] >= k[:-1])
    assert np.array_equal(keys[i], k)
    same = k[1:] == k[:-1]
    assert np.all(i[1:][same] > i[:-1][same])
