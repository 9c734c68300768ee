"""CPU tests of the oracle (test infrastructure) against independent sorts.

The restated reference quicksort (stable tie order) must equal numpy's stable
argsort and std::stable_sort on every dtype, size and distribution; the
restated MultiSort heap sort must equal np.sort per array.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import ALL_DTYPES
from turtlesort_gb300 import datagen as dg


def dists(dtype, n, seed):
    lo, hi = dg.dtype_range(dtype)
    yield "uniform", dg.uniform(dtype, n, seed)
    yield "dups", dg.uniform(dtype, n, seed, 0, 3)
    yield "equal", np.full(n, 3, dtype=dtype)
    yield "sorted", np.sort(dg.uniform(dtype, n, seed))
    yield "reverse", np.sort(dg.uniform(dtype, n, seed))[::-1].copy()
    pool = np.array([lo, hi, 0, 1], dtype=dtype)
    yield "extremes", pool[(dg.splitmix64(seed, 0, n) % np.uint64(4)).astype(np.int64)]


@pytest.mark.parametrize("dtype", ALL_DTYPES)
@pytest.mark.parametrize("n", [0, 1, 2, 3, 31, 32, 33, 129, 4097, 60_000])
@pytest.mark.parametrize("leaf", [1, 16, 128])
def test_turtle_restatement_equals_stable_sort(oracle_mod, dtype, n, leaf):
    for name, k in dists(dtype, n, 17 + n):
        idx = np.arange(n, dtype=np.int32)
        a, ai = oracle_mod.turtle_sort(k, idx, leaf_max=leaf)
        b, bi = oracle_mod.stable_sort(k, idx)
        order = np.argsort(k, kind="stable")
        assert np.array_equal(a, k[order]), name
        assert np.array_equal(ai, order.astype(np.int32)), name
        assert np.array_equal(b, a) and np.array_equal(bi, ai), name


def test_turtle_restatement_threads_do_not_change_result(oracle_mod):
    k = dg.uniform(np.int32, 3_000_000, 5)
    idx = dg.uniform(np.int32, k.size, 6)
    a, ai = oracle_mod.turtle_sort(k, idx, leaf_max=8192, threads=1)
    b, bi = oracle_mod.turtle_sort(k, idx, leaf_max=8192, threads=8)
    assert np.array_equal(a, b) and np.array_equal(ai, bi)


@pytest.mark.parametrize("dtype", ALL_DTYPES)
@pytest.mark.parametrize("arr", [1, 2, 10, 33, 1024])
def test_multisort_heap_restatement(oracle_mod, dtype, arr):
    num = 50
    k = dg.uniform(dtype, arr * num, arr)
    h = oracle_mod.multisort_heap(k, arr, num)
    assert np.array_equal(h.reshape(num, arr), np.sort(k.reshape(num, arr), axis=1))


def test_segmented(oracle_mod):
    lens = np.array([0, 1, 5, 100, 0, 3000, 2], dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    k = dg.uniform(np.int16, int(offs[-1]), 3)
    i = np.arange(k.size, dtype=np.int32)
    a, ai = oracle_mod.segmented_sort(k, offs, i)
    for s, e in zip(offs[:-1], offs[1:]):
        o = np.argsort(k[s:e], kind="stable")
        assert np.array_equal(a[s:e], k[s:e][o])
        assert np.array_equal(ai[s:e], i[s:e][o])


def test_cpu_baselines_sort(oracle_mod):
    k = dg.uniform(np.int32, 100_000, 1)
    i = np.arange(k.size, dtype=np.int32)
    for mode in (0, 1, 2):
        kk, ii = k.copy(), i.copy()
        t = oracle_mod.cpu_sort_seconds(kk, ii, mode, 2)
        assert t >= 0
        assert np.array_equal(kk, np.sort(k))
        assert np.array_equal(k[ii], kk)
