"""Parity of the GB300 sort path against the CPU oracle (runs on a GPU).

Every case goes through the C ABI (via the Python mirror of the reference
API).  Values must be bit-identical to np.sort / the oracle; the index output
must equal the oracle's stable order exactly (the GB300 partition and leaf
sorts are stable, so ties keep their input order), which also proves it is a
permutation with orig[idx[i]] == out[i].
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import ALL_DTYPES
from turtlesort_gb300 import TurtleSort, TurtleError, smem_capacity
from turtlesort_gb300 import datagen as dg

pytestmark = pytest.mark.gpu

_SORTERS: dict = {}


def sorter(dtype, track=True, max_n=1 << 21):
    key = (np.dtype(dtype), track, max_n)
    if key not in _SORTERS:
        _SORTERS[key] = TurtleSort(dtype, max_n, compress=False, track_index=track)
    return _SORTERS[key]


def make_keys(dtype, n, dist, seed):
    lo, hi = dg.dtype_range(dtype)
    if dist == "uniform":
        return dg.uniform(dtype, n, seed)
    if dist == "dups":
        return dg.uniform(dtype, n, seed, 0, 3)
    if dist == "equal":
        return np.full(n, 7 if lo >= 0 else -5, dtype=dtype)
    if dist == "sorted":
        return np.sort(dg.uniform(dtype, n, seed))
    if dist == "reverse":
        return np.sort(dg.uniform(dtype, n, seed))[::-1].copy()
    if dist == "organ":
        s = np.sort(dg.uniform(dtype, n, seed))
        return np.concatenate([s[0::2], s[1::2][::-1]])[:n].astype(dtype)
    if dist == "extremes":
        pool = np.array([lo, hi, 0, 1, hi - 1, lo + 1] + ([-1] if lo < 0 else []), dtype=dtype)
        pick = (dg.splitmix64(seed, 0, n) % np.uint64(pool.size)).astype(np.int64)
        return pool[pick]
    if dist == "two":
        pair = np.array([lo, hi], dtype=dtype)
        return pair[(dg.uniform(np.uint8, n, seed) & 1).astype(np.int64)]
    raise ValueError(dist)


def check_sorted_pair(keys_in, out_k, out_i, idx_in):
    order = np.argsort(keys_in, kind="stable")
    exp_k = keys_in[order]
    assert out_k.dtype == keys_in.dtype
    bad = np.nonzero(out_k != exp_k)[0]
    assert bad.size == 0, f"{bad.size} key mismatches, first at {bad[:5]}"
    if idx_in is not None:
        exp_i = idx_in[order]
        badi = np.nonzero(out_i != exp_i)[0]
        assert badi.size == 0, f"{badi.size} index mismatches, first at {badi[:5]}"


def tile(dtype):
    return smem_capacity(dtype)


SIZES_SMALL = [0, 1, 2, 3, 16, 17, 31, 32, 33, 127, 128, 129, 1000]


@pytest.mark.parametrize("dtype", ALL_DTYPES)
@pytest.mark.parametrize("dist", ["uniform", "dups", "equal", "sorted", "reverse", "organ",
                                  "extremes", "two"])
def test_start_sync_sizes(dtype, dist):
    t = tile(dtype)
    sizes = SIZES_SMALL + [t - 1, t, t + 1, 2 * t + 3, 4 * t - 1, 50_000, 300_001]
    s = sorter(dtype)
    for j, n in enumerate(sizes):
        k = make_keys(dtype, n, dist, 1000 + j)
        idx = np.arange(n, dtype=np.int32)
        ko, io = k.copy(), idx.copy()
        s.StartSorting(ko, io)
        s.Sync()
        check_sorted_pair(k, ko, io, idx)


@pytest.mark.parametrize("dtype", ALL_DTYPES)
def test_keys_only(dtype):
    s = sorter(dtype, track=False)
    for n in [5, 4096, 70_000, 1_000_000]:
        k = dg.uniform(dtype, n, 77 + n)
        ko = k.copy()
        s.StartSorting(ko)
        s.Sync()
        assert np.array_equal(ko, np.sort(k))


@pytest.mark.parametrize("dtype", [np.int32, np.uint8, np.int64])
def test_large_matches_oracle(dtype, oracle_mod):
    n = 2_000_000
    s = sorter(dtype)
    for dist, seed in [("uniform", 1), ("dups", 2), ("sorted", 3)]:
        k = make_keys(dtype, n, dist, seed)
        idx = dg.uniform(np.int32, n, seed + 50)  # arbitrary payload
        ko, io = k.copy(), idx.copy()
        s.StartSorting(ko, io)
        s.Sync()
        ek, ei = oracle_mod.turtle_sort(k, idx, leaf_max=tile(dtype), threads=4)
        assert np.array_equal(ko, ek)
        assert np.array_equal(io, ei)


def test_index_equals_value_readme_check():
    # the reference benchmark's own check (README.md:190-209): index
    # initialised to the value must still equal the value after sorting
    v, i = dg.plain_sort_input(1 << 20)
    s = sorter(np.int32)
    s.StartSorting(v, i)
    s.Sync()
    assert np.all(v[:-1] <= v[1:])
    assert np.array_equal(v, i)


def test_device_api_torch():
    torch = pytest.importorskip("torch")
    n = 1 << 20
    k = dg.uniform(np.int32, n, 5)
    i = np.arange(n, dtype=np.int32)
    tk = torch.from_numpy(k.copy()).cuda()
    ti = torch.from_numpy(i.copy()).cuda()
    s = sorter(np.int32)
    stream = torch.cuda.current_stream().cuda_stream
    s.sort_device(tk.data_ptr(), ti.data_ptr(), n, stream)
    s.status(stream)
    check_sorted_pair(k, tk.cpu().numpy(), ti.cpu().numpy(), i)


@pytest.mark.parametrize("dtype", [np.int32, np.int16, np.uint64])
def test_batched_uneven(dtype, oracle_mod):
    torch = pytest.importorskip("torch")
    num = 3000
    lens = dg.loguniform_lengths(num, 1, 40000, 11)
    lens[::97] = 0
    offs = np.zeros(num + 1, dtype=np.int64)
    np.cumsum(lens, out=offs[1:])
    total = int(offs[-1])
    k = dg.uniform(dtype, total, 12)
    i = np.arange(total, dtype=np.int32)
    s = sorter(dtype, max_n=max(total, 1 << 21))
    tk = torch.from_numpy(k.copy()).cuda()
    ti = torch.from_numpy(i.copy()).cuda()
    to = torch.from_numpy(offs).cuda()
    for rep in range(2):  # second call replays the captured graph
        tk.copy_(torch.from_numpy(k))
        ti.copy_(torch.from_numpy(i))
        s.sort_batched_device(tk.data_ptr(), ti.data_ptr(), to.data_ptr(), num, total)
        s.status()
        ek, ei = oracle_mod.segmented_sort(k, offs, i)
        assert np.array_equal(tk.cpu().numpy(), ek)
        assert np.array_equal(ti.cpu().numpy(), ei)


@pytest.mark.parametrize("dtype", ALL_DTYPES)
@pytest.mark.parametrize("arr", [1, 2, 10, 16, 17, 32, 100, 1024, 2038])
def test_multisort_matches_heap_oracle(dtype, arr, oracle_mod):
    num = 64 * 37
    s = sorter(dtype, track=False, max_n=1 << 23)
    k = dg.uniform(dtype, arr * num, 300 + arr)
    h = k.copy()
    s.MultiSort(arr, num, h, block_size=64)
    exp = oracle_mod.multisort_heap(k, arr, num)
    assert np.array_equal(h, exp)


def test_multisort_long_arrays_use_batched_path(oracle_mod):
    dtype = np.int32
    arr = tile(dtype) * 3 + 5
    num = 7
    s = sorter(dtype, track=False, max_n=1 << 23)
    k = dg.uniform(dtype, arr * num, 9)
    h = k.copy()
    s.MultiSort(arr, num, h, block_size=1)
    assert np.array_equal(h.reshape(num, arr), np.sort(k.reshape(num, arr), axis=1))


def test_errors():
    s = sorter(np.int32)
    big = np.zeros(s.max_elements + 1, dtype=np.int32)
    with pytest.raises(TurtleError) as e:
        s.StartSorting(big)
    assert e.value.status == 2  # TURTLE_ERR_TOO_LARGE
    with pytest.raises(TurtleError) as e:
        s.Sync()  # no StartSorting pending
    assert e.value.status == 7
    h = np.zeros(10 * 33, dtype=np.int32)
    with pytest.raises(TurtleError):
        s.MultiSort(10, 33, h, block_size=32)  # 33 % 32 != 0, as the reference requires


@pytest.mark.parametrize("dtype", [np.int32, np.uint8, np.int64, np.uint16])
def test_pivot_rules_give_the_same_result(dtype):
    """The reference pivot rule (median of start/middle/stop), the sampled rule
    (quartiles of 31 evenly spaced keys) and the two-level passes (31 classes
    per pass) must all produce the stable order: pivots and pass shape form
    the partition tree, never the output."""
    n = 700_001
    for dist, seed in [("uniform", 4), ("dups", 5), ("sorted", 6), ("organ", 7)]:
        k = make_keys(dtype, n, dist, seed)
        idx = np.arange(n, dtype=np.int32)
        outs = []
        for rule in ("reference", "sampled", "two_level", "auto"):
            s = TurtleSort(dtype, n, track_index=True)
            s.set_pivot_rule(rule)
            ko, io = k.copy(), idx.copy()
            s.StartSorting(ko, io)
            s.Sync()
            s.close()
            check_sorted_pair(k, ko, io, idx)
            outs.append((ko, io))
        for o in outs[1:]:
            assert np.array_equal(outs[0][0], o[0]) and np.array_equal(outs[0][1], o[1])


_TWO_LEVEL: dict = {}


@pytest.mark.parametrize("dtype", ALL_DTYPES)
@pytest.mark.parametrize("dist", ["uniform", "dups", "equal", "sorted", "reverse", "organ",
                                  "extremes", "two"])
def test_two_level_passes(dtype, dist):
    """Two-level passes: every dtype and key distribution, sizes from one tile
    to several passes deep, with and without ids."""
    key = np.dtype(dtype)
    if key not in _TWO_LEVEL:
        _TWO_LEVEL[key] = TurtleSort(dtype, 1 << 21, track_index=True)
        _TWO_LEVEL[key].set_pivot_rule("two_level")
    s = _TWO_LEVEL[key]
    t = tile(dtype)
    for n in [t + 1, 4 * t + 7, 70_001, 1 << 21]:
        k = make_keys(dtype, n, dist, n % 97)
        idx = np.arange(n, dtype=np.int32)
        ko, io = k.copy(), idx.copy()
        s.StartSorting(ko, io)
        s.Sync()
        check_sorted_pair(k, ko, io, idx)
        ko = k.copy()
        s.StartSorting(ko)
        s.Sync()
        assert np.array_equal(ko, np.sort(k, kind="stable"))


def _pinned(dtype, n):
    """A pinned host array of n elements (torch pinned bytes viewed as dtype)."""
    import torch
    t = torch.empty(n * np.dtype(dtype).itemsize, dtype=torch.uint8, pin_memory=True)
    return t, t.numpy().view(dtype)


@pytest.mark.parametrize("rule", ["auto", "two_level"])
@pytest.mark.parametrize("dtype,track", [(np.int32, True), (np.uint64, False), (np.int16, True),
                                         (np.int64, True)])
def test_overlapped_result_copies(dtype, track, rule):
    """Pinned buffers of at least 4M keys: under a pivot form the result comes
    back slice by slice while later slices are still being sorted (the radix
    form completes every slice at its end); it must equal the stable sort."""
    n = (1 << 22) + 12345
    s = TurtleSort(dtype, n, track_index=track)
    s.set_pivot_rule(rule)
    for dist, seed in [("uniform", 11), ("dups", 12), ("sorted", 13)]:
        keys = make_keys(dtype, n, dist, seed)
        kt, kb = _pinned(dtype, n)
        kb[:] = keys
        it, ib = (None, None)
        idx0 = None
        if track:
            idx0 = np.arange(n, dtype=np.int32)[::-1].copy()
            it, ib = _pinned(np.int32, n)
            ib[:] = idx0
        launches = s.launches
        s.StartSorting(kb, ib)
        s.Sync()
        assert s.launches - launches > 2  # partition + one leaf launch per slice, or radix kernels
        check_sorted_pair(keys, kb, ib, idx0)
    s.close()


@pytest.mark.parametrize("rule", ["sampled", "reference", "two_level"])
@pytest.mark.parametrize("pinned", [False, True])
def test_yield_and_resume(rule, pinned):
    """The partition stops to drain the leaf lists and resumes where it left
    off (forced by a low yield threshold); the result is unchanged, also when
    the result copies were already queued slice by slice."""
    n = (1 << 22) + 777
    s = TurtleSort(np.int32, n, track_index=True)
    s.set_pivot_rule(rule)
    plain = s.launches
    keys = make_keys(np.int32, n, "uniform", 21)
    ko = keys.copy()
    s.StartSorting(ko)
    s.Sync()
    plain = s.launches - plain
    s.yield_threshold(64)
    for dist, seed in [("uniform", 21), ("dups", 22), ("organ", 23)]:
        keys = make_keys(np.int32, n, dist, seed)
        idx0 = np.arange(n, dtype=np.int32)
        if pinned:
            kt, ko = _pinned(np.int32, n)
            it, io = _pinned(np.int32, n)
            ko[:] = keys
            io[:] = idx0
        else:
            ko, io = keys.copy(), idx0.copy()
        launches = s.launches
        s.StartSorting(ko, io)
        s.Sync()
        if dist == "uniform":
            assert s.launches - launches > plain  # it did yield
        check_sorted_pair(keys, ko, io, idx0)
    s.yield_threshold(0)
    s.close()


@pytest.mark.parametrize("dtype", [np.int32, np.uint16, np.int64, np.float64])
@pytest.mark.parametrize("arr", [5, 1024, 5000])
def test_multisort_host_with_ids(dtype, arr):
    """The host MultiSort with an id per key (turtle_multisort_idx): each
    array sorted, its ids permuted stably with it; arbitrary ids."""
    num = 32 * 5
    n = arr * num
    if dtype == np.float64:
        # + 0.0 turns -0.0 into +0.0: numpy's order ties them, totalOrder does not
        keys = np.random.default_rng(arr).standard_normal(n).round(1) + 0.0
    else:
        keys = make_keys(dtype, n, "dups", arr + 7)
    ids = np.random.default_rng(arr + 1).integers(-2**31, 2**31 - 1, n).astype(np.int32)
    with TurtleSort(dtype, n, track_index=True) as s:
        k, i = keys.copy(), ids.copy()
        secs = s.MultiSort(arr, num, k, block_size=32, index=i)
        assert secs > 0
        with pytest.raises(ValueError):
            s.MultiSort(arr, num, k, index=i[:-1])
    rows, irows = keys.reshape(num, arr), ids.reshape(num, arr)
    for r in range(num):
        order = np.argsort(rows[r], kind="stable")
        assert np.array_equal(k.reshape(num, arr)[r], rows[r][order])
        assert np.array_equal(i.reshape(num, arr)[r], irows[r][order])


@pytest.mark.parametrize("dtype", [np.int32, np.uint8, np.int64, np.float32])
@pytest.mark.parametrize("arr", [7, 100, 2038, 9000])
def test_multisort_device_with_ids(dtype, arr):
    """MultiSort with an id payload (not available in the reference,
    README.md:46): every row sorted stably, its ids reordered with it.  Rows
    up to the shared-memory capacity use the MultiSort kernel, longer rows
    the batched partition path."""
    import torch
    num = 64 * 3
    n = arr * num
    if dtype == np.float32:
        keys = np.random.default_rng(arr).standard_normal(n).astype(np.float32)
    else:
        keys = make_keys(dtype, n, "dups" if arr % 2 else "uniform", arr)
    ids = np.arange(n, dtype=np.int32)
    s = TurtleSort(dtype, n, track_index=True)
    dk = torch.from_numpy(keys.copy()).cuda()
    di = torch.from_numpy(ids.copy()).cuda()
    st = torch.cuda.current_stream().cuda_stream
    s.multisort_device(dk.data_ptr(), di.data_ptr(), arr, num, st)
    s.status(st)
    ko = dk.cpu().numpy().reshape(num, arr)
    io = di.cpu().numpy().reshape(num, arr)
    rows = keys.reshape(num, arr)
    for r in range(num):
        order = np.argsort(rows[r], kind="stable")
        assert np.array_equal(ko[r], rows[r][order]), r  # no NaN in these rows
        assert np.array_equal(io[r], (order + r * arr).astype(np.int32)), r
    s.close()


@pytest.mark.parametrize("dtype", [np.int32, np.uint64, np.int16])
def test_default_rule_above_two_level_threshold(dtype):
    """The default pivot rule switches to two-level passes from 2^23 keys up;
    those sorts must be exact too (with and without ids)."""
    n = (1 << 23) + 5
    s = TurtleSort(dtype, n, track_index=True)
    for dist, seed in [("uniform", 31), ("dups", 32), ("organ", 33)]:
        k = make_keys(dtype, n, dist, seed)
        idx = np.arange(n, dtype=np.int32)
        ko, io = k.copy(), idx.copy()
        s.StartSorting(ko, io)
        s.Sync()
        check_sorted_pair(k, ko, io, idx)
    s.close()
