"""The LSD radix form (TURTLE_FORM_RADIX) on the GPU.

The radix form moves keys by 8-bit digits, least significant first, each
pass a stable counting scatter; digits on which every key agrees are
skipped.  Its output must be the stable sort, the same bytes as the pivot
forms and as the reference (keys and ids; integer data, zero tolerance).
The cases cover every dtype, sizes around the pass tiles (4096 keys, 2048 for
64-bit keys, 6144 for keys-only sorts of at least 2^24 8- to 32-bit keys), inputs on which some, all or no digits are skipped (even and odd
numbers of moving passes: the result ends in the scratch buffer and is copied
back), float keys in totalOrder, the device entry point, and the fallback of
batched sorts to a pivot form.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import ALL_DTYPES
from test_float_gpu import bits, expected_order, make_floats
from turtlesort_gb300 import TurtleSort
from turtlesort_gb300 import datagen as dg

pytestmark = pytest.mark.gpu


def _sort_radix(keys, ids, cap=None):
    with TurtleSort(keys.dtype, cap or max(keys.size, 2), track_index=ids is not None) as s:
        s.set_pivot_rule("radix")
        k = keys.copy()
        i = ids.copy() if ids is not None else None
        s.StartSorting(k, i)
        s.Sync()
        return k, i, s.last_levels


def _check(keys, ids, k, i):
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k, keys[order])
    if ids is not None:
        assert np.array_equal(i, ids[order])


@pytest.mark.parametrize("dtype", ALL_DTYPES)
@pytest.mark.parametrize("n", [2, 3, 255, 2047, 2048, 2049, 4095, 4096, 4097, 3 * 4096 + 5,
                               6143, 6144, 6145, 3 * 6144 + 7, 100_003, 1_048_583])
def test_radix_dtypes_and_tile_edges(gpu, dtype, n):
    keys = dg.uniform(dtype, n, 9000 + n)
    ids = np.arange(n, dtype=np.int32)[::-1].copy()
    for with_ids in (True, False):
        k, i, _ = _sort_radix(keys, ids if with_ids else None)
        _check(keys, ids if with_ids else None, k, i)


@pytest.mark.parametrize("dtype", [np.uint8, np.int16, np.int32, np.uint32, np.float32])
@pytest.mark.parametrize("n", [(1 << 24) - 1, (1 << 24) + 3 * 6144 + 7])
def test_radix_wide_tiles_without_ids(gpu, dtype, n):
    """Keys-only sorts of 2^24 keys and more rank 6144-key tiles; one key
    fewer takes the 4096-key tiles.  Both sides of the switch, ragged last
    tiles, uniform and narrow keys (two moving passes)."""
    if dtype == np.float32:
        keys = make_floats(dtype, n, "wide", 61)
        k, _, _ = _sort_radix(keys, None)
        assert np.array_equal(bits(k), bits(keys[expected_order(keys)]))
        return
    for name in ("uniform", "narrow"):
        keys = _dist(dtype, n, name, 6144)
        k, _, _ = _sort_radix(keys, None)
        assert np.array_equal(k, np.sort(keys, kind="stable")), name


def _dist(dtype, n, name, seed):
    u = dg.uniform(np.uint64, n, seed)
    w = np.dtype(dtype).itemsize * 8
    if name == "uniform":
        return dg.uniform(dtype, n, seed)
    if name == "narrow":  # [0, 1023]: only the low two digits move keys
        return (u % 1024).astype(dtype)
    if name == "equal":  # no digit moves keys
        return np.full(n, 77, dtype=dtype)
    if name == "sorted":
        return np.sort(dg.uniform(dtype, n, seed))
    if name == "reverse":
        return np.sort(dg.uniform(dtype, n, seed))[::-1].copy()
    if name == "top_byte":  # one moving digit (the top one): odd number of passes
        return ((u % 251) << np.uint64(w - 8)).astype(np.uint64).astype(dtype) if w > 8 else (u % 251).astype(dtype)
    if name == "two_spread":  # digits 0 and the top one move keys, the middle ones not
        lo = u % 7
        hi = (u >> np.uint64(8)) % 5
        return (lo | (hi << np.uint64(w - 8))).astype(np.uint64).astype(dtype)
    raise ValueError(name)


@pytest.mark.parametrize("dtype", [np.int32, np.uint64, np.int16, np.int8])
@pytest.mark.parametrize("dist", ["uniform", "narrow", "equal", "sorted", "reverse",
                                  "top_byte", "two_spread"])
def test_radix_distributions(gpu, dtype, dist):
    n = 2_000_003
    keys = _dist(dtype, n, dist, 4242)
    ids = np.arange(n, dtype=np.int32)
    k, i, levels = _sort_radix(keys, ids)
    _check(keys, ids, k, i)
    if dist == "equal":
        assert levels == 0
    if dist == "top_byte" and np.dtype(dtype).itemsize > 1:
        assert levels == 1
    k2, _, _ = _sort_radix(keys, None)
    assert np.array_equal(k2, k)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("dist", ["normal", "wide", "dups", "specials"])
def test_radix_float_keys(gpu, dtype, dist):
    n = 700_001
    x = make_floats(dtype, n, dist, 515)
    ids = np.arange(n, dtype=np.int32)
    k, i, _ = _sort_radix(x, ids)
    order = expected_order(x)
    assert np.array_equal(bits(k), bits(x[order]))
    assert np.array_equal(i, ids[order])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_radix_float_all_equal(gpu, dtype):
    """No digit moves keys: the keys are mapped to their images and back in place."""
    x = np.full(50_000, -2.5, dtype=dtype)
    k, i, levels = _sort_radix(x, np.arange(x.size, dtype=np.int32))
    assert levels == 0
    assert np.array_equal(bits(k), bits(x))
    assert np.array_equal(i, np.arange(x.size, dtype=np.int32))


@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.uint16, np.float32])
@pytest.mark.parametrize("dist", ["uniform", "equal", "top_byte", "narrow"])
def test_radix_late_ids_start_sorting(gpu, dtype, dist):
    """StartSorting with ids in pinned buffers (at least 4M keys): the ids'
    copy-in overlaps the key passes, which carry positions; a gather then
    turns positions into ids.  No, one and two moving passes (positions left
    as the identity, odd and even pass counts) and float keys."""
    torch = pytest.importorskip("torch")
    n = (1 << 22) + 4321
    if dtype == np.float32:
        keys = make_floats(dtype, n, {"uniform": "wide", "equal": "dups", "top_byte": "dups",
                                      "narrow": "specials"}[dist], 77)
        if dist == "equal":
            keys[:] = dtype(-0.75)
    else:
        keys = _dist(dtype, n, dist, 5150)
    ids = dg.uniform(np.int32, n, 99)  # arbitrary ids, not positions
    kt = torch.empty(keys.nbytes, dtype=torch.uint8, pin_memory=True)
    it = torch.empty(n, dtype=torch.int32, pin_memory=True)
    kb = kt.numpy().view(keys.dtype)[:n]
    ib = it.numpy()
    with TurtleSort(keys.dtype, n, track_index=True) as s:
        for _ in range(2):
            kb[:] = keys
            ib[:] = ids
            s.StartSorting(kb, ib)
            s.Sync()
            assert s.last_form == "radix"
            if dtype == np.float32:
                order = expected_order(keys)
                assert np.array_equal(bits(kb), bits(keys[order]))
            else:
                order = np.argsort(keys, kind="stable")
                assert np.array_equal(kb, keys[order])
            assert np.array_equal(ib, ids[order])


def test_radix_equals_pivot_forms(gpu):
    n = (1 << 24) + 3
    keys = dg.uniform(np.int32, n, 31337)
    ids = np.arange(n, dtype=np.int32)
    outs = []
    with TurtleSort(np.int32, n, track_index=True) as s:
        for rule in ("radix", "two_level", "sampled"):
            s.set_pivot_rule(rule)
            k, i = keys.copy(), ids.copy()
            s.StartSorting(k, i)
            s.Sync()
            outs.append((k, i))
    for k, i in outs[1:]:
        assert np.array_equal(k, outs[0][0]) and np.array_equal(i, outs[0][1])
    _check(keys, ids, *outs[0])


def test_radix_device_entry(gpu):
    torch = pytest.importorskip("torch")
    n = 4_000_037
    keys = dg.uniform(np.int64, n, 77)
    ids = np.arange(n, dtype=np.int32)
    dk = torch.from_numpy(keys).cuda()
    di = torch.from_numpy(ids).cuda()
    stream = torch.cuda.Stream()
    with TurtleSort(np.int64, n, track_index=True) as s:
        s.set_pivot_rule("radix")
        s.sort_device(dk.data_ptr(), di.data_ptr(), n, stream.cuda_stream)
        s.status(stream.cuda_stream)
        launches = s.launches
    _check(keys, ids, dk.cpu().numpy(), di.cpu().numpy())
    assert launches >= 3  # histogram, plan, passes, finish


def test_radix_rule_keeps_batched_sorts_on_pivots(gpu):
    torch = pytest.importorskip("torch")
    lens = np.array([5, 4097, 1, 0, 20000, 3000], dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    total = int(offs[-1])
    keys = dg.uniform(np.int32, total, 5)
    dk = torch.from_numpy(keys).cuda()
    do = torch.from_numpy(offs).cuda()
    with TurtleSort(np.int32, total, track_index=False) as s:
        s.set_pivot_rule("radix")
        s.sort_batched_device(dk.data_ptr(), None, do.data_ptr(), lens.size, total)
        s.status()
    got = dk.cpu().numpy()
    for a in range(lens.size):
        seg = keys[offs[a]:offs[a + 1]]
        assert np.array_equal(got[offs[a]:offs[a + 1]], np.sort(seg, kind="stable"))
