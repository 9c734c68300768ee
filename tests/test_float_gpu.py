"""Float keys (float32 / float64) on the GPU.

The reference instantiates its kernels for float and double
(turtle-sort.cu:1136-1174) and compares with `<`, so where NaNs land is
undefined there.  Here float keys sort in IEEE-754 totalOrder:
-NaN < -inf < ... < -0.0 < +0.0 < ... < +inf < +NaN, equal bit patterns in
input order.  The expected order is numpy's stable argsort of the totalOrder
images; on inputs without NaN or negative zero it equals a stable sort by
value, which is also checked.
"""
from __future__ import annotations

import numpy as np
import pytest

from turtlesort_gb300 import TurtleSort
from turtlesort_gb300 import datagen as dg

pytestmark = pytest.mark.gpu

FLOATS = [np.float32, np.float64]


def total_order_image(x: np.ndarray) -> np.ndarray:
    """Unsigned image whose integer order is IEEE-754 totalOrder."""
    u = x.view(np.uint32 if x.dtype == np.float32 else np.uint64)
    sign = u.dtype.type(1) << u.dtype.type(8 * u.itemsize - 1)
    neg = (u & sign) != 0
    return np.where(neg, ~u, u | sign)


def expected_order(x: np.ndarray) -> np.ndarray:
    return np.argsort(total_order_image(x), kind="stable")


def bits(x: np.ndarray) -> np.ndarray:
    return x.view(np.uint32 if x.dtype == np.float32 else np.uint64)


def make_floats(dtype, n, dist, seed):
    rng = np.random.default_rng(seed)
    if dist == "normal":
        return rng.standard_normal(n).astype(dtype)
    if dist == "wide":  # magnitudes over the whole exponent range, both signs
        u = dg.uniform(np.uint32 if dtype == np.float32 else np.uint64, n, seed)
        x = u.view(dtype).copy()
        x[~np.isfinite(x)] = dtype(1.5)
        return x
    if dist == "dups":
        return (rng.integers(-3, 4, n)).astype(dtype) * dtype(0.5)
    if dist == "specials":
        pool = np.array([np.nan, -np.nan, np.inf, -np.inf, 0.0, -0.0, 1.0, -1.0,
                         np.finfo(dtype).max, -np.finfo(dtype).max, np.finfo(dtype).tiny,
                         -np.finfo(dtype).tiny], dtype=dtype)
        # a second NaN payload, so equal-looking NaNs keep their bit patterns
        x = pool[rng.integers(0, pool.size, n)]
        odd = rng.random(n) < 0.05
        b = bits(x).copy()
        nan = np.isnan(x) & odd
        b[nan] |= b.dtype.type(1)
        return b.view(dtype)
    if dist == "sorted":
        return np.sort(rng.standard_normal(n).astype(dtype))
    if dist == "equal":
        return np.full(n, dtype(-0.0))
    raise ValueError(dist)


_S: dict = {}


def sorter(dtype, track=True):
    key = (np.dtype(dtype), track)
    if key not in _S:
        _S[key] = TurtleSort(dtype, 1 << 22, track_index=track)
    return _S[key]


@pytest.mark.parametrize("dtype", FLOATS)
@pytest.mark.parametrize("dist", ["normal", "wide", "dups", "specials", "sorted", "equal"])
def test_float_total_order(dtype, dist):
    s = sorter(dtype)
    t = 8192 if dtype == np.float32 else 4096
    for n in [0, 1, 2, 33, 1000, t - 1, t + 1, 70_001, 1_000_003]:
        x = make_floats(dtype, n, dist, n + 5)
        idx = np.arange(n, dtype=np.int32)
        xo, io = x.copy(), idx.copy()
        s.StartSorting(xo, io)
        s.Sync()
        order = expected_order(x)
        assert np.array_equal(bits(xo), bits(x[order])), (n, dist)
        assert np.array_equal(io, order.astype(np.int32)), (n, dist)
        if dist in ("normal", "dups", "sorted"):  # no NaN, no negative zero
            assert np.array_equal(xo, x[np.argsort(x, kind="stable")])


@pytest.mark.parametrize("dtype", FLOATS)
def test_float_keys_only_and_pivot_rules(dtype):
    n = 600_001
    x = make_floats(dtype, n, "specials", 3)
    outs = []
    for rule in ("sampled", "reference", "two_level"):
        s = TurtleSort(dtype, n, track_index=False)
        s.set_pivot_rule(rule)
        xo = x.copy()
        s.StartSorting(xo)
        s.Sync()
        s.close()
        outs.append(bits(xo))
    exp = bits(x[expected_order(x)])
    for o in outs:
        assert np.array_equal(o, exp)


@pytest.mark.parametrize("dtype", FLOATS)
def test_float_multisort(dtype):
    """MultiSort<float, 2038, 32> as in the reference's main.cpp, and short rows."""
    for arr, na in [(2038, 32 * 20), (100, 64 * 40)]:
        s = TurtleSort(dtype, arr * na, track_index=False)
        h = make_floats(dtype, arr * na, "specials", arr)
        rows = h.reshape(na, arr)
        exp = np.stack([r[expected_order(r)] for r in rows]).ravel()
        s.MultiSort(arr, na, h)
        s.close()
        assert np.array_equal(bits(h), bits(exp))


def test_float_overlapped_copies_and_yields():
    """Pinned buffers of >= 4M keys (slice-by-slice result copies) and a forced
    yield: the keys are mapped back exactly once, after the last launch."""
    import torch
    n = (1 << 22) + 99
    x = make_floats(np.float32, n, "wide", 8)
    kt = torch.empty(n, dtype=torch.float32, pin_memory=True)
    it = torch.empty(n, dtype=torch.int32, pin_memory=True)
    kb, ib = kt.numpy(), it.numpy()
    s = TurtleSort(np.float32, n, track_index=True)
    s.set_pivot_rule("two_level")  # yields are a partition-kernel path
    order = expected_order(x)
    for thresh in (0, 64):
        s.yield_threshold(thresh)
        kb[:] = x
        ib[:] = np.arange(n, dtype=np.int32)
        s.StartSorting(kb, ib)
        s.Sync()
        assert np.array_equal(bits(kb), bits(x[order]))
        assert np.array_equal(ib, order.astype(np.int32))
    s.close()


def test_float_device_batched():
    """Uneven float64 arrays in one batched launch (device API)."""
    import torch
    rng = np.random.default_rng(4)
    lens = rng.integers(0, 20_000, 300)
    offs = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    x = make_floats(np.float64, int(offs[-1]), "specials", 6)
    s = TurtleSort(np.float64, int(offs[-1]), track_index=True)
    dk = torch.from_numpy(x.copy()).cuda()
    di = torch.arange(x.size, dtype=torch.int32, device="cuda")
    do = torch.from_numpy(offs).cuda()
    st = torch.cuda.current_stream().cuda_stream
    s.sort_batched_device(dk.data_ptr(), di.data_ptr(), do.data_ptr(), len(lens), x.size, st)
    s.status(st)
    ko, io = dk.cpu().numpy(), di.cpu().numpy()
    for a in range(len(lens)):
        lo, hi = offs[a], offs[a + 1]
        seg = x[lo:hi]
        o = expected_order(seg)
        assert np.array_equal(bits(ko[lo:hi]), bits(seg[o]))
        assert np.array_equal(io[lo:hi], (o + lo).astype(np.int32))
    s.close()
