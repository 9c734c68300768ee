"""Serving loop (turtle_server_*): continuous batching under an HBM budget.

Mixed requests (three dtypes, with and without ids, sizes log-uniform, some
empty) are submitted from several host threads; every result must equal the
stable sort of that request alone (keys and ids are integers: zero tolerance)
and the same request sorted alone by a TurtleSort sorter.  Budget admission is
checked with a request that can never fit.
"""
from __future__ import annotations

import threading

import numpy as np
import pytest

import turtlesort_gb300 as ts
from turtlesort_gb300 import datagen as dg

pytestmark = pytest.mark.gpu

MIX = [(np.int32, 0.60), (np.int64, 0.25), (np.uint16, 0.15)]


def _torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _requests(count, seed, lo=1, hi=1 << 18, pinned=True):
    torch = _torch_cuda()
    rng = np.random.default_rng(seed)
    out = []
    for r in range(count):
        u = rng.random()
        dt = MIX[0][0] if u < 0.60 else (MIX[1][0] if u < 0.85 else MIX[2][0])
        n = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        if r % 17 == 0:
            n = 0 if r % 34 == 0 else 1
        keys = dg.uniform(dt, n, seed * 1000 + r)
        with_idx = rng.random() < 0.5
        if pinned:
            kt = torch.empty(n, dtype=getattr(torch, np.dtype(dt).name if dt != np.uint16 else "int16"),
                             pin_memory=True)
            k = kt.numpy().view(dt)
            k[:] = keys
            it = None
            if with_idx:
                it = torch.empty(n, dtype=torch.int32, pin_memory=True)
                it.numpy()[:] = np.arange(n, dtype=np.int32)[::-1]
            out.append((keys, k, it.numpy() if it is not None else None, (kt, it)))
        else:
            k = keys.copy()
            i = np.arange(n, dtype=np.int32)[::-1].copy() if with_idx else None
            out.append((keys, k, i, None))
    return out


def _expect(keys, idx0):
    order = np.argsort(keys, kind="stable")
    return keys[order], (idx0[order] if idx0 is not None else None)


def test_server_mixed_requests_match_alone():
    _torch_cuda()
    reqs = _requests(160, 3)
    with ts.TurtleServer(hbm_budget_bytes=8 << 30) as srv:
        tickets = [None] * len(reqs)

        def submit(lo, hi):
            for r in range(lo, hi):
                _, k, i, _ = reqs[r]
                tickets[r] = srv.submit(k, i)

        th = [threading.Thread(target=submit, args=(a, min(a + 40, len(reqs))))
              for a in range(0, len(reqs), 40)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        lats = [srv.wait(t) for t in tickets]
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["batches"] >= 1 and st["batches"] <= len(reqs)
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"] + 1e-9
    assert all(x >= 0 for x in lats)
    for r, (keys, k, i, _) in enumerate(reqs):
        n = keys.size
        ek, ei = _expect(keys, np.arange(n, dtype=np.int32)[::-1] if i is not None else None)
        assert np.array_equal(k, ek), f"request {r} ({keys.dtype}, n={n}): keys differ"
        if i is not None:
            assert np.array_equal(i, ei), f"request {r} ({keys.dtype}, n={n}): ids differ"
    # the same requests sorted alone by the drop-in sorter give the same bytes
    for r in (1, 2, 3, 5, 8):
        keys, k, i, _ = reqs[r]
        alone_k = keys.copy()
        alone_i = np.arange(keys.size, dtype=np.int32)[::-1].copy() if i is not None else None
        with ts.TurtleSort(keys.dtype, max(keys.size, 2), track_index=i is not None) as s:
            s.StartSorting(alone_k, alone_i)
            s.Sync()
        assert np.array_equal(alone_k, k)
        if i is not None:
            assert np.array_equal(alone_i, i)


def test_server_pageable_buffers_and_large_request():
    _torch_cuda()
    reqs = _requests(12, 5, lo=1 << 16, hi=1 << 21, pinned=False)
    keys = dg.uniform(np.int32, 3_000_000, 77)
    big = keys.copy()
    big_idx = np.arange(keys.size, dtype=np.int32)
    with ts.TurtleServer(hbm_budget_bytes=4 << 30, max_batch_keys=1 << 20) as srv:
        tb = srv.submit(big, big_idx)
        tickets = [srv.submit(k, i) for _, k, i, _ in reqs]
        srv.drain()
        srv.wait(tb)
        for t in tickets:
            srv.wait(t)
    ek, ei = _expect(keys, np.arange(keys.size, dtype=np.int32))
    assert np.array_equal(big, ek) and np.array_equal(big_idx, ei)
    for keys_r, k, i, _ in reqs:
        ek, ei = _expect(keys_r, np.arange(keys_r.size, dtype=np.int32)[::-1] if i is not None else None)
        assert np.array_equal(k, ek)
        if i is not None:
            assert np.array_equal(i, ei)


def test_server_budget_rejects_what_never_fits():
    _torch_cuda()
    small = dg.uniform(np.int32, 10_000, 1)
    s_copy = small.copy()
    huge = np.zeros(40_000_000, dtype=np.int64)
    with ts.TurtleServer(hbm_budget_bytes=64 << 20) as srv:
        th = srv.submit(huge)
        ts_ = srv.submit(s_copy)
        with pytest.raises(ts.TurtleError) as ei:
            srv.wait(th)
        assert ei.value.status == 10  # TURTLE_ERR_BUDGET
        srv.wait(ts_)
        st = srv.stats()
    assert np.array_equal(s_copy, np.sort(small))
    assert st["failed"] == 1 and st["completed"] == 1


def test_server_float_requests():
    """float32 / float64 requests (IEEE-754 totalOrder), one of them above the
    size where batches switch to two-level passes."""
    _torch_cuda()
    rng = np.random.default_rng(9)

    def image(x):
        u = x.view(np.uint32 if x.dtype == np.float32 else np.uint64)
        sign = u.dtype.type(1) << u.dtype.type(8 * u.itemsize - 1)
        return np.where((u & sign) != 0, ~u, u | sign)

    reqs = []
    for r, (dt, n) in enumerate([(np.float32, 1000), (np.float64, 70_000), (np.float32, 9_000_000),
                                 (np.float64, 5), (np.float32, 300_001)]):
        x = rng.standard_normal(n).astype(dt)
        x[:: 97] = np.nan
        x[1:: 89] = -0.0
        x[2:: 83] = np.inf
        idx = np.arange(n, dtype=np.int32) if r % 2 == 0 else None
        reqs.append((x, x.copy(), None if idx is None else idx.copy(), idx))
    with ts.TurtleServer(hbm_budget_bytes=8 << 30) as srv:
        tickets = [srv.submit(k, i) for _, k, i, _ in reqs]
        for t in tickets:
            srv.wait(t)
    for x, k, i, idx in reqs:
        order = np.argsort(image(x), kind="stable")
        bits = np.uint32 if x.dtype == np.float32 else np.uint64
        assert np.array_equal(k.view(bits), x[order].view(bits)), (x.dtype, x.size)
        if i is not None:
            assert np.array_equal(i, idx[order]), (x.dtype, x.size)


def test_serving_workload_small_stream():
    """The benchmark suite's serving stream at 64 requests: the three passes
    (saturated, Poisson, serial StartSorting) run and every result is checked
    exactly inside the workload, which raises on any wrong request."""
    import json
    import os
    import subprocess
    import sys
    _torch_cuda()
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--workload", "serving",
                          "--requests", "64", "--arena-gb", "1"],
                         cwd=root, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads([s for s in out.stdout.splitlines() if s.startswith("{")][-1])
    assert line["config"]["requests"] == 64 and line["config"]["waves"] >= 1
    assert line["value"] > 0 and line["serial_startsorting_keys_per_s"] > 0
    assert line["checked"].startswith("all 64 requests")
