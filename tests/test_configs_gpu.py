"""Every benchmark configuration at its full size, checked bit-exactly.

Each test runs one configuration of the benchmark suite at the size it is
measured at, through the same entry point the benchmark uses, and compares
the result with the oracle (the reference's 3-pivot quicksort restated on the
CPU, run on all host cores) on the same seeded input:

  plain        12,582,912 int32 in [0, 2^31-1], index initialised to the
               value: StartSorting(&values, &index) (turtle-sort.cuh:124-184;
               the reference README's benchmark, README.md:190-209)
  distribution 2^26 int32 + int32 index, distributions a-e (uniform, uniform
               [0,1023], sorted, reverse sorted, sorted with n/20 swaps)
  multisort    262,144 arrays x 1024 int32: MultiSort (turtle-sort.cuh:265-276)
  batched      100,000 uneven int32 / int16 arrays, one batched launch
  wide/narrow  2^28 int64 + index, 2^30 uint8 keys, 2^29 uint16 Zipf(1.1) keys

Keys must be bit-identical; ids must be the oracle's stable permutation (the
GB300 partition and leaf sorts are stable, so ties keep their input order).
Where the reference's own sort ran the same input (tests/golden/
ref_outputs.json: distributions a-e, int64, uint8 and the Zipf keys, keys
only), the keys must also equal the reference's output bytes.
"""
from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path

import numpy as np
import pytest

from turtlesort_gb300 import TurtleSort
from turtlesort_gb300 import datagen as dg

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
REF = json.loads((Path(__file__).resolve().parent / "golden" / "ref_outputs.json")
                 .read_text())["cases"]


def _sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _expect_reference(case, keys_in, keys_out):
    """The reference's own sort of the same input gave these bytes."""
    e = REF[case]
    assert e["ran"] and e["keys_sorted"]
    assert _sha(keys_in) == e["input_sha256"], f"{case}: input differs from the reference run's"
    assert _sha(keys_out) == e["keys_sha256"], f"{case}: keys differ from the reference's output"


def _pinned_copy(torch, arr):
    t = torch.empty(arr.nbytes, dtype=torch.uint8, pin_memory=True)
    v = t.numpy().view(arr.dtype)[: arr.size]
    v[:] = arr
    return t, v


def _first_diff(a, b) -> str:
    bad = np.flatnonzero(a != b)
    return f"{bad.size} mismatches, first at {bad[:5].tolist()}"


def _expect_equal(name, got, want):
    assert got.dtype == want.dtype and got.shape == want.shape, name
    if not np.array_equal(got, want):
        pytest.fail(f"{name}: {_first_diff(got, want)}")


def test_plain_12m_index_equals_value(gpu, oracle_mod):
    values, index = dg.plain_sort_input()  # n = 12,582,912; index = value
    ek, ei = oracle_mod.turtle_sort(values, index, threads=THREADS)
    with TurtleSort(np.int32, values.size, track_index=True) as s:
        v, i = values.copy(), index.copy()
        s.StartSorting(v, i)
        s.Sync()
    _expect_equal("keys", v, ek)
    _expect_equal("ids", i, ei)
    # the reference program's own check: every index still equals its value
    assert np.array_equal(i, v)


@pytest.mark.parametrize("kind", ["a", "b", "c", "d", "e"])
def test_distribution_2p26(gpu, oracle_mod, kind):
    torch = pytest.importorskip("torch")
    keys, idx = dg.sweep_input(kind, 1 << 26)
    ek, ei = oracle_mod.turtle_sort(keys, idx, threads=THREADS)
    with TurtleSort(np.int32, keys.size, track_index=True) as s:
        # pinned host buffers: the copy-back overlaps the leaf phase slice by slice
        tk, hk = _pinned_copy(torch, keys)
        ti, hi = _pinned_copy(torch, idx)
        s.StartSorting(hk, hi)
        s.Sync()
        _expect_equal("keys (StartSorting, pinned)", hk, ek)
        _expect_equal("ids (StartSorting, pinned)", hi, ei)
        _expect_reference(f"sweep_{kind}_2p26", keys, hk)
        # the device-resident form on the same input
        dk = torch.from_numpy(keys).cuda()
        di = torch.from_numpy(idx).cuda()
        torch.cuda.synchronize()
        s.sort_device(dk.data_ptr(), di.data_ptr(), keys.size, None)
        s.status(None)
        _expect_equal("keys (device)", dk.cpu().numpy(), ek)
        _expect_equal("ids (device)", di.cpu().numpy(), ei)


def test_multisort_262144x1024(gpu, oracle_mod):
    num, arr = 262_144, 1024
    keys = dg.uniform(np.int32, num * arr, dg.seed_for(2) + 7)
    expect = oracle_mod.multisort_heap(keys, arr, num, threads=THREADS)
    with TurtleSort(np.int32, num * arr, track_index=False) as s:
        got = keys.copy()
        s.MultiSort(arr, num, got, block_size=32)
    _expect_equal("MultiSort keys", got, expect)


@pytest.mark.parametrize("dtype", [np.int32, np.int16])
def test_batched_100k_uneven(gpu, oracle_mod, dtype):
    torch = pytest.importorskip("torch")
    keys, offs, idx = dg.batched_input(dtype, with_index=True)
    num, total = offs.size - 1, int(offs[-1])
    ek, ei = oracle_mod.segmented_sort(keys, offs, idx, threads=THREADS)
    with TurtleSort(dtype, total, track_index=True) as s:
        src_k = torch.from_numpy(keys.view(np.uint8).copy()).cuda()
        src_i = torch.from_numpy(idx).cuda()
        d_off = torch.from_numpy(offs).cuda()
        k, i = torch.empty_like(src_k), torch.empty_like(src_i)
        # the first call captures the launch in a graph, the second replays it
        for call in range(2):
            k.copy_(src_k)
            i.copy_(src_i)
            torch.cuda.synchronize()
            s.sort_batched_device(k.data_ptr(), i.data_ptr(), d_off.data_ptr(), num, total, None)
            s.status(None)
            _expect_equal(f"keys (call {call})", k.cpu().numpy().view(dtype), ek)
            _expect_equal(f"ids (call {call})", i.cpu().numpy(), ei)


def test_int64_2p28_with_index(gpu, oracle_mod):
    keys = dg.uniform(np.int64, 1 << 28, dg.seed_for(3))
    idx = np.arange(keys.size, dtype=np.int32)
    ek, ei = oracle_mod.turtle_sort(keys, idx, threads=THREADS)
    with TurtleSort(np.int64, keys.size, track_index=True) as s:
        k, i = keys.copy(), idx.copy()
        s.StartSorting(k, i)
        s.Sync()
    _expect_equal("keys", k, ek)
    _expect_equal("ids", i, ei)
    _expect_reference("int64_2p28", keys, k)


def test_uint8_2p30_keys_only(gpu, oracle_mod):
    keys = dg.uniform(np.uint8, 1 << 30, dg.seed_for(3) + 1)
    ek, _ = oracle_mod.turtle_sort(keys, None, threads=THREADS)
    with TurtleSort(np.uint8, keys.size, track_index=False) as s:
        k = keys.copy()
        s.StartSorting(k)
        s.Sync()
    _expect_equal("keys", k, ek)
    _expect_reference("uint8_2p30", keys, k)


def test_uint16_zipf_2p29_keys_only(gpu, oracle_mod):
    keys = dg.zipf_u16(1 << 29, dg.seed_for(3) + 2)
    ek, _ = oracle_mod.turtle_sort(keys, None, threads=THREADS)
    with TurtleSort(np.uint16, keys.size, track_index=False) as s:
        k = keys.copy()
        s.StartSorting(k)
        s.Sync()
    _expect_equal("keys", k, ek)
    _expect_reference("uint16_zipf_2p29", keys, k)
