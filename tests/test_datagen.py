"""Seeded generators: known answers and workload shapes (CPU)."""
from __future__ import annotations

import numpy as np

from turtlesort_gb300 import datagen as dg


def test_splitmix64_known_answers():
    # splitmix64 with state 0: the published first outputs of the generator
    out = dg.splitmix64(0, 0, 3)
    assert [hex(int(x)) for x in out] == ["0xe220a8397b1dcdaf", "0x6e789e6aa1b965f4",
                                          "0x6c45d188009454f"]


def test_chunks_are_independent():
    a = dg.splitmix64(5, 0, 1000)
    b = np.concatenate([dg.splitmix64(5, 0, 400), dg.splitmix64(5, 400, 600)])
    assert np.array_equal(a, b)


def test_ranges():
    v = dg.uniform(np.int32, 100_000, 1, 0, 1023)
    assert v.min() >= 0 and v.max() <= 1023
    f = dg.uniform(np.int8, 100_000, 2)
    assert f.min() == -128 and f.max() == 127
    u = dg.uniform(np.uint64, 1000, 3)
    assert u.dtype == np.uint64


def test_workloads_shapes():
    v, i = dg.plain_sort_input(1000)
    assert np.array_equal(v, i) and v.min() >= 0
    for kind in "abcde":
        k, idx = dg.sweep_input(kind, 4000)
        assert k.dtype == np.int32 and np.array_equal(idx, np.arange(4000))
    k, _ = dg.sweep_input("c", 4000)
    assert np.all(k[:-1] <= k[1:])
    k, _ = dg.sweep_input("d", 4000)
    assert np.all(k[:-1] >= k[1:])
    lens = dg.loguniform_lengths(10_000, 16, 65536, 9)
    assert lens.min() >= 16 and lens.max() <= 65536
    z = dg.zipf_u16(100_000, 4)
    assert z.dtype == np.uint16 and np.bincount(z).argmax() == 0
