"""Golden fixtures (tests/golden/, made by tests/golden/make_golden.py).

CPU: the oracle reproduces every fixture.  GPU: the CUDA path, called through
the C ABI, reproduces every fixture bit for bit (keys and ids are integers, so
the tolerance is zero), and the reference README's sample program gives the
documented output.
"""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import ROOT

GOLDEN = ROOT / "tests" / "golden"


def bits(a: np.ndarray) -> np.ndarray:
    """Bit patterns of float keys (NaN payloads and signed zeros compared
    exactly); integer keys unchanged."""
    if a.dtype == np.float32:
        return a.view(np.uint32)
    if a.dtype == np.float64:
        return a.view(np.uint64)
    return a


def load_cases():
    z = np.load(GOLDEN / "sort_cases.npz")
    for line in z["index"]:
        tag, dt, n, dist = str(line).split()
        yield tag, dt, int(n), dist, z[f"{tag}_keys"], z[f"{tag}_perm"]


def test_fixture_set_is_complete():
    seen = {(dt, dist) for _, dt, _, dist, _, _ in load_cases()}
    assert len({dt for dt, _ in seen}) == 10  # 8 integer types, float32, float64
    assert {"uniform", "dups", "extremes", "reverse"} <= {d for _, d in seen}


def test_oracle_reproduces_fixtures(oracle_mod):
    for tag, dt, n, dist, keys, perm in load_cases():
        idx = np.arange(n, dtype=np.int32)
        k, i = oracle_mod.turtle_sort(keys, idx, leaf_max=128)
        assert np.array_equal(bits(k), bits(keys[perm])), tag
        assert np.array_equal(i, perm), tag


@pytest.mark.gpu
def test_cuda_path_reproduces_fixtures(gpu):
    import turtlesort_gb300 as ts
    sorters = {}
    try:
        for tag, dt, n, dist, keys, perm in load_cases():
            key = (dt, True)
            if key not in sorters:
                sorters[key] = ts.TurtleSort(np.dtype(dt), 20_000, track_index=True)
            k = keys.copy()
            i = np.arange(n, dtype=np.int32)
            sorters[key].StartSorting(k, i)
            sorters[key].Sync()
            assert np.array_equal(bits(k), bits(keys[perm])), f"{tag} {dt} {n} {dist}"
            assert np.array_equal(i, perm), f"{tag} {dt} {n} {dist}"
            # ids initialised to the values (the reference README benchmark)
            if np.dtype(dt).kind in "iu" and np.dtype(dt).itemsize <= 4 and np.dtype(dt) != np.uint32:
                k2 = keys.copy()
                i2 = keys.astype(np.int32)
                sorters[key].StartSorting(k2, i2)
                sorters[key].Sync()
                assert np.array_equal(i2, k2.astype(np.int32)), tag
    finally:
        for s in sorters.values():
            s.close()


@pytest.mark.gpu
def test_readme_sample(gpu):
    import turtlesort_gb300 as ts
    sample = json.loads((GOLDEN / "readme_sample.json").read_text())
    v = np.array(sample["input"], dtype=np.int32)
    with ts.TurtleSort(np.int32, 1000, track_index=False) as s:
        s.StartSorting(v)
        s.Sync()
    assert v.tolist() == sample["expected"]
