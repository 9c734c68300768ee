"""Generates the golden sort fixtures in this folder.

    python tests/golden/make_golden.py

The reference (tugrul512bit/TurtleSort) ships no golden vectors and its sort
runs only on a GPU, so the fixtures are:
  * readme_sample.json -- the reference README's sample program
    (README.md:58-75 and :104-110): {5,4,3,9,8,1} sorted through
    StartSorting/Sync must print "1 3 4 5 8 9" (the output block printed at
    README.md:79-82 does not match its own input and is not used);
  * sort_cases.npz -- seeded inputs for every dtype (the eight integer
    types, float32 and float64) and several distributions with the expected
    stable order computed by numpy's stable argsort (of the IEEE-754
    totalOrder images for float keys), an implementation independent of both
    the oracle and the CUDA path.  The expected keys are keys[perm]; the expected ids of a sort with
    ids initialised to 0..n-1 are perm itself (and, with ids initialised to the
    values as in the reference README benchmark, README.md:132-142, the ids
    equal the sorted keys).
Inputs come from the splitmix64 generator in turtlesort_gb300/datagen.py.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
from turtlesort_gb300 import datagen as dg  # noqa: E402

DTYPES = [np.int8, np.uint8, np.int16, np.uint16, np.int32, np.uint32, np.int64, np.uint64]
FLOATS = [np.float32, np.float64]
SIZES = [0, 1, 2, 3, 32, 33, 129, 1000, 4097]


def total_order_image(x: np.ndarray) -> np.ndarray:
    """Float keys -> unsigned images ordered as IEEE-754 totalOrder."""
    u = x.view(np.uint32 if x.dtype == np.float32 else np.uint64)
    sign = u.dtype.type(1) << u.dtype.type(8 * u.itemsize - 1)
    return np.where((u & sign) != 0, ~u, u | sign)


def float_cases():
    """Float keys: random bit patterns (every class of value, NaNs of both
    signs included), few distinct values, the special values, and reverse
    totalOrder.  Expected order: numpy's stable argsort of the totalOrder
    images."""
    for fi, dt in enumerate(FLOATS):
        ut = np.uint32 if dt == np.float32 else np.uint64
        specials = np.array([np.nan, -np.nan, np.inf, -np.inf, 0.0, -0.0, 1.0, -1.0,
                             np.finfo(dt).max, -np.finfo(dt).max, np.finfo(dt).tiny], dtype=dt)
        for n in SIZES:
            seed = 0x7475727431 + 101 * n + 8 + fi
            bits = dg.uniform(ut, n, seed)
            yield dt, n, "uniform", bits.view(dt).copy()
            yield dt, n, "dups", (dg.uniform(np.int32, n, seed + 1, -3, 3).astype(dt) * dt(0.25))
            pick = (dg.splitmix64(seed + 2, 0, n) % np.uint64(specials.size)).astype(np.int64)
            yield dt, n, "extremes", specials[pick]
            x = dg.uniform(ut, n, seed + 3).view(dt)
            yield dt, n, "reverse", x[np.argsort(total_order_image(x), kind="stable")][::-1].copy()
        yield dt, 20_000, "uniform", dg.uniform(ut, 20_000, 0x7475727431 + 8 + fi).view(dt).copy()


def cases():
    yield from int_cases()
    yield from float_cases()


def int_cases():
    for dt in DTYPES:
        lo, hi = dg.dtype_range(dt)
        for n in SIZES:
            seed = 0x7475727431 + 101 * n + DTYPES.index(dt)
            yield dt, n, "uniform", dg.uniform(dt, n, seed)
            yield dt, n, "dups", dg.uniform(dt, n, seed + 1, 0, 7)
            pool = np.array([lo, hi, 0, 1], dtype=dt)
            yield dt, n, "extremes", pool[(dg.splitmix64(seed + 2, 0, n) % np.uint64(4)).astype(np.int64)]
            yield dt, n, "reverse", np.sort(dg.uniform(dt, n, seed + 3))[::-1].copy()
        yield dt, 20_000, "uniform", dg.uniform(dt, 20_000, 0x7475727431 + DTYPES.index(dt))


def main() -> None:
    arrays = {}
    names = []
    for i, (dt, n, dist, keys) in enumerate(cases()):
        order_keys = total_order_image(keys) if keys.dtype in (np.float32, np.float64) else keys
        perm = np.argsort(order_keys, kind="stable").astype(np.int32)
        tag = f"c{i:03d}"
        arrays[f"{tag}_keys"] = keys
        arrays[f"{tag}_perm"] = perm
        names.append(f"{tag} {np.dtype(dt).name} {n} {dist}")
    arrays["index"] = np.array(names)
    np.savez_compressed(HERE / "sort_cases.npz", **arrays)
    sample = {"source": "README.md:58-75,104-110", "input": [5, 4, 3, 9, 8, 1],
              "dtype": "int32", "expected": [1, 3, 4, 5, 8, 9]}
    (HERE / "readme_sample.json").write_text(json.dumps(sample, indent=1) + "\n")
    print(f"{len(names)} cases written")


if __name__ == "__main__":
    main()
