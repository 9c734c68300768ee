"""Inputs of the cases run through the reference's own code.

make_ref_golden.py runs these cases through the reference (its StartSorting /
Sync and MultiSort, built from its sources by oracle/ref_build.sh) on a GPU
machine and records the output bytes in ref_outputs.json / ref_small.npz.
The tests regenerate the same inputs here and compare the oracle's and the
GB300 path's outputs with the reference's.

Each case: name, reference type code (i8 .. u64, f32, f64, or m<A>x<B> for
MultiSort<int, A, B, true>), n (keys; arrays for MultiSort), whether an index
array is passed to StartSorting, and how the input is generated.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from turtlesort_gb300 import datagen as dg

NP_TYPES = {"i8": np.int8, "u8": np.uint8, "i16": np.int16, "u16": np.uint16,
            "i32": np.int32, "u32": np.uint32, "i64": np.int64, "u64": np.uint64,
            "f32": np.float32, "f64": np.float64}

# Without a merge (n < 8,200: one chunk, turtle-sort.cuh:139-163) the
# reference's index output is the permutation its partition applied; above
# that its merge writes key values into the index (turtle-sort.cu:220,255),
# so larger cases pass ids only when they start equal to the keys.
SMALL_SIZES = [2, 31, 33, 128, 1000, 4097, 8199]
FULL = 1 << 26


@dataclass(frozen=True)
class Case:
    name: str
    type: str
    n: int
    ids: bool
    gen: str          # generator name (see make_input)
    seed: int
    reps: int = 1
    full_size: bool = False  # a benchmark configuration at its full size

    @property
    def multi(self) -> tuple[int, int] | None:
        if not self.type.startswith("m"):
            return None
        a, b = self.type[1:].split("x")
        return int(a), int(b)

    @property
    def dtype(self):
        return np.int32 if self.multi else NP_TYPES[self.type]


def cases() -> list[Case]:
    out = [Case("readme_sample", "i32", 6, False, "readme", 0),
           Case("plain12m", "i32", 12_582_912, True, "plain12m", dg.seed_for(0), reps=3)]
    for j, t in enumerate(["i8", "u8", "i16", "u16", "i32", "u32", "i64", "u64"]):
        for k, n in enumerate(SMALL_SIZES):
            out.append(Case(f"small_{t}_{n}", t, n, True, "uniform", dg.seed_for(10) + 100 * j + k))
        out.append(Case(f"medium_{t}_100003", t, 100_003, False, "uniform",
                        dg.seed_for(11) + j))
        out.append(Case(f"dups_{t}_100003", t, 100_003, False, "dups", dg.seed_for(12) + j))
    out.append(Case("real_f32_1000003", "f32", 1_000_003, False, "real", dg.seed_for(13)))
    out.append(Case("real_f64_100003", "f64", 100_003, False, "real", dg.seed_for(13) + 1))
    out += [Case("multisort_10x64", "m10x64", 64_000, False, "uniform", dg.seed_for(14)),
            Case("multisort_32x32", "m32x32", 32_768, False, "uniform", dg.seed_for(14) + 1),
            Case("multisort_128x32", "m128x32", 4_096, False, "uniform", dg.seed_for(14) + 2)]
    for kind in "abcde":
        out.append(Case(f"sweep_{kind}_2p26", "i32", FULL, False, f"sweep_{kind}", dg.seed_for(1),
                        full_size=True))
    out += [Case("int64_2p28", "i64", 1 << 28, False, "wide_i64", dg.seed_for(3), full_size=True),
            Case("uint8_2p30", "u8", 1 << 30, False, "wide_u8", dg.seed_for(3) + 1, full_size=True),
            Case("uint16_zipf_2p29", "u16", 1 << 29, False, "zipf", dg.seed_for(3) + 2,
                 full_size=True)]
    return out


def make_input(c: Case) -> tuple[np.ndarray, np.ndarray | None]:
    """(keys, ids) of a case; ids is None when the case passes no index."""
    dt = c.dtype
    total = c.n * c.multi[0] if c.multi else c.n
    if c.gen == "readme":
        return np.array([5, 4, 3, 9, 8, 1], dtype=np.int32), None
    if c.gen == "plain12m":
        return dg.plain_sort_input(c.n)
    if c.gen.startswith("sweep_"):
        k, _ = dg.sweep_input(c.gen[-1], c.n)
        return k, None
    if c.gen == "wide_i64":
        return dg.uniform(np.int64, c.n, c.seed), None
    if c.gen == "wide_u8":
        return dg.uniform(np.uint8, c.n, c.seed), None
    if c.gen == "zipf":
        return dg.zipf_u16(c.n, c.seed), None
    if c.gen == "real":
        # finite values of both signs from plain IEEE arithmetic on the
        # splitmix64 stream (no libm calls, so every platform makes the same
        # bits); no NaN or -0.0, where the reference's `<` order is defined
        u = dg.uniform_real(total, c.seed)
        return ((u - 0.5) * 2.0e6).astype(dt), None
    if c.gen == "uniform":
        keys = dg.uniform(dt, total, c.seed)
    elif c.gen == "dups":
        keys = dg.uniform(dt, total, c.seed, 0, 15)
    else:
        raise ValueError(c.gen)
    ids = np.arange(total, dtype=np.int32) if c.ids else None
    return keys, ids
