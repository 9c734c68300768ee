"""Seeded synthetic inputs for the TurtleSort workloads (numpy, host side).

Every value comes from a counter-based splitmix64 stream: element i of a
stream with seed s is mix(s + (i + 1) * 0x9E3779B97F4A7C15), so any slice can
be generated independently and in chunks.  Integer ranges map as
``lo + (x mod (hi - lo + 1))`` (``x`` itself for a full 64-bit range).

Workloads (seeds are ``0x7475727431 + k`` for workload k):
  0  n = 12,582,912 int32 in [0, 2^31-1], index = value
  1  n = 2^26 int32 + int32 index (= position):
       a uniform full range, b uniform [0, 1023], c sorted ascending,
       d sorted descending, e ascending with n/20 random position-pair swaps
  2  batched: 262,144 x 1024 int32; 100,000 arrays with lengths
       floor(exp(U(ln 16, ln 65536))), int32 and int16 full range
  3  int64 2^28 full range + index; uint8 2^30 in [0,255];
       uint16 2^29 Zipf(s=1.1) over ranks 1..65536 (value = rank - 1)
  4  serving: Poisson arrivals, sizes log-uniform in [1024, 16 * 2^20],
       dtype int32 60% / int64 25% / uint16 15%, half with an index
"""
from __future__ import annotations

import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

GAMMA = np.uint64(0x9E3779B97F4A7C15)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)
SEED_BASE = 0x7475727431
CHUNK = 1 << 24


def seed_for(workload: int) -> int:
    return SEED_BASE + workload


def splitmix64(seed: int, start: int, count: int) -> np.ndarray:
    """Outputs start .. start+count-1 of the stream with this seed (uint64)."""
    i = np.arange(start + 1, start + count + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + i * GAMMA
        z = (z ^ (z >> np.uint64(30))) * M1
        z = (z ^ (z >> np.uint64(27))) * M2
        z = z ^ (z >> np.uint64(31))
    return z


def _map_range(x: np.ndarray, lo: int, hi: int, dtype) -> np.ndarray:
    r = hi - lo + 1
    with np.errstate(over="ignore"):
        if r >= (1 << 64):
            u = x
        else:
            u = x % np.uint64(r) + np.uint64(lo & 0xFFFFFFFFFFFFFFFF)
    return u.view(np.int64).astype(dtype) if np.dtype(dtype).kind == "i" else u.astype(dtype)


def dtype_range(dtype) -> tuple[int, int]:
    info = np.iinfo(np.dtype(dtype))
    return int(info.min), int(info.max)


def _chunked(n: int, fill) -> None:
    """Calls fill(c0, c) for the CHUNK-sized pieces of [0, n), on several
    threads for large n (numpy's array loops release the GIL).  The values do
    not depend on the split: every element is a function of its index."""
    starts = list(range(0, n, CHUNK))
    workers = min(len(starts), os.cpu_count() or 1, 16)
    if workers <= 1:
        for c0 in starts:
            fill(c0, min(CHUNK, n - c0))
        return
    with ThreadPoolExecutor(workers) as ex:
        list(ex.map(lambda c0: fill(c0, min(CHUNK, n - c0)), starts))


def uniform(dtype, n: int, seed: int, lo: int | None = None, hi: int | None = None,
            start: int = 0) -> np.ndarray:
    """n keys uniform in [lo, hi] (default: the dtype's full range)."""
    dlo, dhi = dtype_range(dtype)
    lo = dlo if lo is None else lo
    hi = dhi if hi is None else hi
    out = np.empty(n, dtype=dtype)

    def fill(c0, c):
        out[c0:c0 + c] = _map_range(splitmix64(seed, start + c0, c), lo, hi, dtype)

    _chunked(n, fill)
    return out


def uniform_real(n: int, seed: int, start: int = 0) -> np.ndarray:
    """n doubles in [0, 1): the top 53 bits of each draw."""
    x = splitmix64(seed, start, n)
    return (x >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def plain_sort_input(n: int = 12_582_912) -> tuple[np.ndarray, np.ndarray]:
    """Workload 0: int32 in [0, 2^31-1] with index initialised to the value."""
    v = uniform(np.int32, n, seed_for(0), 0, 2**31 - 1)
    return v, v.copy()


def sweep_input(kind: str, n: int = 1 << 26) -> tuple[np.ndarray, np.ndarray]:
    """Workload 1 (a-e): int32 keys + int32 index = position."""
    seed = seed_for(1)
    idx = np.arange(n, dtype=np.int32)
    if kind == "a":
        k = uniform(np.int32, n, seed)
    elif kind == "b":
        k = uniform(np.int32, n, seed, 0, 1023)
    elif kind in ("c", "d", "e"):
        k = np.sort(uniform(np.int32, n, seed))
        if kind == "d":
            k = k[::-1].copy()
        elif kind == "e":
            m = n // 20
            pos = (splitmix64(seed + 100, 0, 2 * m) % np.uint64(n)).astype(np.int64)
            p, q = pos[0::2], pos[1::2]
            for a, b in zip(p.tolist(), q.tolist()):  # sequential swaps, in order
                k[a], k[b] = k[b], k[a]
    else:
        raise ValueError(kind)
    return k, idx


def loguniform_lengths(num: int, lo: int, hi: int, seed: int) -> np.ndarray:
    u = uniform_real(num, seed)
    return np.floor(np.exp(np.log(lo) + u * (np.log(hi) - np.log(lo)))).astype(np.int64)


def batched_input(dtype, num: int = 100_000, lo: int = 16, hi: int = 65536,
                  with_index: bool = False) -> tuple[np.ndarray, np.ndarray, np.ndarray | None]:
    """Workload 2b: arrays packed back to back; returns (keys, offsets, idx)."""
    lens = loguniform_lengths(num, lo, hi, seed_for(2))
    offs = np.zeros(num + 1, dtype=np.int64)
    np.cumsum(lens, out=offs[1:])
    keys = uniform(dtype, int(offs[-1]), seed_for(2) + 1)
    idx = np.arange(int(offs[-1]), dtype=np.int32) if with_index else None
    return keys, offs, idx


def zipf_cdf(s: float = 1.1, ranks: int = 65536) -> np.ndarray:
    w = 1.0 / np.power(np.arange(1, ranks + 1, dtype=np.float64), s)
    c = np.cumsum(w)
    return c / c[-1]


def zipf_u16(n: int, seed: int, s: float = 1.1) -> np.ndarray:
    cdf = zipf_cdf(s)
    out = np.empty(n, dtype=np.uint16)

    def fill(c0, c):
        u = uniform_real(c, seed, c0)
        out[c0:c0 + c] = np.minimum(np.searchsorted(cdf, u, side="right"), 65535)

    _chunked(n, fill)
    return out
