"""The launch-configuration table and its lookup (no GPU needed).

turtlesort_gb300/tune.py measures configurations on the GPU and writes
turtlesort_gb300/csrc/turtle_tuning_table.inc, which is compiled into the
library.  These tests parse that file and check that the library's lookup
(turtle_tuning_lookup, turtle_tuning_multisort_geometry) returns exactly its
entries, band by band, and that every entry is a valid configuration.
"""
from __future__ import annotations

import ctypes as C
import re

import numpy as np
import pytest

from conftest import ROOT

TABLE = ROOT / "turtlesort_gb300" / "csrc" / "turtle_tuning_table.inc"
WIDTH_DTYPE = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}


def parse_table():
    text = TABLE.read_text()
    sorts = [tuple(int(x) for x in m.groups()) for m in re.finditer(
        r"\{(\d+), (\d+), (\d+)LL, \{(\d+), (\d+), (\d+), (\d+), (\d+), (\d+)\}\}", text)]
    multi = [tuple(int(x) for x in m.groups()) for m in re.finditer(
        r"^\s+\{(\d+), (\d+), (\d+), (\d+)\},$", text, re.M)]
    sorts = [r for r in sorts if r[0] != 0]
    multi = [r for r in multi if r[0] != 0]
    return sorts, multi


def lookup(lib, width, ids, n):
    import turtlesort_gb300 as ts
    out = (C.c_int32 * 6)()
    assert lib.turtle_tuning_lookup(ts.dtype_code(WIDTH_DTYPE[width]), int(ids), int(n), out) == 0
    return tuple(out)


def geometry(lib, width, g):
    import turtlesort_gb300 as ts
    out = (C.c_int32 * 4)()
    assert lib.turtle_leaf_geometry(ts.dtype_code(WIDTH_DTYPE[width]), g, out) == 1
    return tuple(out)


def test_leaf_geometries(native_lib):
    # CTA threads x keys per thread, capacity, size classes
    assert geometry(native_lib, 4, 0) == (256, 16, 4096, 9)
    assert geometry(native_lib, 4, 1) == (512, 16, 8192, 10)
    assert geometry(native_lib, 4, 2) == (1024, 16, 16384, 11)
    assert geometry(native_lib, 4, 3) == (512, 8, 4096, 10)
    assert geometry(native_lib, 8, 1) == (512, 8, 4096, 10)
    assert geometry(native_lib, 8, 3) == (512, 4, 2048, 10)
    out = (C.c_int32 * 4)()
    assert native_lib.turtle_leaf_geometry(4, 4, out) == 0
    assert native_lib.turtle_leaf_geometry(99, 0, out) == 0


def test_table_entries_are_valid(native_lib):
    sorts, multi = parse_table()
    for w, ids, max_n, form, tile, g, cut, gd, radix in sorts:
        assert w in WIDTH_DTYPE and ids in (0, 1) and max_n > 0
        assert form in (1, 2) and 10 <= tile <= 12 and 0 <= g <= 3 and gd in (1, 2, 4)
        assert radix in (0, 1)
        assert 1024 <= cut <= geometry(native_lib, w, g)[2]
    for key in {(r[0], r[1]) for r in sorts}:
        bands = [r[2] for r in sorts if (r[0], r[1]) == key]
        assert bands == sorted(bands) and len(set(bands)) == len(bands)
    for w, ids, arr, g in multi:
        assert 0 <= g <= 3 and arr <= geometry(native_lib, w, g)[2]


def test_lookup_returns_the_table(native_lib):
    sorts, _ = parse_table()
    for w in (1, 2, 4, 8):
        for ids in (0, 1):
            rows = [r for r in sorts if (r[0], r[1]) == (w, ids)]
            if not rows:
                # no entry: the compile-time defaults (two-level from 2^23 keys,
                # 2048-key tiles, geometry 1 at full capacity, whole grid)
                cap = geometry(native_lib, w, 1)[2]
                assert lookup(native_lib, w, ids, 1 << 20) == (1, 11, 1, cap, 1, 0)
                assert lookup(native_lib, w, ids, 1 << 23) == (2, 11, 1, cap, 1, 0)
                continue
            prev = 0
            for r in rows:
                for n in (prev + 1, r[2]):
                    assert lookup(native_lib, w, ids, n) == r[3:], (w, ids, n)
                prev = r[2]
            # past the last band: the last entry
            assert lookup(native_lib, w, ids, rows[-1][2] * 4) == rows[-1][3:]


def test_multisort_lookup_returns_the_table(native_lib):
    import turtlesort_gb300 as ts
    _, multi = parse_table()
    for w in (1, 2, 4, 8):
        for ids in (0, 1):
            rows = [r for r in multi if (r[0], r[1]) == (w, ids)]
            code = ts.dtype_code(WIDTH_DTYPE[w])
            if not rows:
                assert native_lib.turtle_tuning_multisort_geometry(code, ids, 1000) == -1
                continue
            prev = 0
            for r in rows:
                assert native_lib.turtle_tuning_multisort_geometry(code, ids, r[2]) == r[3]
                assert native_lib.turtle_tuning_multisort_geometry(code, ids, prev + 1) == r[3]
                prev = r[2]


def test_source_string(native_lib):
    src = native_lib.turtle_tuning_source().decode()
    assert src
    sorts, _ = parse_table()
    assert ("tune.py" in src) == bool(sorts)


def test_tuner_table_round_trip(tmp_path, monkeypatch):
    """tune.py reads the compiled table (the radix-only mode re-measures only
    the radix flags of it) and writes it back unchanged."""
    import turtlesort_gb300.tune as tune
    sorts, multi, src = tune.read_table()
    assert sorts and multi and src
    expect_sorts, expect_multi = parse_table()
    assert [tuple(r) for r in sorts] == [tuple(r) for r in expect_sorts]
    rows = [{"width": w, "ids": i, "n": n,
             "best": {"form": f, "tile_shift": t, "geometry": g, "leaf_cut": c, "grid_div": d,
                      "radix": r}}
            for w, i, n, f, t, g, c, d, r in sorts]
    mrows = [{"width": w, "ids": i, "arr": a, "best": g} for w, i, a, g in multi]
    out = tmp_path / "table.inc"
    monkeypatch.setattr(tune, "TABLE", out)
    tune.write_table(rows, mrows, src)
    monkeypatch.setattr(tune, "TABLE", tune.HERE / "csrc" / "turtle_tuning_table.inc")
    text = out.read_text()
    assert text == tune.TABLE.read_text()
