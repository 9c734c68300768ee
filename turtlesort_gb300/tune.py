"""Autotuner of the GB300 sort path's launch configuration.

Runs on a machine with the GPU.  For every key width (1, 2, 4, 8 bytes) x
index flag x size band it times device-resident sorts (uniform keys, CUDA
events on the sorting stream, input restored untimed before each sort) under
every combination of

  form       one-level passes with sampled pivots / two-level passes
  tile       partition tile of 1024, 2048 or 4096 keys
  geometry   shared-memory sort geometry 0..3 (CTA size x keys per thread)
  leaf cut   the geometry's capacity, or half of it
  grid       every resident partition CTA, or half of them (small sorts)

then times the LSD radix form at the same size: the entry's radix flag is set
when it beats the best pivot configuration (plain sorts then use it; batched
sorts keep the pivot configuration).  Per width x index flag x MultiSort array
length it times every shared-memory geometry that holds the arrays.  It writes

  turtlesort_gb300/csrc/turtle_tuning_table.inc   the table compiled into the
                                                  library (rebuild to use it)
  <out>/tuning.json                               every measurement, the
                                                  winner and the default time

    python -m turtlesort_gb300.tune --out <dir> [--quick]
    python -m turtlesort_gb300.tune --out <dir> --radix-only   # keep the pivot
        configurations of the compiled table, re-measure only the radix flags

The reference has no tuner: its geometry is fixed at compile time
(turtle-sort.cu:7,12; turtle-multi-sort.cuh:11,13).
"""
from __future__ import annotations

import argparse
import ctypes as C
import datetime
import itertools
import json
import re
import statistics
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))

import turtlesort_gb300 as ts  # noqa: E402
from turtlesort_gb300 import datagen as dg  # noqa: E402

TABLE = HERE / "csrc" / "turtle_tuning_table.inc"
SAMPLED, TWO_LEVEL, RADIX = 1, 2, 4
COMBOS = [(np.uint8, False), (np.uint8, True), (np.uint16, False), (np.uint16, True),
          (np.uint32, False), (np.uint32, True), (np.uint64, False), (np.uint64, True)]


def geometry(lib, dtype, g):
    out = (C.c_int32 * 4)()
    assert lib.turtle_leaf_geometry(ts.dtype_code(dtype), g, out)
    return {"threads": out[0], "items": out[1], "capacity": out[2], "classes": out[3]}


def configs(lib, dtype, n, quick):
    forms = [SAMPLED, TWO_LEVEL]
    tiles = [11] if quick else [10, 11, 12]
    grids = [1, 2] if n <= (1 << 22) else [1]
    out = []
    for form, tile, g, half, gd in itertools.product(forms, tiles, range(4), (False, True), grids):
        cap = geometry(lib, dtype, g)["capacity"]
        cut = cap // 2 if half else cap
        if cut < 1024 or (quick and half):
            continue
        out.append((form, tile, g, cut, gd))
    return out


class Timer:
    """Device-resident sorts of one input on one stream."""

    def __init__(self, torch, dtype, n, ids, reps):
        self.torch, self.n, self.reps = torch, n, reps
        keys = dg.uniform(dtype, n, 0x5EED + n)
        view = np.int64 if np.dtype(dtype).itemsize == 8 else {1: np.int8, 2: np.int16, 4: np.int32}[
            np.dtype(dtype).itemsize]
        self.src = torch.from_numpy(keys.view(view)).cuda()
        self.k = torch.empty_like(self.src)
        self.src_i = torch.arange(n, dtype=torch.int32, device="cuda") if ids else None
        self.i = torch.empty_like(self.src_i) if ids else None
        self.stream = torch.cuda.Stream()
        self.sorter = ts.TurtleSort(dtype, n, track_index=ids)
        self.expect = np.sort(keys).view(view)

    def run(self, cfg):
        t = self.torch
        s = self.sorter
        if cfg is None:
            s._lib.turtle_set_config(s._h, -1, 0, 0, 0, 0)
            s._lib.turtle_set_tuning(s._h, 0)
        else:
            st = s._lib.turtle_set_config(s._h, *cfg)
            if st != 0:
                return None
        times = []
        for r in range(self.reps + 1):
            with t.cuda.stream(self.stream):
                self.k.copy_(self.src)
                if self.i is not None:
                    self.i.copy_(self.src_i)
                e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
                e0.record(self.stream)
                s.sort_device(self.k.data_ptr(), self.i.data_ptr() if self.i is not None else None,
                              self.n, self.stream.cuda_stream)
                e1.record(self.stream)
            s.status(self.stream.cuda_stream)
            if r > 0:
                times.append(e0.elapsed_time(e1))
        if not np.array_equal(self.k.cpu().numpy(), self.expect):
            raise RuntimeError(f"configuration {cfg} sorted {self.n} keys wrongly")
        s._lib.turtle_set_tuning(s._h, 1)
        return statistics.median(times)

    def close(self):
        self.sorter.close()


def tune_sorts(torch, lib, bands, quick, reps, log):
    rows = []
    for dtype, ids in COMBOS:
        for n in bands:
            if np.dtype(dtype).itemsize == 8 and n > (1 << 26):
                continue
            tm = Timer(torch, dtype, n, ids, reps)
            default = tm.run(None)
            results = []
            for cfg in configs(lib, dtype, n, quick):
                ms = tm.run(cfg)
                if ms is not None:
                    results.append((ms, cfg))
            results.sort()
            best_ms, best = results[0]
            radix_ms = tm.run(radix_config(lib, dtype))
            tm.close()
            row = {"width": np.dtype(dtype).itemsize, "ids": int(ids), "n": n,
                   "default_ms": default, "best_ms": best_ms, "radix_ms": radix_ms,
                   "best": dict(zip(("form", "tile_shift", "geometry", "leaf_cut", "grid_div"), best),
                                radix=int(radix_ms < best_ms)),
                   "tried": len(results) + 1,
                   "top5": [{"ms": m, "cfg": list(c)} for m, c in results[:5]]}
            rows.append(row)
            log(f"w{row['width']} ids{ids} n={n}: default {default:.3f} ms, best {best_ms:.3f} ms "
                f"{row['best']}, radix {radix_ms:.3f} ms")
    return rows


def radix_config(lib, dtype):
    """set_config arguments of the radix form (the other values are unused by
    plain sorts)."""
    return (RADIX, 11, 1, geometry(lib, dtype, 1)["capacity"], 1)


def read_table():
    """Sort and MultiSort entries of the compiled table."""
    text = TABLE.read_text()
    sorts = [tuple(int(x) for x in m.groups()) for m in re.finditer(
        r"\{(\d+), (\d+), (\d+)LL, \{(\d+), (\d+), (\d+), (\d+), (\d+), (\d+)\}\}", text)]
    multi = [tuple(int(x) for x in m.groups()) for m in re.finditer(
        r"^\s+\{(\d+), (\d+), (\d+), (\d+)\},$", text, re.M)]
    src = re.search(r'kTuneSourceText\[\] = "([^"]*)"', text).group(1)
    return sorts, multi, src


def tune_radix_flags(torch, lib, reps, log):
    """The compiled table's pivot configurations, each timed against the radix
    form at its band size; returns the rows with their radix flags."""
    sorts, multi, src = read_table()
    dtypes = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}
    rows = []
    for w, ids, max_n, form, tile, g, cut, gd, _ in sorts:
        dtype = dtypes[w]
        tm = Timer(torch, dtype, max_n, bool(ids), reps)
        best_ms = tm.run((form, tile, g, cut, gd))
        radix_ms = tm.run(radix_config(lib, dtype))
        tm.close()
        rows.append({"width": w, "ids": ids, "n": max_n, "best_ms": best_ms, "radix_ms": radix_ms,
                     "best": {"form": form, "tile_shift": tile, "geometry": g, "leaf_cut": cut,
                              "grid_div": gd, "radix": int(radix_ms < best_ms)}})
        log(f"w{w} ids{ids} n={max_n}: pivot {best_ms:.3f} ms, radix {radix_ms:.3f} ms")
    multi_rows = [{"width": w, "ids": i, "arr": a, "best": g} for w, i, a, g in multi]
    return rows, multi_rows, src


def tune_multisort(torch, lib, lens, reps, log):
    rows = []
    for dtype, ids in [(np.uint16, False), (np.uint32, False), (np.uint32, True), (np.uint64, False)]:
        for arr in lens:
            num = max(1, (1 << 24) // arr)
            keys = dg.uniform(dtype, num * arr, 0xA11 + arr)
            view = {1: np.int8, 2: np.int16, 4: np.int32, 8: np.int64}[np.dtype(dtype).itemsize]
            src = torch.from_numpy(keys.view(view)).cuda()
            k = torch.empty_like(src)
            idx = torch.arange(num * arr, dtype=torch.int32, device="cuda") if ids else None
            expect = np.sort(keys.reshape(num, arr), axis=1).reshape(-1).view(view)
            best = None
            timings = {}
            for g in range(4):
                cap = geometry(lib, dtype, g)["capacity"]
                if arr > cap:
                    continue
                times = []
                for r in range(reps + 1):
                    k.copy_(src)
                    torch.cuda.synchronize()
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    st = lib.turtle_debug_multisort_geometry(
                        ts.dtype_code(dtype), C.c_void_p(k.data_ptr()),
                        C.c_void_p(idx.data_ptr()) if ids else None, arr, num, g,
                        C.c_void_p(torch.cuda.current_stream().cuda_stream))
                    e1.record()
                    torch.cuda.synchronize()
                    if st != 0:
                        raise RuntimeError(f"multisort geometry {g}: status {st}")
                    if r > 0:
                        times.append(e0.elapsed_time(e1))
                if not np.array_equal(k.cpu().numpy(), expect):
                    raise RuntimeError(f"multisort geometry {g} sorted wrongly ({arr})")
                timings[g] = statistics.median(times)
                if best is None or timings[g] < timings[best]:
                    best = g
            rows.append({"width": np.dtype(dtype).itemsize, "ids": int(ids), "arr": arr,
                         "ms": timings, "best": best})
            log(f"multisort w{np.dtype(dtype).itemsize} ids{int(ids)} arr={arr}: {timings} -> {best}")
    return rows


def write_table(sort_rows, multi_rows, source):
    lines = ["// Launch configuration table (see turtle_tuning.h), written by",
             "// turtlesort_gb300/tune.py; rebuild the library after changing it.",
             f'static const char kTuneSourceText[] = "{source}";',
             "static const turtle::TuneEntry kTuneTable[] = {"]
    for r in sorted(sort_rows, key=lambda r: (r["width"], r["ids"], r["n"])):
        b = r["best"]
        lines.append(f"    {{{r['width']}, {r['ids']}, {r['n']}LL, {{{b['form']}, {b['tile_shift']}, "
                     f"{b['geometry']}, {b['leaf_cut']}, {b['grid_div']}, {b.get('radix', 0)}}}}},")
    lines += ["};", "static const turtle::MultiEntry kMultiTable[] = {"]
    for r in sorted(multi_rows, key=lambda r: (r["width"], r["ids"], r["arr"])):
        lines.append(f"    {{{r['width']}, {r['ids']}, {r['arr']}, {r['best']}}},")
    lines += ["};", ""]
    TABLE.write_text("\n".join(lines))


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--quick", action="store_true", help="fewer tiles, full leaf cuts only")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--max-log2", type=int, default=26)
    ap.add_argument("--radix-only", action="store_true",
                    help="re-measure only the radix flags of the compiled table")
    args = ap.parse_args()
    import torch
    out = Path(args.out)
    out.mkdir(parents=True, exist_ok=True)
    lib = ts.load_library()
    logf = open(out / "tune.log", "w")

    def log(msg):
        print(msg, flush=True)
        logf.write(msg + "\n")

    name = torch.cuda.get_device_name(0)
    when = datetime.datetime.now(datetime.timezone.utc).strftime("%Y-%m-%d")
    if args.radix_only:
        sort_rows, multi_rows, old = tune_radix_flags(torch, lib, args.reps, log)
        source = f"{old.split('; radix flags')[0]}; radix flags {when}"
    else:
        bands = [1 << k for k in range(16, args.max_log2 + 1, 2)]
        sort_rows = tune_sorts(torch, lib, bands, args.quick, args.reps, log)
        multi_rows = tune_multisort(torch, lib, [16, 64, 256, 1024, 2048, 4096, 8192], args.reps, log)
        source = f"tune.py on {name}, {when}, uniform keys, {len(sort_rows)} bands"
    write_table(sort_rows, multi_rows, source)
    (out / "tuning.json").write_text(json.dumps({"source": source, "sorts": sort_rows,
                                                 "multisort": multi_rows}, indent=1))
    log(f"wrote {TABLE}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
