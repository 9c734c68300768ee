"""Runs the reference's own sort on the cases of ref_cases.py and records
its output bytes (run on a machine with a GPU, after
`bash oracle/ref_build.sh build`; the sources were staged with
`bash oracle/ref_build.sh stage` where the reference checkout exists).

    python tests/golden/make_ref_golden.py --out <dir> [--timeout 900]

Writes <dir>/ref_outputs.json (per case: the SHA-256 of the input and of the
reference's key and index output, whether its keys are sorted and its index
output is a permutation that reorders the keys, and the Sync seconds it
printed) and <dir>/ref_small.npz (the full outputs of cases up to 8,199
keys).  Those two files are committed under tests/golden/.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import shutil
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))

from ref_cases import cases, make_input  # noqa: E402

RUNNER = ROOT / "oracle" / "_ref" / "turtle_ref"
SMALL = 8199


def sha(a: np.ndarray | None) -> str | None:
    return None if a is None else hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--timeout", type=int, default=900)
    ap.add_argument("--only", default="", help="comma-separated case names")
    args = ap.parse_args()
    out = Path(args.out)
    out.mkdir(parents=True, exist_ok=True)
    if not RUNNER.exists():
        print(f"missing {RUNNER}: run `bash oracle/ref_build.sh build` first", file=sys.stderr)
        return 2
    todo = [c for c in cases() if not args.only or c.name in args.only.split(",")]
    tmp = Path(tempfile.mkdtemp(prefix="turtle_ref_"))
    record = {"runner": "oracle/ref_driver.cu built by oracle/ref_build.sh (reference sources, "
                        "nvcc -rdc=true, sm_103a)", "cases": {}}
    small = {}
    logs = []
    stopped = None
    # one runner process per case, inputs written and removed case by case
    # (the largest case holds 2 GiB of keys); a failure other than the
    # reference's own argument-error exit stops the run
    for c in todo:
        keys, ids = make_input(c)
        entry = {"type": c.type, "n": c.n, "ids": ids is not None, "gen": c.gen, "seed": c.seed,
                 "full_size": c.full_size, "input_sha256": sha(keys),
                 "input_ids_sha256": sha(ids), "ran": False}
        record["cases"][c.name] = entry
        if stopped:
            continue
        fin, fout = tmp / f"{c.name}.in", tmp / f"{c.name}.out"
        keys.tofile(fin)
        if ids is not None:
            ids.tofile(str(fin) + ".ids")
        (tmp / "case.txt").write_text(
            f"{c.name} {c.type} {c.n} {int(ids is not None)} {c.reps} {fin} {fout}\n")
        t0 = time.time()
        try:
            res = subprocess.run([str(RUNNER), str(tmp / "case.txt")], capture_output=True,
                                 text=True, timeout=args.timeout)
            rc, text = res.returncode, res.stdout + res.stderr
        except subprocess.TimeoutExpired as e:
            rc, text = "timeout", (e.stdout or b"").decode(errors="replace") if isinstance(
                e.stdout, bytes) else (e.stdout or "")
        logs.append(f"== {c.name} rc={rc} {time.time() - t0:.2f} s\n{text}")
        print(f"{c.name}: rc={rc} {time.time() - t0:.2f} s", flush=True)
        if rc != 0 or not fout.exists():
            # exit code 1 is the reference's own abort on a CUDA API error
            # (cudaErrorInvalidValue); anything else stops the run
            if rc != 1:
                stopped = c.name
            entry["failed"] = text.strip().splitlines()[-1:] if text.strip() else [str(rc)]
            continue
        entry["ran"] = True
        entry["sync_seconds"] = [float(f.split()[-1]) for f in text.splitlines()
                                 if f.startswith(c.name + " rep ")]
        raw = np.fromfile(fout, dtype=np.uint8)
        kb = keys.nbytes
        ok = raw[:kb].view(keys.dtype)
        oi = raw[kb:].view(np.int32) if ids is not None else None
        entry["keys_sha256"] = sha(ok)
        entry["ids_sha256"] = sha(oi)
        if c.multi:
            rows = ok.reshape(-1, c.multi[0])
            entry["keys_sorted"] = bool(np.all(rows[:, 1:] >= rows[:, :-1]))
        else:
            entry["keys_sorted"] = bool(ok.size < 2 or np.all(ok[1:] >= ok[:-1]))
        if oi is not None:
            perm = bool(oi.min() >= 0 and oi.max() < oi.size
                        and np.bincount(oi, minlength=oi.size).max() == 1)
            entry["ids_permutation"] = perm
            if c.gen == "plain12m":  # ids start as the keys: they must still equal them
                entry["ids_equal_keys"] = bool(np.array_equal(oi, ok))
            else:
                entry["ids_reorder_keys"] = bool(perm and np.array_equal(keys[oi], ok))
        if keys.size <= SMALL:
            small[f"{c.name}/keys"] = ok.copy()
            if oi is not None:
                small[f"{c.name}/ids"] = oi.copy()
        for f in (fin, Path(str(fin) + ".ids"), fout):
            if f.exists():
                f.unlink()
    record["stopped_at"] = stopped
    (out / "ref_run.log").write_text("\n".join(logs))
    (out / "ref_outputs.json").write_text(json.dumps(record, indent=1, sort_keys=True) + "\n")
    np.savez_compressed(out / "ref_small.npz", **small)
    bad = [n for n, e in record["cases"].items() if not e["ran"]]
    shutil.rmtree(tmp, ignore_errors=True)
    print(f"{len(record['cases']) - len(bad)} cases recorded, not run: {bad}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
