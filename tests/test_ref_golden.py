"""The oracle against the reference's own output bytes (no GPU needed).

tests/golden/ref_outputs.json and ref_small.npz hold what the reference's own
StartSorting/Sync and MultiSort (tugrul512bit/TurtleSort, built from its
sources by oracle/ref_build.sh and run by tests/golden/make_ref_golden.py on a
GB300) produced for the cases of tests/golden/ref_cases.py.  Here the same
inputs are regenerated and the oracle's output must reproduce those bytes:

* keys: bit-identical (SHA-256 of the output, full arrays for small cases);
* ids where the reference's ids are defined: when they start equal to the
  keys (the reference README's own check, README.md:190-209) they must still
  equal them; for inputs below 8,200 keys (no merge, turtle-sort.cuh:139-163)
  the reference's ids are a permutation that reorders the keys, equal to the
  oracle's wherever the key is unique (the reference's quicksort orders equal
  keys arbitrarily, the oracle stably);
* int8: the reference's signed 8-bit key type is `char`, which is unsigned on
  the Arm GPU host, so there it sorts the bytes in unsigned order; the oracle
  must reproduce that order when given the same bytes as uint8.

The benchmark configurations at full size are compared on the GPU only
(tests/test_configs_gpu.py), against the same fixture.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

from ref_cases import cases, make_input  # noqa: E402

REF = json.loads((GOLDEN / "ref_outputs.json").read_text())["cases"]
SMALL = np.load(GOLDEN / "ref_small.npz")
CASES = [c for c in cases() if not c.full_size]


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def oracle_output(oracle_mod, c, keys, ids):
    """(keys, ids) the oracle gives for a case, as the reference's types."""
    if c.multi:
        return oracle_mod.multisort_heap(keys, c.multi[0], c.n, threads=4), None
    if c.type == "i8":  # the reference sorts `char` bytes unsigned on the Arm host
        k, i = oracle_mod.turtle_sort(keys.view(np.uint8), ids, threads=4)
        return k.view(np.int8), i
    return oracle_mod.turtle_sort(keys, ids, threads=4)


def check_against_reference(c, keys, ids, got_k, got_i):
    e = REF[c.name]
    assert e["ran"], f"{c.name}: the reference run recorded no output"
    assert sha(got_k) == e["keys_sha256"], f"{c.name}: keys differ from the reference's"
    if f"{c.name}/keys" in SMALL.files:
        assert np.array_equal(got_k, SMALL[f"{c.name}/keys"])
    if ids is None:
        return
    if c.gen == "plain12m":  # ids start equal to the keys
        assert e["ids_equal_keys"]
        assert sha(got_i) == e["ids_sha256"]
        return
    ref_i = SMALL[f"{c.name}/ids"]
    assert e["ids_permutation"] and e["ids_reorder_keys"]
    assert np.array_equal(keys[ref_i], got_k)
    # where a key occurs once, its id is forced: it must match
    uniq = np.ones(got_k.size, dtype=bool)
    same = got_k[1:] == got_k[:-1]
    uniq[1:] &= ~same
    uniq[:-1] &= ~same
    assert np.array_equal(ref_i[uniq], got_i[uniq])


def test_fixture_covers_every_case():
    names = {c.name for c in cases()}
    assert names <= set(REF), sorted(names - set(REF))
    assert all(REF[n]["ran"] for n in names)
    # the reference's keys are sorted in its own order for every case
    for c in cases():
        e = REF[c.name]
        assert e["keys_sorted"] or c.type == "i8", c.name


@pytest.mark.parametrize("c", CASES, ids=lambda c: c.name)
def test_oracle_reproduces_reference_bytes(c, oracle_mod):
    keys, ids = make_input(c)
    e = REF[c.name]
    assert sha(keys) == e["input_sha256"], "regenerated input differs from the reference's"
    got_k, got_i = oracle_output(oracle_mod, c, keys, ids)
    check_against_reference(c, keys, ids, got_k, got_i)
