"""The GB300 path against the reference's own output bytes (runs on a GPU).

The same fixture and checks as tests/test_ref_golden.py, with the CUDA path
in place of the oracle: StartSorting/Sync (turtle_start/turtle_sync) for the
sort cases and MultiSort (turtle_multisort) for the MultiSort cases.  The
full-size benchmark configurations are checked against the fixture in
tests/test_configs_gpu.py.
"""
from __future__ import annotations

import numpy as np
import pytest

from test_ref_golden import CASES, REF, check_against_reference, make_input, sha
from turtlesort_gb300 import TurtleSort

pytestmark = pytest.mark.gpu

_SORTERS: dict = {}


def _sorter(dtype, track):
    key = (np.dtype(dtype), track)
    if key not in _SORTERS:
        _SORTERS[key] = TurtleSort(dtype, 1 << 21, track_index=track)
    return _SORTERS[key]


@pytest.mark.parametrize("c", CASES, ids=lambda c: c.name)
def test_gpu_reproduces_reference_bytes(gpu, c):
    keys, ids = make_input(c)
    assert sha(keys) == REF[c.name]["input_sha256"]
    if c.multi:
        with TurtleSort(np.int32, keys.size, track_index=False) as s:
            got = keys.copy()
            s.MultiSort(c.multi[0], c.n, got, block_size=c.multi[1])
        check_against_reference(c, keys, None, got, None)
        return
    # the reference sorts `char` keys unsigned on the Arm host: same bytes as uint8
    view = np.uint8 if c.type == "i8" else keys.dtype
    if c.n <= (1 << 21):
        s = _sorter(view, ids is not None)
        k = keys.view(view).copy()
        i = ids.copy() if ids is not None else None
        s.StartSorting(k, i)
        s.Sync()
    else:
        with TurtleSort(view, c.n, track_index=ids is not None) as s:
            k = keys.view(view).copy()
            i = ids.copy() if ids is not None else None
            s.StartSorting(k, i)
            s.Sync()
    check_against_reference(c, keys, ids, k.view(keys.dtype), i)
