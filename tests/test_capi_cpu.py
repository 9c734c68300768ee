"""The C ABI library on a machine without a GPU: it loads, exports every
symbol include/turtle_gb300.h declares, and its host-side logic answers
without touching a device."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import pytest

from conftest import ROOT, has_gpu

HEADER = ROOT / "include" / "turtle_gb300.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(turtle_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(native_lib):
    names = declared_functions()
    assert len(names) >= 18
    missing = [n for n in names if not hasattr(native_lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(native_lib):
    from turtlesort_gb300 import _native
    bound = {n for n, _, _ in _native.SIGNATURES}
    assert set(declared_functions()) <= bound


def test_host_side_answers(native_lib):
    assert native_lib.turtle_status_string(0) == b"ok"
    assert b"capacity" in native_lib.turtle_status_string(6)
    assert native_lib.turtle_max_elements(4, 1) == (1 << 31) - 1
    assert native_lib.turtle_max_elements(99, 1) == 0
    assert native_lib.turtle_smem_capacity(4, 1) == 8192
    assert native_lib.turtle_smem_capacity(6, 1) == 4096
    assert native_lib.turtle_max_elements(8, 1) == (1 << 31) - 1  # float32
    assert native_lib.turtle_smem_capacity(8, 1) == 8192
    assert native_lib.turtle_smem_capacity(9, 1) == 4096          # float64
    assert native_lib.turtle_max_elements(10, 1) == 0
    assert native_lib.turtle_version().startswith(b"turtle-gb300")
    # NULL handles are rejected, never dereferenced
    assert native_lib.turtle_sync(None, None) == 1
    assert native_lib.turtle_start(None, None, None, 0) == 1
    assert native_lib.turtle_destroy(None) == 0
    assert native_lib.turtle_launch_count(None) == 0


def test_create_bad_arguments(native_lib):
    h = C.c_void_p()
    assert native_lib.turtle_create(42, 10, 1, 0, -1, C.byref(h)) == 1  # bad dtype
    assert native_lib.turtle_create(4, -1, 1, 0, -1, C.byref(h)) == 1   # negative size
    assert native_lib.turtle_create(4, 1 << 40, 1, 0, -1, C.byref(h)) == 2  # too large
    assert native_lib.turtle_create(4, 1 << 31, 1, 0, -1, C.byref(h)) == 2


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_create_without_device_reports_no_device(native_lib):
    h = C.c_void_p()
    assert native_lib.turtle_create(4, 1000, 1, 0, -1, C.byref(h)) == 9
    assert not h.value


def test_python_mirror_raises_without_device(native_lib):
    if has_gpu():
        pytest.skip("checks the no-device path")
    import numpy as np
    from turtlesort_gb300 import TurtleSort, TurtleError
    with pytest.raises(TurtleError) as e:
        TurtleSort(np.int32, 1000)
    assert e.value.status == 9


def test_server_host_side_checks(native_lib):
    h = C.c_void_p()
    assert native_lib.turtle_server_create(-1, 0, 0, 0, C.byref(h)) == 1  # no budget
    assert native_lib.turtle_server_create(-1, 1 << 30, 0, 0, None) == 1
    assert native_lib.turtle_server_destroy(None) == 0
    t = C.c_uint64()
    assert native_lib.turtle_server_submit(None, 4, None, None, 0, C.byref(t)) == 1
    assert native_lib.turtle_server_drain(None) == 1
    if not has_gpu():
        assert native_lib.turtle_server_create(-1, 1 << 30, 0, 0, C.byref(h)) == 9
        assert not h.value


def test_dtype_codes_match_header():
    """The Python mirror's dtype codes are the C header's enum values."""
    import re
    import numpy as np
    from conftest import ROOT
    from turtlesort_gb300 import _native, dtype_code
    text = (ROOT / "include" / "turtle_gb300.h").read_text()
    enum = dict((m.group(1), int(m.group(2)))
                for m in re.finditer(r"TURTLE_(\w+) = (\d+)", text.split("turtle_dtype;")[0]))
    for name, dt in [("INT8", np.int8), ("UINT8", np.uint8), ("INT16", np.int16),
                     ("UINT16", np.uint16), ("INT32", np.int32), ("UINT32", np.uint32),
                     ("INT64", np.int64), ("UINT64", np.uint64), ("FLOAT32", np.float32),
                     ("FLOAT64", np.float64)]:
        assert enum[name] == getattr(_native, name) == dtype_code(dt), name
    with pytest.raises(TypeError):
        dtype_code(np.float16)
