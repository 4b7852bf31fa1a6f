"""The C-ABI library builds for sm_103a, loads, and exports every declared symbol.

Runs without a GPU: nvcc cross-compiles, and dlopen resolves symbols without
touching a device.
"""
import ctypes
import re

import pytest

from aerokinetic_gb300 import _native

HEADER = _native.ROOT / "include" / "aerokinetic_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(ak_[a-z_0-9]+)\s*\(", text, re.M)))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for expected in ("ak_case_create", "ak_step", "ak_diagnostics", "ak_get_pdf", "ak_last_error"):
        assert expected in names


def test_library_builds_loads_and_exports_every_symbol():
    path = _native.build()
    lib = ctypes.CDLL(str(path))
    for name in declared_functions():
        assert hasattr(lib, name), name
    loaded = _native.load()
    assert b"sm_103a" in loaded.ak_version()
    # every symbol the header declares has a ctypes signature in the loader
    assert set(declared_functions()) <= set(_native.SIGNATURES)


def test_invalid_description_is_rejected_without_a_device():
    lib = _native.load()
    desc = _native.CaseDesc()
    desc.nx = 2  # too small: rejected before any CUDA call
    handle = ctypes.c_void_p()
    code = lib.ak_case_create(ctypes.byref(desc), ctypes.byref(handle))
    assert code == _native.AK_ERR_INVALID
    assert b"nx" in lib.ak_last_error()
    with pytest.raises(ValueError):
        _native.check(code)


def test_collision_flop_count_runs_on_the_host():
    """ak_collision_flops evaluates the collision templates on a counting type
    (host code, no device): the FP64 and FP16 storage forms share the chimera
    collision, the FP32 form uses the deviation form."""
    import numpy as np
    lib = _native.load()
    counts = {}
    for storage in ("f64", "f32", "f16"):
        c = np.zeros(4)
        assert lib.ak_collision_flops(_native.STORAGE[storage], c.ctypes.data_as(ctypes.c_void_p)) == 0
        assert c[3] == c[0] + c[1] + c[2] and c[2] >= 1
        counts[storage] = c.tolist()
    assert counts["f64"] == counts["f16"] == [236.0, 213.0, 1.0, 450.0]
    assert counts["f32"][3] > counts["f64"][3]
    assert lib.ak_collision_flops(_native.STORAGE["df64"], None) == _native.AK_ERR_INVALID
