"""The C-ABI library loads, exports every entry point of include/*.h, and
rejects malformed input on the host before touching a GPU."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from foamadapter_gb300 import abi, mesh

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(fvgb_\w+)\s*\(", text))
    return sorted(names)


def test_every_declared_symbol_is_exported():
    L = abi.lib()
    names = declared_functions()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_status_strings_and_version():
    assert abi.status_string(abi.OK) == "FVGB_OK"
    assert abi.status_string(abi.ERR_BREAKDOWN) == "FVGB_ERR_BREAKDOWN"
    assert abi.lib().fvgb_abi_version() >> 16 == 1


def test_mesh_create_rejects_bad_labels():
    hm = mesh.box(3, 3, 1, two_d=True)
    bad = hm.own.copy()
    bad[0] = hm.n + 5
    hm.own = bad
    d = hm.desc()
    h = C.c_void_p()
    st = abi.lib().fvgb_mesh_create(C.byref(d), C.byref(h))
    assert st == abi.ERR_INVALID_ARG
    assert b"out of range" in abi.lib().fvgb_last_error()


def test_mesh_create_rejects_duplicate_cell_pair():
    hm = mesh.box(3, 1, 1)
    hm.nei = hm.nei.copy()
    hm.own = hm.own.copy()
    # make face 1 connect the same pair as face 0
    hm.own[1], hm.nei[1] = hm.own[0], hm.nei[0]
    d = hm.desc()
    h = C.c_void_p()
    assert abi.lib().fvgb_mesh_create(C.byref(d), C.byref(h)) == abi.ERR_INVALID_ARG


def test_null_arguments_are_errors():
    L = abi.lib()
    assert L.fvgb_interp_linear(None, 1, None, None, None, None) == abi.ERR_INVALID_ARG
    assert L.fvgb_solve(None, None, None, None, None) == abi.ERR_INVALID_ARG
    assert L.fvgb_assemble(None, None, 0, 1.0, None, None, None) == abi.ERR_INVALID_ARG


def test_box_spec_validation():
    spec = abi.BoxSpec(4, 4, 2, 1, 1, 1, 0.0, 0, 1)   # 2-D with nz != 1
    sizes = (C.c_int64 * 7)()
    assert abi.lib().fvgb_box_sizes(C.byref(spec), sizes) == abi.ERR_INVALID_ARG
    spec = abi.BoxSpec(4, 4, 1, 1, 1, 1, 0.7, 0, 1)   # jitter >= 0.5 could fold cells
    assert abi.lib().fvgb_box_sizes(C.byref(spec), sizes) == abi.ERR_INVALID_ARG
