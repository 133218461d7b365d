"""The C-ABI library builds, loads and exports every symbol include/*.h
declares; host-side argument validation fails cleanly without a GPU."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for header in (ROOT / "include").glob("*.h"):
        text = header.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(rcv_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_header_symbols_exported(rcvlib):
    names = declared_functions()
    assert len(names) >= 15
    for n in sorted(names):
        assert hasattr(rcvlib, n), f"librcv does not export {n}"


def test_binding_covers_header():
    from recursive_control_variates_gb300 import _lib

    assert declared_functions() == set(_lib.SIGNATURES)


def test_library_is_in_tree(rcvlib):
    from recursive_control_variates_gb300 import _lib

    p = Path(_lib.library_path()).resolve()
    assert ROOT in p.parents and p.name == "librcv.so"


def test_invalid_arguments_rejected_on_host(rcvlib):
    from recursive_control_variates_gb300 import _lib

    cnt = C.c_int32(0)
    rc = rcvlib.rcv_cv_step(None, 10, None, None, 0, 1, C.byref(cnt), 0.9, 0.999, 0, None)
    assert rc == _lib.RCV_ERR_INVALID
    assert b"NULL" in rcvlib.rcv_last_error()
    rc = rcvlib.rcv_loss(7, None, None, 10, None, None, None, None)
    assert rc == _lib.RCV_ERR_INVALID
    m = _lib.Medium()
    m.dims[:] = [4, 4, 4]
    rc = rcvlib.rcv_medium_prepare(C.byref(m), None)
    assert rc == _lib.RCV_ERR_INVALID
    assert b"density" in rcvlib.rcv_last_error()
    with pytest.raises(ValueError):
        _lib.check(rc, "prepare")


def test_workspace_sizes(rcvlib):
    dims = (C.c_int32 * 3)(32, 32, 32)
    n0 = rcvlib.rcv_medium_workspace_bytes(dims, 0, 0)
    n1 = rcvlib.rcv_medium_workspace_bytes(dims, 1, 0)
    n8 = rcvlib.rcv_medium_workspace_bytes(dims, 0, 8)  # 4^3 supergrid cells, two arrays
    cells = 33**3
    assert n0 >= cells * (64 + 32)
    assert n1 >= n0 + 32**3 * (32 + 16)
    assert n8 >= n0 + 2 * 4**3 * 4 and n8 <= n0 + 2 * 256
    assert n0 % 256 == 0 and n1 % 256 == 0 and n8 % 256 == 0
    bad = (C.c_int32 * 3)(0, 4, 4)
    assert rcvlib.rcv_medium_workspace_bytes(bad, 0, 0) == 0
    assert rcvlib.rcv_medium_workspace_bytes(dims, 0, -1) == 0
    assert rcvlib.rcv_loss_workspace_bytes(1000) >= 8 * 1024
