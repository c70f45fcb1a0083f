"""The C-ABI library loads and exports every entry point declared in
include/gbchol.h (no GPU calls)."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(gbchol_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_functions():
    names = declared_functions()
    assert "gbchol_solve" in names and "gbchol_create" in names
    assert len(names) >= 12


@pytest.mark.parametrize("name", declared_functions())
def test_symbol_exported(gblib, name):
    assert hasattr(gblib, name), name


def test_version_and_error(gblib):
    from cholespy_gb300 import _ffi
    assert b"sm_103a" in gblib.gbchol_version()
    assert _ffi.last_error() == "" or isinstance(_ffi.last_error(), str)


def test_entry_points_reject_bad_arguments_before_gpu_work(gblib):
    """Argument checks that run on the host before any CUDA call: a null
    handle, batch options out of range and an empty batch are refused with
    GBCHOL_EINVAL and a message, on a machine without a GPU."""
    import ctypes as C

    from cholespy_gb300 import _ffi
    lib = _ffi.lib()
    out = C.c_void_p()
    assert lib.gbchol_solve(None, 0, 4, None, None, None) == _ffi.EINVAL
    assert lib.gbchol_solve_noalloc(None, 0, 4, None, None, None) == _ffi.EINVAL
    assert "handle" in _ffi.last_error().lower()
    assert lib.gbchol_batch_create_ex(1, None, None, 0, None, C.byref(out)) == _ffi.EINVAL
    assert "options" in _ffi.last_error()
    for group, skew, variant in ((8 << 20, -1, 2), (8 << 20, 4, 3), (8 << 20, 4, 0)):
        o = _ffi.BatchOptions(group, skew, variant)
        assert lib.gbchol_batch_create_ex(1, None, None, 0, C.byref(o), C.byref(out)) == _ffi.EINVAL
        assert "skew" in _ffi.last_error()
    o = _ffi.BatchOptions(8 << 20, 4, 2)
    assert lib.gbchol_batch_create_ex(0, None, None, 0, C.byref(o), C.byref(out)) == _ffi.EINVAL
    assert "at least one solver" in _ffi.last_error()
    assert not out.value
