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
