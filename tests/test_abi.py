"""The C-ABI library loads and exports every entry point declared in include/ptn_gb300.h."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ptn_gb300.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ptn_\w+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared()
    assert "ptn_zcontract" in names and "ptn_zqr_keep" in names


def test_library_exports_all_declared_symbols():
    from pytreenet_gb300 import build
    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_signatures_cover_header():
    from pytreenet_gb300 import _lib
    assert set(declared()) <= set(_lib.SIGNATURES)
