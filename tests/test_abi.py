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


def test_zcontract_split_rule_covers_k_exactly():
    """The K split of the FP64 contraction (host arithmetic of the library):
    chunks are multiples of the K step, cover [0, K) exactly, number about
    304 CTAs in all, and only skinny outputs with a long K are split."""
    import ctypes
    from pytreenet_gb300 import _lib
    lib = _lib.load()
    chunk = ctypes.c_int64()
    for tiles in (1, 2, 3, 7, 38, 39, 400):
        for K in (1, 64, 2047, 2048, 4550, 65536, 10 ** 6 + 3):
            s = int(lib.ptn_zcontract_splits(tiles, K, ctypes.byref(chunk)))
            c = chunk.value
            if tiles > 38 or K < 2048:
                assert s == 1 and c == K
                continue
            assert s >= 1 and (s == 1 or c % 8 == 0)
            assert (s - 1) * c < K <= s * c
            assert tiles * s <= 304 + tiles
            assert s == 1 or c >= 256 - 8
