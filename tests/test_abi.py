"""The C-ABI library loads and exports every symbol its headers declare (no GPU needed)."""
import ctypes
import os
import re

import pydugks

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b([a-z_][a-z0-9_]*)\s*\(", text)) - {"if", "sizeof", "return"})


def test_library_exports_every_declared_function():
    L = ctypes.CDLL(pydugks.LIB_PATH)
    names = [n for n in declared("dugks_gb300.h") if n.startswith("dg_")]
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_headers_declare_only_c_types():
    for h in os.listdir(os.path.join(ROOT, "include")):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        assert "torch" not in text and "at::" not in text and "std::" not in text


def test_binding_signatures_cover_header():
    L = pydugks.lib()
    for n in declared("dugks_gb300.h"):
        if n.startswith("dg_"):
            assert getattr(L, n).argtypes is not None, n
