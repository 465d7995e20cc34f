"""The C ABI library builds, loads and exports every entry point include/abd_gb300.h
declares (no GPU call is made here)."""
import os
import re

from adb_gb300 import _lib

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "abd_gb300.h")


def declared_symbols():
    txt = open(HDR).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(abd_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "abd_create" in syms and "abd_step" in syms and "abd_destroy" in syms
    assert sorted(syms) == sorted(_lib.EXPORTED)


def test_library_exports_every_declared_symbol(gpu_lib):
    for s in declared_symbols():
        assert hasattr(gpu_lib, s), s


def test_no_cpu_fallback_in_package():
    """The product package never imports the oracle."""
    pkg = os.path.join(os.path.dirname(HDR), "..", "adb_gb300")
    for root, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                src = open(os.path.join(root, f), errors="replace").read()
                assert "import oracle" not in src and "from oracle" not in src, f
