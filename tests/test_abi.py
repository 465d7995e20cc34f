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


def header_struct_fields(name):
    """(field, C type) of `typedef struct { ... } name;` in the header, in order."""
    txt = re.sub(r"/\*.*?\*/", "", open(HDR).read(), flags=re.S)
    m = re.search(r"typedef\s+struct\s*\{([^}]*)\}\s*" + name + r"\s*;", txt)
    assert m, name
    out = []
    for decl in m.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        parts = decl.replace(",", " , ").split()
        nt = 2 if parts[:2] == ["long", "long"] else 1
        ctype = " ".join(parts[:nt])
        names = [p.strip("*") for p in " ".join(parts[nt:]).split(",")]
        star = "*" in decl
        for n in names:
            out.append((n.strip().lstrip("*"), ctype + ("*" if star else "")))
    return out


def test_structs_match_header():
    """The ctypes mirrors of abd_config and abd_frame_stats have the header's fields,
    types and order (both cross the C ABI by their memory layout)."""
    import ctypes as C
    ct = {"double": C.c_double, "int": C.c_int, "long long": C.c_longlong}
    for name, mirror in (("abd_config", _lib.AbdConfig), ("abd_frame_stats", _lib.AbdFrameStats)):
        fields = header_struct_fields(name)
        assert [n for n, _ in fields] == [n for n, _ in mirror._fields_], name
        for (n, t), (_, t2) in zip(fields, mirror._fields_):
            assert ct[t] is t2, (name, n, t)
