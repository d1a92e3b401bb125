"""The C-ABI library loads and exports every entry point include/kapdqmc.h declares."""
import ctypes
import re
from pathlib import Path

from kapdqmc_gb300 import _lib

HEADER = Path(__file__).resolve().parent.parent / "include" / "kapdqmc.h"


def declared():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*[\w\s\*]+?\b(kdq_\w+)\s*\(", text, re.M)))


def test_header_symbols_exported():
    lib = _lib.load()
    names = declared()
    assert "kdq_phy_update" in names and "kdq_create" in names
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_lib._SIGS), set(names) ^ set(_lib._SIGS)


def test_struct_layout_matches_header():
    # kdq_model_desc: 10 int32 (40 bytes) -> 8-aligned pointer block
    assert ctypes.sizeof(_lib.ModelDesc) == 40 + 4 * 8 + 4 * 8 + 7 * 8
    assert ctypes.sizeof(_lib.Stats) == 40


def test_create_rejects_bad_model_without_gpu_work():
    lib = _lib.load()
    h = ctypes.c_void_p()
    d = _lib.ModelDesc()
    d.kind = 7
    rc = lib.kdq_create(ctypes.byref(h), ctypes.byref(d), 1, 0)
    assert rc == _lib.KDQ_ERR_ARG
    assert b"kind" in lib.kdq_last_error(None)


def _prototypes():
    """name -> number of parameters of every kdq_ function the header declares."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    out = {}
    for m in re.finditer(r"\b(kdq_\w+)\s*\(([^;{)]*)\)\s*;", text):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_ctypes_signatures_match_header_arity():
    protos = _prototypes()
    assert set(protos) == set(_lib._SIGS), set(protos) ^ set(_lib._SIGS)
    wrong = {n: (k, len(_lib._SIGS[n][1])) for n, k in protos.items() if k != len(_lib._SIGS[n][1])}
    assert not wrong, wrong


def test_julia_binding_ccalls_match_header_arity():
    """Julia is not installed here, so its binding is checked as text: every
    ccall names a declared entry point with the header's parameter count."""
    src = (HEADER.parent.parent / "julia" / "KAPDQMCGPU" / "src" / "KAPDQMCGPU.jl").read_text()
    protos = _prototypes()
    calls = re.findall(r"ccall\(\(:(kdq_\w+),\s*libkdq\),\s*\w+,\s*\(([^()]*)\)", src, re.S)
    assert len(calls) >= 20
    for name, types in calls:
        depth, count, cur = 0, 0, ""
        for ch in types + ",":
            if ch == "{":
                depth += 1
            elif ch == "}":
                depth -= 1
            if ch == "," and depth == 0:
                count += bool(cur.strip())
                cur = ""
            else:
                cur += ch
        assert name in protos, name
        assert count == protos[name], (name, count, protos[name])
