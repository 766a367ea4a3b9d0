"""The C-ABI library loads and exports every entry point declared in
include/dd_gb300.h, and the Python binding declares the same set.  No compute
calls (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"^\s*[A-Za-z_][\w \*]*?\b(dd_\w+)\s*\(", txt, flags=re.M))
    return names


def test_header_declares_entry_points():
    names = _declared()
    assert {"dd_plan_create", "dd_fft_r2c", "dd_fft_c2r", "dd_etd1", "dd_etd2rk2"} <= names


def test_library_exports_declared_symbols(dd):
    path = dd._lib.LIB_PATH
    if not os.path.isfile(path):
        pytest.fail("libdd_gb300.so not built (run __graft_entry__.build())")
    lib = ctypes.CDLL(path)
    missing = [n for n in sorted(_declared()) if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_matches_header(dd):
    assert set(dd._lib.SIGNATURES) == _declared()


def test_version_and_error_string(dd):
    L = dd._lib.lib()
    assert L.dd_version() >= 100
    assert isinstance(L.dd_last_error(), bytes)


def _arity():
    out = {}
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            for m in re.finditer(r"^\s*[A-Za-z_][\w \*]*?\b(dd_\w+)\s*\(([^)]*)\)\s*;", txt, flags=re.M):
                args = m.group(2).strip()
                out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_binding_arity_matches_header(dd):
    ar = _arity()
    bad = {n: (ar[n], len(a)) for n, a in dd._lib.SIGNATURES.items() if ar.get(n) != len(a)}
    assert not bad, bad
