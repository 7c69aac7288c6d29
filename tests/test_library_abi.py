"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/hh_dmrg.h (no device calls: runs without a GPU)."""
import ctypes
import os
import re

from hofstadter_hubbard_tsc_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(hh_[a-z0-9_]+)\s*\(", txt))
    return names


def test_build_and_exports(lib_path):
    lib = ctypes.CDLL(lib_path)
    names = declared_symbols()
    assert len(names) > 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(lib_path):
    names = declared_symbols()
    assert names <= set(_lib.SIGNATURES), sorted(names - set(_lib.SIGNATURES))
    lib = _lib.load(lib_path)
    assert lib.hh_version() >= 100
    assert lib.hh_status_string(-4) == b"quantum number mismatch"
