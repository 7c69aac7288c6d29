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


def test_null_handles_are_rejected(lib_path):
    """Every entry point that takes handles or buffers rejects null ones with
    HH_ERR_INVALID before any device work (hh_host_free(NULL) is a no-op, as
    free(NULL) is)."""
    lib = _lib.load(lib_path)
    skip = {"hh_init", "hh_version", "hh_status_string", "hh_last_error", "hh_host_free"}
    checked = 0
    for name, (_, args) in sorted(_lib.SIGNATURES.items()):
        if name in skip:
            continue
        codes = [getattr(a, "_type_", "P") for a in args]
        vals = [0 if isinstance(c, str) and c in "bBhHiIlLqQ" else 0.0 if c in ("f", "d") else None
                for c in codes]
        assert getattr(lib, name)(*vals) == _lib.HH_ERR_INVALID, name
        checked += 1
    assert checked > 40
    assert lib.hh_host_free(None) == 0
