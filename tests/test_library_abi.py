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


def test_header_constants_match_binding():
    """Every numeric #define of include/hh_dmrg.h that the Python binding also
    names has the same value there (precision codes, error codes, array sizes
    of hh_plan_stats and hh_plan_tune)."""
    txt = open(os.path.join(ROOT, "include", "hh_dmrg.h")).read()
    defines = {}
    for name, val in re.findall(r"#define\s+(HH_[A-Z0-9_]+)\s+\(?(-?\d+)\)?", txt):
        defines[name] = int(val)
    assert len(defines) > 15
    shared = [n for n in defines if hasattr(_lib, n)]
    for n in ("HH_PREC_FP64", "HH_PREC_BF16X6", "HH_PREC_BF16X3", "HH_PREC_FP32", "HH_PREC_FP32X2",
              "HH_TILE_SHAPES", "HH_TUNE_VARIANTS", "HH_PLAN_STATS", "HH_EIG_OWN", "HH_EIG_CUSOLVER",
              "HH_ERR_INVALID", "HH_ERR_TIMEOUT"):
        assert n in shared, n
    bad = {n: (defines[n], getattr(_lib, n)) for n in shared if defines[n] != getattr(_lib, n)}
    assert not bad, bad
    assert defines["HH_TUNE_VARIANTS"] == 4 * defines["HH_TILE_SHAPES"]
