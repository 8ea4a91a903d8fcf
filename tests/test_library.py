"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every entry point
declared in include/*.h (no compute calls here)."""
import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names.update(re.findall(r"\b(pimd_\w+)\s*\(", txt))
    return sorted(names)


def test_library_exports_every_declared_symbol(pkg):
    lib_path = pkg.build_lib.build()
    lib = ctypes.CDLL(lib_path)
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header(pkg):
    names = declared_symbols()
    assert set(names) <= set(pkg.engine.SIGNATURES), sorted(set(names) - set(pkg.engine.SIGNATURES))


def test_engine_refuses_without_device_or_bad_args(pkg):
    """Invalid parameters are rejected by pimd_create with an error code, never a crash."""
    L = pkg.engine.load()
    p = pkg.engine.make_params(dict(pot_model=7, natoms=9, box=(10, 10, 10), rc=4.0, nbeads=1))
    h = ctypes.c_void_p()
    assert L.pimd_create(ctypes.byref(h), ctypes.byref(p)) != 0
    assert not h.value
    p = pkg.engine.make_params(dict(pot_model=3, natoms=9, box=(10, 10, 10), rc=6.0, nbeads=1))
    assert L.pimd_create(ctypes.byref(h), ctypes.byref(p)) != 0


def test_nasa_tables_match_reference_source():
    """nasa_tables.h is the mechanical extraction of pot_ttm/nasa_mod.f90 (checked only where
    the reference source tree is present, named by the PIMD_REFERENCE_DIR environment variable)."""
    import subprocess
    import sys

    import pytest

    ref = os.environ.get("PIMD_REFERENCE_DIR")
    if not ref:
        pytest.skip("PIMD_REFERENCE_DIR (the reference source tree) is not set")
    src = os.path.join(ref, "pot_ttm", "nasa_mod.f90")
    if not os.path.exists(src):
        pytest.skip("reference source tree not present at PIMD_REFERENCE_DIR")
    gen = os.path.join(ROOT, "pimd-f90_gb300", "csrc", "gen_nasa_tables.py")
    out = subprocess.run([sys.executable, gen, src], capture_output=True, text=True, check=True).stdout
    with open(os.path.join(ROOT, "pimd-f90_gb300", "csrc", "nasa_tables.h")) as f:
        assert f.read() == out
