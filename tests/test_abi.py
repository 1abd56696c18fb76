"""The C-ABI library builds, loads and exports every entry point declared in
include/ks.h; the Python binding keeps the reference's method names.  No
compute call is made (these run without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "ks.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ks_[a-z_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(ks_lib):
    lib = ctypes.CDLL(ks_lib.library_path())
    syms = header_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header(ks_lib):
    from kynema_sgf_gb300.incflo import SYMBOLS
    assert sorted(SYMBOLS) == header_symbols()


def test_reference_method_names(ks_lib):
    from kynema_sgf_gb300 import Incflo
    for m in ["InitData", "Evolve", "advance", "ApplyPredictor", "ApplyCorrector", "ApplyProjection", "compute_dt"]:
        assert callable(getattr(Incflo, m))


def test_null_handle_is_rejected(ks_lib):
    lib = ks_lib.load_library()
    assert lib.ks_init_data(None) == 6
    assert lib.ks_apply_corrector(None) == 6


def test_driver_executable_usage(ks_lib):
    """ks_run mirrors the reference executable's argument handling (no device needed)."""
    import subprocess
    from kynema_sgf_gb300 import build
    exe = build.driver_path()
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 1 and "Usage:" in r.stdout and "No input file" in r.stderr
    r = subprocess.run([exe, "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "param=value" in r.stdout
    r = subprocess.run([exe, "/nonexistent/deck.inp"], capture_output=True, text=True)
    assert r.returncode == 1 and "does not exist" in r.stderr
