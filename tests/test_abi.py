"""CPU checks of the C ABI boundary: the library builds, loads and exports every
entry point that include/uwg.h declares; the Python binding covers them all."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "uwg.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(uwg_\w+)\s*\(", txt, re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ["uwg_ctx_create", "uwg_pic_map", "uwg_dvc_weights", "uwg_assemble", "uwg_stokes_solve",
              "uwg_rk2_advect", "uwg_update_owners", "uwg_max_dt"]:
        assert s in syms


def test_library_exports_every_declared_symbol():
    from underworld2_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    from underworld2_gb300 import _native
    missing = [s for s in declared_symbols() if s not in _native.SIGNATURES]
    assert not missing, missing
