"""The C ABI library loads without a GPU and exports every entry point include/nbounce.h declares."""
import ctypes
import os
import re

from nbounce_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "nbounce.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nb_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "nb_pathtracer_dispatch" in syms and "nb_scene_create" in syms and "nb_trace_rays" in syms
    assert len(syms) >= 25


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_version_and_status_strings():
    L = _lib.lib()
    assert L.nb_version() == 100
    assert L.nb_status_string(_lib.NB_ERR_STACK_OVERFLOW) == b"NB_ERR_STACK_OVERFLOW"


def test_python_binding_covers_every_symbol():
    L = _lib.lib()
    for s in declared_symbols():
        assert getattr(L, s).argtypes is not None or getattr(L, s).restype is not None, s
