"""The C ABI library loads and exports every symbol that
include/gmorpho_gb300.h declares (no compute: runs without a GPU)."""
import ctypes
import os
import re

from broxy_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(gm_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "gm_close" in names and "gm_mesh" in names and "gm_update" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    from __graft_entry__ import build
    build()
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    assert set(declared_functions()) <= set(_lib.PROTOTYPES)


def test_status_strings_and_version():
    lib = _lib.load()
    assert lib.gm_abi_version() == 1
    assert lib.gm_status_string(_lib.GM_ERR_INVALID_ARGUMENT) == b"invalid argument"


def test_host_only_entry_points_validate():
    lib = _lib.load()
    d = _lib.GridDesc()
    # NULL points / bad resolution are rejected without touching a GPU
    assert lib.gm_grid_attributes(None, 0, 64, 0.1, ctypes.byref(d)) == _lib.GM_ERR_INVALID_ARGUMENT
    assert lib.gm_pyramid_texels(24) == -1
    assert lib.gm_pyramid_texels(16) == 16 ** 3 + 8 ** 3 + 4 ** 3 + 8 + 1
    assert lib.gm_close(None, None, None, None, 4, 0, 0, None, None, None, None) == _lib.GM_ERR_INVALID_ARGUMENT
