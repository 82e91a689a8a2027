"""The drop-in C++ headers (include/gmorpho/) and the C ABI header compile
and link without a GPU: the class test and the reference viewer's call
forms are built against libgmorpho_gb300.so here (they run in the GPU
tests)."""
import os
import subprocess

import pytest

from broxy_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("tu", ["test_classes.cpp", "test_viewer_calls.cpp"])
def test_cpp_tu_compiles_and_links(tmp_path, tu):
    from __graft_entry__ import build
    build()
    libdir = os.path.dirname(L.LIB_PATH)
    exe = str(tmp_path / tu.replace(".cpp", ""))
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"),
                        "-I/usr/local/cuda/include", os.path.join(ROOT, "tests", "cpp", tu), "-o", exe,
                        "-L", libdir, "-lgmorpho_gb300", "-Wl,-rpath," + libdir,
                        "-L/usr/local/cuda/lib64", "-lcudart"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    assert os.path.exists(exe)
