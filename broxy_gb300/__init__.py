"""broxy_gb300 — GB300-native GMorpho (voxelize -> scale-field closing ->
marching cubes) behind the reference library's API.

The compute lives in libgmorpho_gb300.so (hand-written sm_103a kernels,
C ABI in include/gmorpho_gb300.h).  ``broxy_gb300.api`` is the functional
Python binding; the reference's C++ classes are re-created in
include/gmorpho/ over the same library.
"""
from . import _lib  # noqa: F401

__all__ = ["api", "synth", "build"]
