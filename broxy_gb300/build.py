"""Build recipe for libgmorpho_gb300.so (CUDA kernels + C ABI) and the CPU
oracle used by the tests.

Every translation unit is compiled by nvcc for sm_103a only, in parallel,
then linked into ``broxy_gb300/_lib/libgmorpho_gb300.so``.  Object files go
to ``_build/`` at the repository root.  No cmake, no torch extension: the
library exposes a plain C ABI (include/gmorpho_gb300.h).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(ROOT, "_build", "gmorpho")
LIBNAME = "libgmorpho_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]

SOURCES = ["morpho.cu", "mc.cu", "pyramid.cu", "scalefield.cu", "voxelize.cu", "capi.cu", "close_noalloc.cu", "bvh.cu", "batch.cu", "serve.cu", "crop.cu", "rotcube.cu", "framefield.cu"]
HOST_SOURCES = ["gmorpho_classes.cpp", "meshio.cpp"]
# The rotated-cube predicates evaluate the reference's float expressions
# without fused multiply-adds, as the CPU oracle does.
FILE_FLAGS = {"rotcube.cu": ["-fmad=false"]}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + p.stdout)
    return p.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h", ".inc"))]
    inc = os.path.join(ROOT, "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def build(verbose=False, force=False, ptxas_v=False):
    """Compile the CUDA library if any source is newer than it; return its path."""
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    nv = nvcc()
    headers = _headers()
    jobs = []
    objs = []
    for src in SOURCES + HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nv] + ARCH + NVCC_FLAGS + FILE_FLAGS.get(src, []) + (["-Xptxas", "-v"] if ptxas_v else []) + [
                "-c", s, "-o", o]
            jobs.append(cmd)
    out = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for r in ex.map(_run, jobs):
                out.append(r)
    lib = lib_path()
    if force or jobs or _stale(lib, objs):
        _run([nv] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"])
    if verbose:
        for r in out:
            if r.strip():
                print(r)
    return lib


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, ptxas_v="--ptxas" in sys.argv))
