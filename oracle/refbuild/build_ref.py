"""Recipe of oracle/_ref/libgmref.so: the reference GMorpho's CUDA
morphology and meshing path compiled from its own sources for sm_103a, as a
second oracle for the tests.  TEST INFRASTRUCTURE ONLY.

The reference is built from these files (paths within the reference
project): GMorpho/GMorpho.cu, Grid.cu, ScaleField.cu,
MarchingCubesMesher.cu, BVH.cu and the headers they include.  Nothing of the
reference is committed to this repository.  In the container that holds the
reference the recipe stages those files, unmodified, into oracle/_ref/src
(git-ignored, like everything under oracle/_ref/): the GPU machine that runs
the tests has no copy of the reference and cannot run x86 objects, so the
library is compiled there from the staged files.

Adaptations: the edits listed in PATCHES, applied to the staged copy, and,
outside the reference files (oracle/refbuild/shim/):
a force-included header (gmref_shim.h: __shfl -> __shfl_sync, checked
allocation and texture-object wrappers, the voxelizer's GL handle type), an
empty <eigen3/Eigen/Dense> (included, unused), a container-only
Common/Mesh.h (the original pulls in the OpenGL drawing helpers), and
stubs.cpp for the voxelizer and frame-field methods that GMorpho.cu names but
that the morphology path never calls.  The OpenGL voxelizer and the frame
field solver (cuSolver, Eigen) are not built.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
SRC = os.path.join(OUT, "src")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libgmref.so")
REFERENCE = "/root/reference"

FILES = ["GMorpho/GMorpho.cu", "GMorpho/GMorpho.h", "GMorpho/Grid.cu", "GMorpho/Grid.h", "GMorpho/ScaleField.cu",
         "GMorpho/ScaleField.h", "GMorpho/MarchingCubesMesher.cu", "GMorpho/MarchingCubesMesher.h",
         "GMorpho/BVH.cu", "GMorpho/BVH.h", "GMorpho/Voxelizer.h", "GMorpho/FrameField.h", "GMorpho/cuda_math.h",
         "GMorpho/tables.h", "GMorpho/timing.h", "Common/Vec3.h", "Common/BoundingVolume.h", "Common/Ray.h"]
# translation units: the harness compiles GMorpho.cu itself (it includes it)
UNITS = [os.path.join(HERE, "gmref_harness.cu"), "GMorpho/Grid.cu", "GMorpho/ScaleField.cu",
         "GMorpho/MarchingCubesMesher.cu", "GMorpho/BVH.cu", os.path.join(HERE, "stubs.cu")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


# Edits applied to the staged copy, each found exactly `count` times:
#  * tables.h: the triangle table holds -1 sentinels in plain `char`, which
#    is unsigned on the aarch64 host of the GPU machine (and so in its device
#    code): `!= -1` would never end the table walk of
#    createTrianglesAndVertices3D (MarchingCubesMesher.cu:1487-1497).
#  * GMorpho.cu, the persistent erosion kernels (:5349-5360 and two
#    siblings): lane 0 of each 8-lane group initialises a shared byte, the
#    group ANDs into it, lane 0 stores it.  The code relies on the lockstep
#    warps of the GPUs it was written for; a __syncwarp after the
#    initialisation and after the ANDs makes that order explicit under the
#    independent thread scheduling of current GPUs.
PATCHES = [
    ("GMorpho/tables.h", "__constant__ char triTable", "__constant__ signed char triTable", 1),
    ("GMorpho/GMorpho.cu", "\t\tif (tidr == 0) {\n\t\t\tshared_erosion_occup[tidq] = 0xff;\n\t\t}\n",
     "\t\tif (tidr == 0) {\n\t\t\tshared_erosion_occup[tidq] = 0xff;\n\t\t}\n\t\t__syncwarp ();\n", 3),
    ("GMorpho/GMorpho.cu", "\t\t\tmyAtomicAnd (&shared_erosion_occup[tidq], erosion_fine);\n",
     "\t\t\tmyAtomicAnd (&shared_erosion_occup[tidq], erosion_fine);\n\t\t__syncwarp ();\n", 3),
]


def stage():
    """Copy the reference files this build compiles into oracle/_ref/src
    (with PATCHES applied), when the reference is present; returns True when
    the staged sources are there."""
    if os.path.isdir(REFERENCE):
        for f in FILES:
            with open(os.path.join(REFERENCE, f), encoding="latin-1") as fh:
                text = fh.read()
            for (pf, old, new, count) in PATCHES:
                if pf == f:
                    if text.count(old) != count:
                        raise RuntimeError("reference patch for %s: %d matches, expected %d" % (f, text.count(old), count))
                    text = text.replace(old, new)
            dst = os.path.join(SRC, f)
            os.makedirs(os.path.dirname(dst), exist_ok=True)
            cur = open(dst, encoding="latin-1").read() if os.path.exists(dst) else None
            if cur != text:
                with open(dst, "w", encoding="latin-1") as fh:
                    fh.write(text)
    return all(os.path.exists(os.path.join(SRC, f)) for f in FILES)


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + p.stdout[-6000:])
    return p.stdout


def available():
    return os.path.exists(LIB) or stage()


def build(force=False):
    """Build oracle/_ref/libgmref.so from the staged sources; returns its
    path, or None when the sources are not available."""
    if not stage():
        return None
    os.makedirs(OBJ, exist_ok=True)
    nv = _nvcc()
    shim = os.path.join(HERE, "shim")
    deps = [os.path.join(SRC, f) for f in FILES] + [os.path.join(HERE, f) for f in os.listdir(HERE)
                                                     if f.endswith((".cu", ".h"))]
    deps += [os.path.join(shim, f) for f in ("gmref_shim.h", "Common/Mesh.h", "eigen3/Eigen/Dense")]
    flags = ARCH + ["-O2", "-std=c++17", "-w", "-Xcompiler", "-fPIC,-fopenmp", "-I" + shim, "-I" + SRC,
                    "-I" + os.path.join(SRC, "GMorpho"), "-include", os.path.join(shim, "gmref_shim.h")]
    jobs, objs = [], []
    newest = max(os.path.getmtime(d) for d in deps)
    for u in UNITS:
        src = u if os.path.isabs(u) else os.path.join(SRC, u)
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < newest:
            jobs.append([nv] + flags + ["-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or not os.path.exists(LIB):
        _run([nv] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lgomp"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
