"""The reference-style C++ classes (include/gmorpho/) on the GPU: a C++
program links libgmorpho_gb300 and drives GMorpho / ScaleField / Voxelizer
like the reference viewer does; its closing must equal the C-ABI path."""
import os
import subprocess
import sys

import numpy as np
import pytest

from broxy_gb300 import _lib as L
from broxy_gb300 import synth

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def write_off(path, V, F):
    with open(path, "w") as f:
        f.write("OFF\n%d %d 0\n" % (len(V), len(F)))
        for v in V:
            f.write("%.9g %.9g %.9g\n" % tuple(v))
        for t in F:
            f.write("3 %d %d %d\n" % tuple(t))


def test_cpp_classes_drive_the_pipeline(tmp_path):
    from __graft_entry__ import build
    build()
    exe = str(tmp_path / "test_classes")
    libdir = os.path.dirname(L.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I/usr/local/cuda/include",
                    os.path.join(ROOT, "tests", "cpp", "test_classes.cpp"), "-o", exe,
                    "-L", libdir, "-lgmorpho_gb300", "-Wl,-rpath," + libdir,
                    "-L/usr/local/cuda/lib64", "-lcudart"], check=True)
    V, F = synth.spheres_mesh(seed=1000, count=8, level=2)
    off_in, off_out = str(tmp_path / "in.off"), str(tmp_path / "out.off")
    write_off(off_in, V, F)
    r = subprocess.run([exe, off_in, off_out, str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nv, t1, t2, t3, r0, r1 = (int(x) for x in r.stdout.split())
    assert nv > 0 and t1 > 0 and t2 > 0 and t3 > 0
    assert t2 != t1  # the brush changed the radius field and the mesh
    assert r0 > 0 and r1 > 0  # frame-field closings (axis-aligned, then with a constraint)
    # the frame-field closing of the class path against the CPU oracle
    from oracle import oracle as O
    res, dx, dy, dz, qres = (int(v) for v in open(tmp_path / "meta.txt").read().split())
    X = np.fromfile(tmp_path / "input.bin", np.uint8)
    Cg = np.fromfile(tmp_path / "closing.bin", np.uint8)
    R = np.fromfile(tmp_path / "scale.bin", np.int8)
    Q = np.fromfile(tmp_path / "quats.bin", np.float32).reshape(-1, 4)
    _, _, Co = O.close_rotcube(X, res, [dx, dy, dz], R, Q, qres, 0)
    assert np.array_equal(Cg, Co)


def test_contour_matches_oracle(gm_ctx):
    import torch
    from broxy_gb300 import api
    from oracle import oracle as O
    res = 32
    X = synth.random_grid(res, 171)
    desc = api.make_desc(res)
    for mode in (L.GM_REF, L.GM_EXACT):
        D, S, _ = O.close(X, res, [res] * 3, O.scale_grid(res, uniform=3), mode, 0)
        Dd = torch.as_tensor(D).cuda()
        out = gm_ctx.contour(desc, Dd, mode)
        inplace = gm_ctx.contour(desc, Dd.clone(), mode, inplace=True)
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), S)
        assert np.array_equal(inplace.cpu().numpy(), S)


def test_viewer_calls_compile_and_run(tmp_path, gm_ctx):
    """The reference viewer's own call forms (gmorpho.bbox().min(),
    2u * gmorpho.res(), Vec3i from res / 16, streaming a Vec3i, the closing
    toggles and base scale steps) compile against include/gmorpho/ and run;
    GMorpho::ErodeByBVH equals the C ABI's gm_erode_bvh on the same grids."""
    import torch
    from __graft_entry__ import build
    from broxy_gb300 import api
    build()
    exe = str(tmp_path / "test_viewer_calls")
    libdir = os.path.dirname(L.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I/usr/local/cuda/include",
                    os.path.join(ROOT, "tests", "cpp", "test_viewer_calls.cpp"), "-o", exe,
                    "-L", libdir, "-lgmorpho_gb300", "-Wl,-rpath," + libdir,
                    "-L/usr/local/cuda/lib64", "-lcudart"], check=True)
    V, F = synth.spheres_mesh(seed=1001, count=8, level=2)
    off_in = str(tmp_path / "in.off")
    write_off(off_in, V, F)
    r = subprocess.run([exe, off_in, str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    last = r.stdout.strip().splitlines()[-1].split()
    t_asym, t_sym, t_up, t_down, res, radius, no_map, dx, dy, dz = (int(v) for v in last)
    assert min(t_asym, t_sym, t_up, t_down) > 0 and no_map == 1
    assert t_down == t_sym or t_up != t_sym  # the scale steps changed the closing
    X = np.fromfile(tmp_path / "input.bin", np.uint8)
    D = np.fromfile(tmp_path / "dilation.bin", np.uint8)
    Cb = np.fromfile(tmp_path / "bvh_closing.bin", np.uint8)
    desc = api.make_desc(res, data_res=(dx, dy, dz))
    Cg = gm_ctx.erode_bvh(desc, torch.as_tensor(X).cuda(), torch.as_tensor(D).cuda(), radius)
    torch.cuda.synchronize()
    assert np.array_equal(Cg.cpu().numpy(), Cb)
