"""Whole-grid parity at the benchmark's own sizes and inputs (the reference
path GMorpho::Load + GMorpho::Update, GMorpho/GMorpho.cu:7731-7817: the
mesh voxelized, then the GM_REF sphere closing and contour marching cubes
with 20 bilateral iterations):

* 512^3 fine grid, the 200-blob field's ~1M-triangle isosurface (seed 2000)
  voxelized, uniform radius 12; the voxelization itself equals the oracle's;
* 1024^3 fine grid, the ~4M-triangle isosurface (seed 3000) voxelized, radius
  field r = 2 + floor(30 s(x)): exactly the inputs bench.py times.

The GPU closing must equal the oracle's on every cell, the meshes must have
identical triangle index arrays, vertices within 1e-6 relative and normals
within 2e-3.  SHA-256 digests of the inputs and outputs are kept in
tests/golden/bench_manifest.json; when this run's inputs hash as recorded
there, its outputs must hash as recorded too (the same bits as the run that
wrote the manifest, which was itself checked against the oracle).

* 2048^3 resident serving grid (the ~8M-triangle isosurface, seed 5000, voxelized;
  base radius 8): after a stream of brush edits, the server's resident
  closing equals a full closing of the edited radius field (both on the GPU).
"""
import hashlib
import json
import os

import numpy as np
import pytest

from broxy_gb300 import _lib as L
from broxy_gb300 import api, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
MANIFEST = os.path.join(HERE, "golden", "bench_manifest.json")
VERT_RTOL = 1e-6
NORMAL_ATOL = 2e-3


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


CASES = {"blob_512_uniform_12": 2, "blob_1024_radius_field": 3}


@pytest.mark.parametrize("name", list(CASES))
def test_bench_config_whole_grid_equals_oracle(gm_ctx, name):
    import torch
    inp = synth.config_inputs(gm_ctx, CASES[name])
    res, desc, X, R, uniform = inp["res"], inp["desc"], inp["X"], inp["R"], inp["uniform"]
    dr = [int(v) for v in desc.data_res]
    Xh = X.cpu().numpy()
    if CASES[name] == 2:
        # the voxelization of the ~1M-triangle mesh, against the oracle's
        Xo = O.voxelize(inp["P"].cpu().numpy(), inp["T"].cpu().numpy().astype(np.uint32), res,
                        np.array(desc.bbox_min, np.float32), desc.cell_size)
        assert len(inp["T"]) > 500000
        assert np.array_equal(Xh, Xo)
    Cd = gm_ctx.close(desc, X, R, uniform, L.GM_REF, L.GM_SE_SPHERE)
    Vd, Nd, Td = gm_ctx.mesh(desc, Cd, 20)
    torch.cuda.synchronize()
    Rh = R.cpu().numpy() if R is not None else O.scale_grid(res, uniform=uniform)
    Cg, Vg, Ng, Tg = Cd.cpu().numpy(), Vd.cpu().numpy(), Nd.cpu().numpy(), Td.cpu().numpy()
    del Cd, Vd, Nd, Td
    rec = {"res": res, "seed": inp["seed"], "uniform": uniform, "variable": R is not None, "data_res": dr,
           "input_triangles": int(len(inp["T"])),
           "X": _sha(Xh), "R": _sha(Rh) if R is not None else None,
           "C": _sha(Cg), "T": _sha(Tg), "V": _sha(Vg), "nv": int(len(Vg)), "nt": int(len(Tg))}
    out = os.environ.get("GM_BENCH_MANIFEST_OUT")
    if out:
        prev = json.load(open(out)) if os.path.exists(out) else {}
        prev[name] = rec
        with open(out, "w") as f:
            json.dump(prev, f, indent=1, sort_keys=True)
    # the oracle on the whole grid
    _, _, Co = O.close(Xh, res, dr, Rh, 0, 0)
    assert np.array_equal(Cg, Co)
    Vo, To = O.mc(Co, res, np.array(desc.bbox_min), desc.cell_size)
    assert len(To) > 100000
    assert np.array_equal(Tg, To)
    np.testing.assert_allclose(Vg, Vo, rtol=VERT_RTOL, atol=0)
    No = O.normals(Vo, To, 20)
    np.testing.assert_allclose(Ng, No, atol=NORMAL_ATOL, rtol=0, equal_nan=True)
    # and the recorded digests, when the inputs are the recorded ones
    if os.path.exists(MANIFEST):
        m = json.load(open(MANIFEST)).get(name)
        if m is not None and m["X"] == rec["X"] and m["R"] == rec["R"]:
            for k in ("C", "T", "V", "nv", "nt"):
                assert m[k] == rec[k], k


def test_server_2048_edits_equal_full_closing(gm_ctx):
    import torch
    inp = synth.config_inputs(gm_ctx, 5)
    res, X, desc = inp["res"], inp["X"], inp["desc"]
    del inp
    R = torch.full(((2 * res) ** 3,), 8, dtype=torch.int8, device="cuda")
    srv = api.Server(desc, X, R, slots=4, max_crop_res=512, rmax=32, mode=L.GM_REF, bilateral_iters=0)
    rng = np.random.default_rng(5002)
    cs = 0.5 * desc.cell_size
    lo, hi = np.array(desc.bbox_min, np.float64), np.array(desc.bbox_max, np.float64)
    for i in range(32):
        c = lo + (hi - lo) * rng.uniform(0.2, 0.8, size=3)
        reach = float(rng.uniform(16, 256))
        r_new = int(rng.integers(1, 33))
        core = min(r_new, reach - 1)
        support = (core + (reach - core) * np.sqrt(1 - np.sqrt(0.5))) * cs
        srv.submit(c, r_new * cs, support, 0.0, L.GM_BRUSH_MAX if r_new >= 8 else L.GM_BRUSH_MIN)
        srv.poll()
    out = srv.drain()
    torch.cuda.synchronize()
    assert len(out) > 0 and all(r["status"] == L.GM_OK for r in out)
    resident = srv.closing().clone()
    srv.destroy()
    torch.cuda.empty_cache()
    full = gm_ctx.close(desc, X, R, 0, L.GM_REF, L.GM_SE_SPHERE)
    torch.cuda.synchronize()
    assert not torch.equal(R, torch.full_like(R, 8))  # the edits reached the field
    assert torch.equal(resident, full)
