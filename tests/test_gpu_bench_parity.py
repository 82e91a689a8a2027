"""Whole-grid parity at the benchmark's own sizes and inputs (the reference
path GMorpho::Update, GMorpho/GMorpho.cu:7775-7817, GM_REF sphere closing
then contour marching cubes with 20 bilateral iterations):

* 512^3 fine grid, 200-blob solid (seed 2000), uniform radius 12;
* 1024^3 fine grid, 200-blob solid and radius field r = 2 + floor(30 s(x))
  (seed 3000): exactly the inputs bench.py times.

The GPU closing must equal the oracle's on every cell, the meshes must have
identical triangle index arrays, vertices within 1e-6 relative and normals
within 2e-3.  SHA-256 digests of the inputs and outputs are kept in
tests/golden/bench_manifest.json; when this run's inputs hash as recorded
there, its outputs must hash as recorded too (the same bits as the run that
wrote the manifest, which was itself checked against the oracle).

* 2048^3 resident serving grid (seed 5000, base radius 8): after a stream of
  brush edits, the server's resident closing equals a full closing of the
  edited radius field (both on the GPU).
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


CASES = {
    "blob_512_uniform_12": dict(res=256, seed=2000, uniform=12, variable=False),
    "blob_1024_radius_field": dict(res=512, seed=3000, uniform=0, variable=True),
}


@pytest.mark.parametrize("name", list(CASES))
def test_bench_config_whole_grid_equals_oracle(gm_ctx, name):
    import torch
    c = CASES[name]
    res = c["res"]
    X = synth.blob_grid(res, c["seed"], count=200, device="cuda").contiguous()
    R = synth.radius_field(res, c["seed"], base=2, span=30, device="cuda").contiguous() if c["variable"] else None
    desc = api.make_desc(res, cell_size=1.0 / res)
    Cd = gm_ctx.close(desc, X, R, c["uniform"], L.GM_REF, L.GM_SE_SPHERE)
    Vd, Nd, Td = gm_ctx.mesh(desc, Cd, 20)
    torch.cuda.synchronize()
    Xh = X.cpu().numpy()
    Rh = R.cpu().numpy() if R is not None else O.scale_grid(res, uniform=c["uniform"])
    Cg, Vg, Ng, Tg = Cd.cpu().numpy(), Vd.cpu().numpy(), Nd.cpu().numpy(), Td.cpu().numpy()
    del Cd, Vd, Nd, Td
    rec = {"res": res, "seed": c["seed"], "uniform": c["uniform"], "variable": c["variable"],
           "X": _sha(Xh), "R": _sha(Rh) if R is not None else None,
           "C": _sha(Cg), "T": _sha(Tg), "V": _sha(Vg), "nv": int(len(Vg)), "nt": int(len(Tg))}
    out = os.environ.get("GM_BENCH_MANIFEST_OUT")
    if out:
        prev = json.load(open(out)) if os.path.exists(out) else {}
        prev[name] = rec
        with open(out, "w") as f:
            json.dump(prev, f, indent=1, sort_keys=True)
    # the oracle on the whole grid
    _, _, Co = O.close(Xh, res, [res] * 3, Rh, 0, 0)
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
    res = 1024
    X = synth.blob_grid(res, 5000, count=200, device="cuda").contiguous()
    R = torch.full(((2 * res) ** 3,), 8, dtype=torch.int8, device="cuda")
    desc = api.make_desc(res, cell_size=1.0 / res)
    srv = api.Server(desc, X, R, slots=4, max_crop_res=512, rmax=32, mode=L.GM_REF, bilateral_iters=0)
    rng = np.random.default_rng(5002)
    cs = 0.5 / res
    for i in range(32):
        c = rng.uniform(0.2, 0.8, size=3)
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
