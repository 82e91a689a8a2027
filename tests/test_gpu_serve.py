"""Edit server: after a stream of brush edits, the resident closing equals a
full closing of the edited radius field (the local re-closing is exact);
the same edits give the same grid and radius field with one slot
(sequential) and with several slots (concurrent, continuous batching); the
re-meshed patch of an edit equals the full mesh's triangles in its box."""
import numpy as np
import pytest

from broxy_gb300 import _lib as L
from broxy_gb300 import api, synth

pytestmark = pytest.mark.gpu


def _setup(res=128, seed=301):
    import torch
    X = torch.as_tensor(synth.blob_grid(res, seed, count=60)).cuda()
    R = torch.full(((2 * res) ** 3,), 4, dtype=torch.int8, device="cuda")
    desc = api.make_desc(res, cell_size=1.0 / res)
    return desc, X, R


def _edits(res, n=12, seed=7):
    rng = np.random.default_rng(seed)
    cs = 0.5 / res  # fine voxel (scale-field cell)
    out = []
    for i in range(n):
        c = rng.uniform(0.25, 0.75, size=3)
        r_new = int(rng.integers(1, 9))
        Rb = float(rng.uniform(3, 12))  # brush reach in fine voxels
        scale = r_new * cs
        support = scale + max(Rb - r_new, 1.0) * cs * np.sqrt(1 - np.sqrt(0.5))
        mode = L.GM_BRUSH_MAX if r_new >= 4 else L.GM_BRUSH_MIN
        out.append((c, scale, support, mode))
    return out


def _run(slots, edits, res=128):
    import torch
    desc, X, R = _setup(res)
    srv = api.Server(desc, X, R, slots=slots, max_crop_res=64, rmax=8, mode=L.GM_REF)
    results = []
    for c, scale, support, mode in edits:
        srv.submit(c, scale, support, 0.0, mode)
        results += srv.poll()
    results += srv.drain()
    torch.cuda.synchronize()
    C = srv.closing().clone()
    return desc, X, R, C, results, srv


def test_local_reclosing_equals_full_closing(gm_ctx):
    import torch
    edits = _edits(128)
    desc, X, R, C, results, srv = _run(3, edits)
    assert len(results) == len(edits) and all(r["status"] == L.GM_OK for r in results)
    full = gm_ctx.close(desc, X, R, 0, L.GM_REF, L.GM_SE_SPHERE)
    torch.cuda.synchronize()
    assert torch.equal(C, full)
    srv.destroy()


def test_same_alone_and_in_the_mix():
    import torch
    edits = _edits(128, seed=11)
    _, _, R1, C1, r1, s1 = _run(1, edits)
    _, _, R4, C4, r4, s4 = _run(4, edits)
    assert torch.equal(C1, C4)
    assert torch.equal(R1, R4)
    s1.destroy()
    s4.destroy()


def test_patch_matches_full_mesh(gm_ctx):
    import torch
    desc, X, R = _setup(128, seed=305)
    srv = api.Server(desc, X, R, slots=2, max_crop_res=64, rmax=8, mode=L.GM_REF)
    c = np.array([0.5, 0.5, 0.5])
    cs = 0.5 / 128
    srv.submit(c, 6 * cs, 6 * cs + 4 * cs * np.sqrt(1 - np.sqrt(0.5)), 0.0, L.GM_BRUSH_MAX)
    res = srv.drain()
    assert len(res) == 1 and res[0]["status"] == L.GM_OK
    r = res[0]
    pv = torch.as_tensor(api.DevicePtrArray(r["patch"].vertices, (r["patch"].num_vertices, 3), "<f4"), device="cuda")
    pt = torch.as_tensor(api.DevicePtrArray(r["patch"].triangles, (r["patch"].num_triangles, 3), "<u4"),
                         device="cuda")
    keep = torch.as_tensor(api.DevicePtrArray(r["patch_keep"], (r["patch"].num_triangles,), "|u1"), device="cuda")
    tri_patch = pv[pt[keep.bool()].long()].cpu().numpy()  # (k, 3, 3) triangle corner positions
    V, N, T = gm_ctx.mesh(desc, srv.closing().clone(), 0)
    torch.cuda.synchronize()
    tri_full = V[T.long()].cpu().numpy()
    lo, hi = np.array(r["dirty_lo"]), np.array(r["dirty_hi"])
    cen = tri_full.mean(1) / cs
    sel = np.all((cen >= lo) & (cen < hi), axis=1)
    def rows(t):
        m = np.round(t.reshape(len(t), -1) / cs, 3)
        return m[np.lexsort(m.T[::-1])]
    a, b = rows(tri_patch), rows(tri_full[sel])
    assert len(a) > 0 and a.shape == b.shape and np.allclose(a, b, atol=1e-3)
    srv.destroy()
