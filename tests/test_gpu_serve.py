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
    """Brush edits of two sizes: crops (rmax 8) of several edges, not only
    powers of two."""
    rng = np.random.default_rng(seed)
    cs = 0.5 / res  # fine voxel (scale-field cell)
    out = []
    for i in range(n):
        c = rng.uniform(0.25, 0.75, size=3)
        small = i % 2 == 0
        r_new = int(rng.integers(1, 5 if small else 9))
        Rb = float(rng.uniform(2, 6) if small else rng.uniform(20, 30))  # brush reach in fine voxels
        scale = r_new * cs
        support = scale + max(Rb - r_new, 1.0) * cs * np.sqrt(1 - np.sqrt(0.5))
        mode = L.GM_BRUSH_MAX if r_new >= 4 else L.GM_BRUSH_MIN
        out.append((c, scale, support, mode))
    return out


def _run(slots, edits, res=128, mode=L.GM_REF):
    import torch
    desc, X, R = _setup(res)
    srv = api.Server(desc, X, R, slots=slots, max_crop_res=96, rmax=8, mode=mode)
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
    crops = {r["crop_res"] for r in results}
    assert len(crops) >= 2 and any(c & (c - 1) for c in crops)  # several sizes, not only powers of two
    full = gm_ctx.close(desc, X, R, 0, L.GM_REF, L.GM_SE_SPHERE)
    torch.cuda.synchronize()
    assert torch.equal(C, full)
    srv.destroy()


def test_local_reclosing_exact_mode(gm_ctx):
    """The pure ball closing (GM_EXACT) served the same way: its dilation is
    the threshold of the resident distance field too."""
    import torch
    edits = _edits(128, n=8, seed=17)
    desc, X, R, C, results, srv = _run(2, edits, mode=L.GM_EXACT)
    assert all(r["status"] == L.GM_OK for r in results)
    full = gm_ctx.close(desc, X, R, 0, L.GM_EXACT, L.GM_SE_SPHERE)
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


def _case91_cubes(C, res, lo_cell, hi_cell):
    """MC cubes of value 91 with their min corner in the cell box (fine
    corner order 000,100,110,010,001,101,111,011)."""
    occ = synth.unpack_dense(C, res)  # [z, y, x]
    N = 2 * res
    o = np.zeros((N + 1,) * 3, dtype=np.uint8)
    o[:N, :N, :N] = occ
    v = np.zeros((N, N, N), dtype=np.int32)
    for bit, (dx, dy, dz) in enumerate([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0),
                                        (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]):
        v |= o[dz:dz + N, dy:dy + N, dx:dx + N].astype(np.int32) << bit
    f0, f1 = 2 * np.asarray(lo_cell), 2 * np.asarray(hi_cell)
    sub = v[f0[2]:f1[2], f0[1]:f1[1], f0[0]:f1[0]]
    return int((sub == 91).sum())


def test_patch_matches_full_mesh(gm_ctx):
    """The patch holds exactly the whole mesh's triangles emitted by the cubes
    of the dirty box, with bit-identical vertices (up to the reference's
    case-91 late write, which lands on the next triangle slot of the run)."""
    import torch
    res = 128
    desc, X, R = _setup(res, seed=305)
    srv = api.Server(desc, X, R, slots=2, max_crop_res=96, rmax=8, mode=L.GM_REF)
    c = np.array([0.5, 0.5, 0.5])
    cs = 0.5 / res
    srv.submit(c, 6 * cs, 6 * cs + 10 * cs * np.sqrt(1 - np.sqrt(0.5)), 0.0, L.GM_BRUSH_MAX)
    out = srv.drain()
    assert len(out) == 1 and out[0]["status"] == L.GM_OK
    r = out[0]
    pv = torch.as_tensor(api.DevicePtrArray(r["patch"].vertices, (r["patch"].num_vertices, 3), "<f4"), device="cuda")
    pt = torch.as_tensor(api.DevicePtrArray(r["patch"].triangles, (r["patch"].num_triangles, 3), "<u4"),
                         device="cuda")
    tri_patch = pv.cpu().numpy()[pt.view(torch.int32).cpu().numpy()]  # (k, 3, 3) corner positions
    Cres = srv.closing().clone()
    V, N, T = gm_ctx.mesh(desc, Cres, 0)
    torch.cuda.synchronize()
    tri_full = V.cpu().numpy()[T.view(torch.int32).cpu().numpy()]
    lo_cell, hi_cell = np.array(r["dirty_lo"]) // 2, np.array(r["dirty_hi"]) // 2
    # emitting cube of a triangle: floor of its smallest vertex coordinates
    # (fine units; every vertex has one non-integer coordinate, x.05 or x.95)
    cube = np.floor(tri_full.min(axis=1) / cs).astype(np.int64)
    cell = cube // 2
    sel = np.all((cell >= lo_cell) & (cell < hi_cell), axis=1)

    def keyset(t):
        from collections import Counter
        return Counter(map(bytes, np.ascontiguousarray(t.reshape(len(t), -1)).view(np.uint8).reshape(len(t), -1)))

    a, b = keyset(tri_patch), keyset(tri_full[sel])
    diff = sum(((a - b) + (b - a)).values())
    n91 = _case91_cubes(Cres.cpu().numpy(), res, lo_cell, hi_cell)
    assert len(tri_patch) > 1000
    assert diff <= 4 * n91, (diff, n91)
    srv.destroy()


def test_snapshot_restore_and_patch_export(tmp_path):
    """A server restored from a snapshot continues exactly like the original;
    a patch exports as OFF with only the vertices its triangles use."""
    import torch
    edits = _edits(128, n=6, seed=21)
    desc, X, R, C, results, srv = _run(2, edits[:3])
    Cs, Rs = srv.snapshot()
    p = tmp_path / "patch.off"
    exported = None
    for c, scale, support, mode in edits[3:]:
        srv.submit(c, scale, support, 0.0, mode)
        for r in srv.drain():
            if r["patch_triangles"] > 0:
                srv.export_patch(r, p)  # while its slot still holds it
                exported = r
    Ca = srv.closing().clone()
    desc2, X2, R2 = _setup(128)
    srv2 = api.Server(desc2, X2, R2, slots=2, max_crop_res=96, rmax=8, mode=L.GM_REF)
    srv2.restore(Cs, Rs)
    for c, scale, support, mode in edits[3:]:
        srv2.submit(c, scale, support, 0.0, mode)
    srv2.drain()
    torch.cuda.synchronize()
    assert torch.equal(srv2.closing(), Ca)
    assert torch.equal(R2, R)
    r = exported
    assert r is not None
    tok = open(p).read().split()
    nv, nf = int(tok[1]), int(tok[2])
    assert nf == r["patch_triangles"] and 0 < nv <= r["patch_vertices"]
    srv.destroy()
    srv2.destroy()


def test_admission_by_memory_failures_and_timeout(gm_ctx):
    """Admission by memory, with failures injected on the host (no GPU
    fault): allocations that fail leave their edits queued and retried; a
    budget that holds one edit at a time serialises the edits; an edit
    larger than the budget is refused; a queue timeout answers the edits
    that cannot get memory.  Every edit that ran was applied exactly: the
    resident closing equals a full closing of the edited field."""
    import torch
    edits = _edits(128, n=10, seed=11)
    desc, X, R = _setup(128)
    srv = api.Server(desc, X, R, slots=3, max_crop_res=96, rmax=8)
    inflight, budget = srv.memory()
    assert inflight == 0 and budget > 0
    # 1. the first allocations fail: the edits wait and are retried
    srv.inject_alloc_failures(3)
    results = []
    for c, scale, support, mode in edits[:5]:
        srv.submit(c, scale, support, 0.0, mode)
        results += srv.poll()
    results += srv.drain()
    assert len(results) == 5 and all(r["status"] == L.GM_OK for r in results)
    assert srv.memory()[0] == 0
    # 2. a budget that holds one edit: edits run one after the other
    one = max(1, budget // 3 // 2)
    srv.set_admission(budget_bytes=one, timeout_ms=0.0)
    results = []
    for c, scale, support, mode in edits[5:8]:
        srv.submit(c, scale, support, 0.0, mode)
        assert srv.memory()[0] <= one
        results += srv.poll()
    results += srv.drain()
    statuses = sorted(r["status"] for r in results)
    # an edit needing more than the budget is refused at once, the others run
    assert all(st in (L.GM_OK, L.GM_ERR_OUT_OF_MEMORY) for st in statuses)
    ran = [r for r in results if r["status"] == L.GM_OK]
    # 3. failures without end and a timeout: the edits are answered
    srv.set_admission(budget_bytes=budget, timeout_ms=50.0)
    srv.inject_alloc_failures(1 << 20)
    for c, scale, support, mode in edits[8:]:
        srv.submit(c, scale, support, 0.0, mode)
    timed = srv.drain()
    assert len(timed) == 2 and all(r["status"] == L.GM_ERR_OUT_OF_MEMORY for r in timed)
    srv.inject_alloc_failures(0)
    srv.set_admission(budget_bytes=budget, timeout_ms=0.0)
    # still serving
    c, scale, support, mode = edits[0]
    srv.submit(c, scale, support, 0.0, mode)
    assert all(r["status"] == L.GM_OK for r in srv.drain())
    torch.cuda.synchronize()
    full = gm_ctx.close(desc, X, R, 0, L.GM_REF, L.GM_SE_SPHERE)
    torch.cuda.synchronize()
    assert torch.equal(srv.closing(), full)
    assert srv.memory()[0] == 0
    assert len(ran) >= 1
    srv.destroy()
