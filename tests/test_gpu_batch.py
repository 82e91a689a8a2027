"""Batched closing + meshing of uneven grids: every instance must equal a
separate gm_close + gm_mesh of it, bit for bit (closing bytes, triangle
indices, vertices, filtered normals — the batch filters all its meshes in
one launch per iteration), with the lane count forced and autotuned, and on
the replay of the captured CUDA graph."""
import numpy as np
import pytest

from broxy_gb300 import _lib as L
from broxy_gb300 import api, synth

pytestmark = pytest.mark.gpu


def _instances():
    import torch
    inst = synth.batch_instances(seed=4100, count=6, lo=40, hi=120)
    for it in inst:
        it["X"] = torch.as_tensor(it["X"]).cuda()
    return inst


@pytest.mark.parametrize("lanes", [1, 3, 0, L.GM_BATCH_GROUPED])
def test_batch_equals_separate_calls(gm_ctx, lanes):
    import torch
    inst = _instances()
    items, descs = [], []
    for it in inst:
        d = api.make_desc(it["res"], it["data_res"], bbox_min=(0.1, 0.2, 0.3), cell_size=0.5 / it["res"])
        descs.append(d)
        items.append((d, it["X"], None, it["radius"], torch.empty_like(it["X"])))
    for rep in range(2):  # the second pass replays the captured graph
        meshes = gm_ctx.batch_close_mesh(items, bilateral_iters=2, lanes=lanes)
        torch.cuda.synchronize()
        got = [(items[i][4].cpu().numpy(), meshes[i][0].cpu().numpy(), meshes[i][2].cpu().numpy(),
                meshes[i][1].cpu().numpy()) for i in range(len(items))]
        for i, it in enumerate(inst):
            ref = gm_ctx.close(descs[i], it["X"], None, it["radius"])
            V, N, T = gm_ctx.mesh(descs[i], ref, 2)
            torch.cuda.synchronize()
            assert np.array_equal(got[i][0], ref.cpu().numpy())
            assert np.array_equal(got[i][2], T.cpu().numpy())
            assert np.array_equal(got[i][1], V.cpu().numpy())
            assert np.array_equal(got[i][3], N.cpu().numpy(), equal_nan=True)
    if lanes == 0:
        assert gm_ctx.batch_lanes in (1, 2, 4, 8, 16, L.GM_BATCH_GROUPED)


@pytest.mark.parametrize("lanes", [2, L.GM_BATCH_GROUPED])
def test_batch_variable_radius(gm_ctx, lanes):
    import torch
    inst = _instances()[:3]
    rng = np.random.default_rng(5)
    items, refs = [], []
    for it in inst:
        d = api.make_desc(it["res"], it["data_res"])
        R = torch.as_tensor(rng.integers(0, 9, size=(2 * it["res"]) ** 3).astype(np.int8)).cuda()
        items.append((d, it["X"], R, 0, torch.empty_like(it["X"])))
        refs.append(gm_ctx.close(d, it["X"], R, 0))
    gm_ctx.batch_close_mesh(items, mesh=False, lanes=lanes)
    torch.cuda.synchronize()
    for (d, X, R, r, out), ref in zip(items, refs):
        assert torch.equal(out, ref)


@pytest.mark.parametrize("lanes", [2, L.GM_BATCH_GROUPED])
@pytest.mark.parametrize("mode,se", [(L.GM_REF, L.GM_SE_SPHERE), (L.GM_EXACT, L.GM_SE_SPHERE),
                                     (L.GM_REF, L.GM_SE_CUBE)])
def test_batch_occupied_extent(gm_ctx, mode, se, lanes):
    """Grids closed on their occupied extent (solid in a corner of a larger
    cube, an empty grid, a grid full to its border, a radius field) equal
    the whole-grid closings and meshes."""
    import torch
    rng = np.random.default_rng(77)
    specs = [(128, synth._blob_box(128, 80, 901, 12, None), 5, None),
             (128, np.zeros(128 ** 3, np.uint8), 3, None),
             (64, synth.random_grid(64, 902), 2, None),
             (128, synth._blob_box(128, 150, 903, 20, None), 0, rng.integers(0, 13, size=256 ** 3).astype(np.int8))]
    items, descs = [], []
    for res, X, r, R in specs:
        d = api.make_desc(res, bbox_min=(0.25, -0.5, 0.125), cell_size=1.0 / res)
        Xd = torch.as_tensor(np.ascontiguousarray(X)).cuda()
        Rd = torch.as_tensor(R).cuda() if R is not None else None
        descs.append(d)
        items.append((d, Xd, Rd, r, torch.empty_like(Xd)))
    meshes = gm_ctx.batch_close_mesh(items, mode=mode, se=se, bilateral_iters=3, lanes=lanes)
    torch.cuda.synchronize()
    got = [(items[i][4].cpu().numpy(), meshes[i][0].cpu().numpy(), meshes[i][2].cpu().numpy(),
            meshes[i][1].cpu().numpy()) for i in range(len(items))]
    for i, (d, Xd, Rd, r, _) in enumerate(items):
        ref = gm_ctx.close(d, Xd, Rd, r, mode, se)
        V, N, T = gm_ctx.mesh(d, ref, 3)
        torch.cuda.synchronize()
        assert np.array_equal(got[i][0], ref.cpu().numpy())
        assert np.array_equal(got[i][2], T.cpu().numpy())
        assert np.array_equal(got[i][1], V.cpu().numpy())
        assert np.array_equal(got[i][3], N.cpu().numpy(), equal_nan=True)


@pytest.mark.parametrize("lanes", [3, L.GM_BATCH_GROUPED])
def test_batch_normals_of_large_meshes(gm_ctx, lanes):
    """Ten larger grids (over half a million vertices in all) filtered
    together, one launch per iteration: every mesh's normals equal its own
    gm_mesh filtering, bit for bit."""
    import torch
    inst = synth.batch_instances(seed=4200, count=10, lo=200, hi=300, device="cuda")
    items = []
    for it in inst:
        d = api.make_desc(it["res"], it["data_res"], cell_size=1.0 / it["res"])
        items.append((d, it["X"].contiguous(), None, it["radius"], torch.empty_like(it["X"])))
    meshes = gm_ctx.batch_close_mesh(items, bilateral_iters=5, lanes=lanes)
    torch.cuda.synchronize()
    got = [(m[0].cpu().numpy(), m[1].cpu().numpy(), m[2].cpu().numpy()) for m in meshes]
    assert sum(len(g[0]) for g in got) > 3 * 192 * 1024
    for (d, X, R, r, out), (Vb, Nb, Tb) in zip(items, got):
        V, N, T = gm_ctx.mesh(d, out, 5)
        torch.cuda.synchronize()
        assert np.array_equal(Vb, V.cpu().numpy())
        assert np.array_equal(Tb, T.cpu().numpy())
        assert np.array_equal(Nb, N.cpu().numpy(), equal_nan=True)


def test_batch_allocation_failure_injected(gm_ctx):
    """A batch whose lane buffers cannot be allocated (failure injected on
    the host) fails with GM_ERR_OUT_OF_MEMORY and leaves the context usable:
    the next batch gives the same grids as separate calls."""
    import torch
    from broxy_gb300 import _lib as L_
    items = []
    for i, res in enumerate((32, 64)):
        X = torch.as_tensor(synth.random_grid(res, 990 + i)).cuda()
        d = api.make_desc(res)
        items.append((d, X, None, 3 + i, torch.empty_like(X)))
    # a fresh context, so that its lanes have no buffers yet
    ctx = api.Context(0)
    try:
        assert L_.load().gm_batch_inject_alloc_failures(ctx.ctx, 1) == L_.GM_OK
        with pytest.raises(L_.GMError) as e:
            ctx.batch_close_mesh(items, bilateral_iters=0, lanes=2, mesh=False)
        assert e.value.status == L_.GM_ERR_OUT_OF_MEMORY
        ctx.batch_close_mesh(items, bilateral_iters=0, lanes=2, mesh=False)
        torch.cuda.synchronize()
        for d, X, R, r, out in items:
            ref = gm_ctx.close(d, X, None, r)
            torch.cuda.synchronize()
            assert torch.equal(out, ref)
    finally:
        ctx.close_ctx()


def test_batch_grouped_radius_limit(gm_ctx):
    """The grouped form takes radius bounds up to 91 (15-bit saturation
    values of its passes): above, it is refused with
    GM_ERR_INVALID_ARGUMENT, and the autotuned form closes such a batch
    with lanes, equal to separate calls."""
    import torch
    X = torch.as_tensor(synth.random_grid(64, 991)).cuda()
    d = api.make_desc(64)
    items = [(d, X, None, 100, torch.empty_like(X)), (d, X, None, 4, torch.empty_like(X))]
    with pytest.raises(L.GMError) as e:
        gm_ctx.batch_close_mesh(items, bilateral_iters=0, lanes=L.GM_BATCH_GROUPED, mesh=False)
    assert e.value.status == L.GM_ERR_INVALID_ARGUMENT
    gm_ctx.batch_close_mesh(items, bilateral_iters=0, lanes=0, mesh=False)
    torch.cuda.synchronize()
    assert gm_ctx.batch_lanes in (1, 2, 4, 8, 16)
    for dd, XX, R, r, out in items:
        assert torch.equal(out, gm_ctx.close(dd, XX, None, r))


def test_batch_grouped_allocation_failure_injected(gm_ctx):
    """The grouped form's per-grid workspaces failing to allocate (injected
    on the host) give GM_ERR_OUT_OF_MEMORY; the context stays usable."""
    import torch
    items = []
    for i, res in enumerate((32, 64)):
        X = torch.as_tensor(synth.random_grid(res, 995 + i)).cuda()
        items.append((api.make_desc(res), X, None, 2 + i, torch.empty_like(X)))
    ctx = api.Context(0)
    try:
        assert L.load().gm_batch_inject_alloc_failures(ctx.ctx, 1) == L.GM_OK
        with pytest.raises(L.GMError) as e:
            ctx.batch_close_mesh(items, bilateral_iters=0, lanes=L.GM_BATCH_GROUPED, mesh=False)
        assert e.value.status == L.GM_ERR_OUT_OF_MEMORY
        ctx.batch_close_mesh(items, bilateral_iters=0, lanes=L.GM_BATCH_GROUPED, mesh=False)
        torch.cuda.synchronize()
        for d, X, R, r, out in items:
            assert torch.equal(out, gm_ctx.close(d, X, None, r))
    finally:
        ctx.close_ctx()
