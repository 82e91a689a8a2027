"""BVH (reference row a18): build over the set voxels of a packed grid,
exact radius queries and the ErodeByBVH predicate, against numpy brute
force; leaves come out in Morton order."""
import numpy as np
import pytest

from broxy_gb300 import api, synth

pytestmark = pytest.mark.gpu


def morton64(x, y, z):
    m = np.zeros_like(x, dtype=np.uint64)
    for b in range(21):
        m |= ((x >> b) & 1).astype(np.uint64) << np.uint64(3 * b)
        m |= ((y >> b) & 1).astype(np.uint64) << np.uint64(3 * b + 1)
        m |= ((z >> b) & 1).astype(np.uint64) << np.uint64(3 * b + 2)
    return m


@pytest.mark.parametrize("res,seed,radius", [(16, 201, 3), (32, 202, 5), (32, 203, 1)])
def test_bvh_query_matches_brute_force(gm_ctx, res, seed, radius):
    import torch
    rng = np.random.default_rng(seed)
    N = 2 * res
    occ = rng.random((N, N, N)) < 0.002  # sparse sites
    grid = synth.pack_dense(occ)
    desc = api.make_desc(res)
    bvh = gm_ctx.bvh_build(desc, torch.as_tensor(grid).cuda())
    zz, yy, xx = np.nonzero(occ)
    assert bvh.n == len(xx)
    keys = bvh.leaves().cpu().numpy().view(np.uint64)
    assert np.array_equal(keys, np.sort(morton64(xx, yy, zz)))
    q = rng.integers(0, 2 * N + 1, size=(4000, 3)).astype(np.int32)
    hits = bvh.query(torch.as_tensor(q).cuda(), radius).cpu().numpy()
    centres = np.stack([2 * xx + 1, 2 * yy + 1, 2 * zz + 1], 1)
    d2 = ((q[:, None, :] - centres[None, :, :]) ** 2).sum(-1)
    ref = (d2 < 4 * radius * radius).any(1)
    assert np.array_equal(hits.astype(bool), ref)
    bvh.destroy()


def test_bvh_empty_and_single(gm_ctx):
    import torch
    res = 16
    desc = api.make_desc(res)
    g = torch.zeros(res ** 3, dtype=torch.uint8, device="cuda")
    bvh = gm_ctx.bvh_build(desc, g)
    assert bvh.n == 0
    q = torch.zeros((5, 3), dtype=torch.int32, device="cuda")
    assert bvh.query(q, 4).sum().item() == 0
    g[0] = 1
    bvh1 = gm_ctx.bvh_build(desc, g)
    assert bvh1.n == 1
    q = torch.tensor([[1, 1, 1], [9, 1, 1]], dtype=torch.int32, device="cuda")
    assert bvh1.query(q, 2).cpu().tolist() == [1, 0]


def test_erode_bvh_matches_brute_force(gm_ctx):
    import torch
    from oracle import oracle as O
    res = 16
    X = synth.random_grid(res, 211)
    D, S, _ = O.close(X, res, [res] * 3, O.scale_grid(res, uniform=3), 0, 0)
    radius = 3
    desc = api.make_desc(res)
    Cg = gm_ctx.erode_bvh(desc, torch.as_tensor(X).cuda(), torch.as_tensor(D).cuda(), radius)
    torch.cuda.synchronize()
    Ds, Ss, Xs = synth.unpack_dense(D, res), synth.unpack_dense(S, res), X.reshape(res, res, res)
    sz, sy, sx = np.nonzero(Ss)
    centres = np.stack([sx, sy, sz], 1)
    ref = Ds.copy()
    for z, y, x in zip(*np.nonzero(Ds)):
        c = (x // 2) + res * (y // 2) + res * res * (z // 2)
        if X[c] == 0xff:
            continue
        if (((centres - np.array([x, y, z])) ** 2).sum(1) < radius * radius).any():
            ref[z, y, x] = False
    assert np.array_equal(Cg.cpu().numpy(), synth.pack_dense(ref))
