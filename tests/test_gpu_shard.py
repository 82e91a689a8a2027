"""Z-slab sharding on one GPU with simulated ranks (each rank's work runs in
turn; no rank waits on another): the owned slabs of the box closings,
concatenated, equal the whole closing; the stitched meshes, concatenated,
hold exactly the whole mesh's triangles (bit-identical vertex positions)
and its normals (within the normal tolerance of the mesh tests)."""
import numpy as np
import pytest

from broxy_gb300 import _lib as L
from broxy_gb300 import api, shard, synth

pytestmark = pytest.mark.gpu

NORMAL_ATOL = 2e-3


def _sharded(gm_ctx, res, X, R, r, rmax, world, iters, mode):
    import torch
    desc = api.make_desc(res, bbox_min=(0.125, -0.25, 0.5), cell_size=1.0 / res)
    slabs = shard.plan_slabs(res, world, rmax, iters)
    Xv = X.view(res, res, res)
    Rv = R.view(2 * res, 2 * res, 2 * res) if R is not None else None
    owns, parts = [], []
    for s in slabs:
        Xs = Xv[s.zlo:s.zhi].contiguous().view(-1)
        Rs = Rv[2 * s.zlo:2 * s.zhi].contiguous().view(-1) if Rv is not None else None
        own, V, N, T = shard.close_mesh_slab(gm_ctx, s, desc, Xs, Rs, r, mode, 0, iters)
        owns.append(own)
        part = shard.local_mesh(s, V, N, T, desc.bbox_min[2], desc.cell_size)
        assert part["dropped"] == 0
        parts.append(part)
    torch.cuda.synchronize()
    out = shard.stitch_local(slabs, parts)
    return desc, torch.cat([o.view(-1) for o in owns]), out


def _tri_keys(V, T):
    return sorted(map(bytes, np.ascontiguousarray(V[T]).view(np.uint8).reshape(len(T), -1)))


@pytest.mark.parametrize("world,variable", [(2, False), (3, True), (4, True)])
def test_sharded_equals_whole(gm_ctx, world, variable):
    import torch
    res = 128
    X = synth.blob_grid(res, 7000 + world, count=80, device="cuda").contiguous()
    R = synth.radius_field(res, 7000, base=2, span=10, device="cuda").contiguous() if variable else None
    r, rmax = (0, 12) if variable else (5, 5)
    iters = 4
    desc, C_sh, parts = _sharded(gm_ctx, res, X, R, r, rmax, world, iters, L.GM_REF)
    C = gm_ctx.close(desc, X, R, r, L.GM_REF, L.GM_SE_SPHERE)
    V, N, T = gm_ctx.mesh(desc, C, iters)
    torch.cuda.synchronize()
    assert torch.equal(C_sh, C)
    V, N, T = V.cpu().numpy(), N.cpu().numpy(), T.view(torch.int32).cpu().numpy()
    Vs = np.concatenate([p[0] for p in parts])
    Ns = np.concatenate([p[1] for p in parts])
    Ts = np.concatenate([p[2] for p in parts])
    assert len(Vs) == len(V)
    assert _tri_keys(Vs, Ts) == _tri_keys(V, T)
    # normals by vertex position
    order_s = np.lexsort(Vs.view(np.uint32).T[::-1])
    order = np.lexsort(V.view(np.uint32).T[::-1])
    assert np.array_equal(Vs[order_s], V[order])
    np.testing.assert_allclose(Ns[order_s], N[order], atol=NORMAL_ATOL, rtol=0)
