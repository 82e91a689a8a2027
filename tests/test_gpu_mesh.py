"""GPU parity of the contour marching cubes and normals (rows a12..a16),
the scale-field brush (a3), the voxelizer (a2), the layout conversion and
the host-buffer Update (a17), against the CPU oracle.

Meshes: identical vertex and triangle counts, identical triangle index
triples (connectivity and emission order), vertices within 1e-6 relative.
Normals after bilateral filtering: within 2e-3 absolute per component (the
reference accumulates them with float atomics, so their order and last
bits are not fixed; the GPU path sums in triangle order like the oracle and
differs through the fast exp and division of the bilateral weights, which
the reference's own fast-math build uses too).
"""
import numpy as np
import pytest

from broxy_gb300 import _lib as L
from broxy_gb300 import api, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

VERT_RTOL = 1e-6
NORMAL_ATOL = 2e-3


def _dev(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


def _mesh(ctx, res, Cg, iters, bbox_min=(0.0, 0.0, 0.0), cell=None):
    import torch
    desc = api.make_desc(res, bbox_min=bbox_min, cell_size=cell)
    V, N, T = ctx.mesh(desc, _dev(Cg), iters)
    torch.cuda.synchronize()
    return V.cpu().numpy(), N.cpu().numpy(), T.cpu().numpy(), desc


@pytest.mark.parametrize("res,seed", [(16, 101), (32, 102), (64, 103)])
def test_mc_matches_oracle(gm_ctx, res, seed):
    X = synth.random_grid(res, seed)
    _, _, Cg = O.close(X, res, [res] * 3, O.scale_grid(res, uniform=3), 0, 0)
    V, N, T, desc = _mesh(gm_ctx, res, Cg, 0, bbox_min=(-0.3, 0.1, 0.7), cell=0.037)
    Vo, To = O.mc(Cg, res, np.array(desc.bbox_min), desc.cell_size)
    assert V.shape == Vo.shape and T.shape == To.shape
    assert np.array_equal(T, To)
    np.testing.assert_allclose(V, Vo, rtol=VERT_RTOL, atol=0)


def test_mc_case91_slot_overwrite(gm_ctx):
    # MC case 91 (corners 0,1,3,4,6 set) holds 5 triangles but the
    # reference sizes its slot for 4: the 5th lands on the next cube's first
    # slot.  Build a grid with such cubes and compare with the oracle.
    res = 16
    N = 2 * res
    occ = np.zeros((N, N, N), bool)  # [z, y, x]
    corners = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 1)]  # v0 v1 v3 v4 v6 as (x,y,z)
    for bx in range(6, 20, 4):
        for by in range(6, 20, 4):
            for (x, y, z) in corners:
                occ[10 + z, by + y, bx + x] = True
    Cg = synth.pack_dense(occ)
    V, N_, T, desc = _mesh(gm_ctx, res, Cg, 0)
    Vo, To = O.mc(Cg, res, np.array(desc.bbox_min), desc.cell_size)
    assert np.array_equal(T, To)
    np.testing.assert_allclose(V, Vo, rtol=VERT_RTOL, atol=0)


@pytest.mark.parametrize("iters", [0, 2, 20])
def test_normals_match_oracle(gm_ctx, iters):
    res = 32
    X = synth.random_grid(res, 111)
    _, _, Cg = O.close(X, res, [res] * 3, O.scale_grid(res, uniform=3), 0, 0)
    V, N, T, desc = _mesh(gm_ctx, res, Cg, iters)
    Vo, To = O.mc(Cg, res, np.array(desc.bbox_min), desc.cell_size)
    No = O.normals(Vo, To, iters)
    np.testing.assert_allclose(N, No, atol=NORMAL_ATOL, rtol=0)


def test_normals_are_deterministic(gm_ctx):
    """Normals and bilateral filtering sum in a fixed order (per-vertex
    gathers, not the reference's float atomics, GMorpho.cu:6498-6620): two
    runs on the same grid, and a run in another context, give the same bits."""
    from broxy_gb300 import api
    res = 64
    X = synth.random_grid(res, 131)
    _, _, Cg = O.close(X, res, [res] * 3, O.scale_grid(res, uniform=4), 0, 0)
    runs = [_mesh(gm_ctx, res, Cg, 20) for _ in range(2)]
    other = api.Context(0)
    try:
        runs.append(_mesh(other, res, Cg, 20))
    finally:
        other.close_ctx()
    V0, N0, T0, _ = runs[0]
    assert len(T0) > 1000
    for V, N, T, _ in runs[1:]:
        assert np.array_equal(T, T0)
        assert V.tobytes() == V0.tobytes()
        assert N.tobytes() == N0.tobytes()


@pytest.mark.parametrize("iters", [0, 20])
def test_border_solid_matches_oracle(gm_ctx, iters):
    # A solid cut by the grid border: cubes of border cells are never
    # tagged, so the reference's triangles next to them take vertex index 0
    # for the missing edges and vertex 0 collects thousands of corners.
    res = 64
    N = 2 * res
    rng = np.random.default_rng(121)
    z, y, x = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    occ = (x + 0.3 * y < 0.7 * N) | (rng.random((N, N, N)) < 0.002)
    Cg = synth.pack_dense(occ)
    V, N_, T, desc = _mesh(gm_ctx, res, Cg, iters)
    Vo, To = O.mc(Cg, res, np.array(desc.bbox_min), desc.cell_size)
    assert np.array_equal(T, To)
    assert (To == 0).sum() > 1000
    np.testing.assert_allclose(V, Vo, rtol=VERT_RTOL, atol=0)
    No = O.normals(Vo, To, iters)
    np.testing.assert_allclose(N_, No, atol=NORMAL_ATOL, rtol=0, equal_nan=True)


def test_empty_mesh(gm_ctx):
    res = 16
    V, N, T, _ = _mesh(gm_ctx, res, np.zeros(res ** 3, np.uint8), 20)
    assert V.shape == (0, 3) and T.shape == (0, 3)


@pytest.mark.parametrize("mode", [L.GM_BRUSH_MAX, L.GM_BRUSH_MIN, L.GM_BRUSH_ZERO])
def test_scale_brush_bit_exact(gm_ctx, mode):
    import torch
    n = 48
    rng = np.random.default_rng(7 + mode)
    base = rng.integers(0, 20, size=n ** 3).astype(np.int8)
    bm = np.array([-0.2, 0.1, 0.3], np.float32)
    cell = 0.013
    pos = np.array([0.1, 0.4, 0.55], np.float32)
    R = _dev(base)
    gm_ctx.scale_brush(R, n, bm, cell, pos, 0.08, 0.21, 0.05, mode)
    torch.cuda.synchronize()
    ref = O.scale_brush(base, n, bm, cell, pos, 0.08, 0.21, 0.05, mode)
    assert np.array_equal(R.cpu().numpy(), ref)


def test_voxelize_matches_oracle(gm_ctx):
    import torch
    P, T = synth.spheres_mesh(seed=1000, count=12, level=2)
    desc = api.grid_attributes(P, 32, 0.05)
    g = gm_ctx.voxelize(desc, _dev(P), _dev(T))
    torch.cuda.synchronize()
    ref = O.voxelize(P, T, 32, np.array(desc.bbox_min), desc.cell_size)
    assert np.array_equal(g.cpu().numpy(), ref)
    assert ref.any()


def test_grid_attributes_match_oracle():
    P, _ = synth.spheres_mesh(seed=1001, count=5, level=1)
    d = api.grid_attributes(P, 64, 0.1)
    bmin, bmax, cell, dr = O.grid_attributes(P, 64, 0.1)
    assert np.array_equal(np.array(d.bbox_min, np.float32), bmin)
    assert np.float32(d.cell_size) == np.float32(cell)
    assert list(d.data_res) == list(dr)


def test_layout_roundtrip(gm_ctx):
    import torch
    res = 32
    X = _dev(synth.random_grid(res, 121))
    zw = torch.empty((2 * res) ** 3 // 32, dtype=torch.int32, device="cuda")
    gm_ctx.packed_to_zwords(res, X, zw)
    back = torch.empty_like(X)
    gm_ctx.zwords_to_packed(res, zw, back)
    torch.cuda.synchronize()
    assert torch.equal(X, back)
    # z-word bit s of column (x, y), bucket k is fine voxel z = 32k + s
    occ = synth.unpack_dense(X.cpu().numpy(), res)  # [z, y, x]
    w = zw.cpu().numpy().view(np.uint32).reshape(2 * res, 2 * res, -1)  # [y, x, k]
    z = 37
    got = (w[5, 9, z // 32] >> (z % 32)) & 1
    assert got == occ[z, 5, 9]


def test_update_host_buffers_match_oracle(gm_ctx):
    res = 32
    X = synth.random_grid(res, 131)
    desc = api.make_desc(res, cell_size=0.01)
    # global_scale 0.02 -> uniform radius floor(0.02 / 0.005) = 4
    nv, nt = gm_ctx.update(desc, X, None, 0.02, asymmetric=False, bilateral=True)
    V, N, T = gm_ctx.mesh_download(nv, nt)
    _, _, Co = O.close(X, res, [res] * 3, O.scale_grid(res, uniform=4), 0, 0)
    Vo, To = O.mc(Co, res, np.array(desc.bbox_min), desc.cell_size)
    assert np.array_equal(T, To)
    np.testing.assert_allclose(V, Vo, rtol=VERT_RTOL)
    np.testing.assert_allclose(N, O.normals(Vo, To, 20), atol=NORMAL_ATOL)


@pytest.mark.parametrize("with_field", [False, True])
def test_update_to_host_equals_update_and_download(gm_ctx, with_field):
    """The overlapped host-buffer update gives the same mesh as gm_update +
    gm_mesh_download; too small buffers answer GM_ERR_CAPACITY with the
    counts and keep the mesh on the device."""
    res = 64
    X = synth.random_grid(res, 141)
    R = np.random.default_rng(3).integers(0, 9, size=(2 * res) ** 3).astype(np.int8) if with_field else None
    desc = api.make_desc(res, cell_size=0.01)
    nv, nt = gm_ctx.update(desc, X, R, 0.02)
    V, N, T = gm_ctx.mesh_download(nv, nt)
    hV = np.zeros((nv + 5, 3), np.float32)
    hN = np.zeros((nv + 5, 3), np.float32)
    hT = np.zeros((nt + 5, 3), np.uint32)
    assert gm_ctx.update_to_host(desc, X, R, 0.02, hV, hN, hT) == (nv, nt)
    assert np.array_equal(hT[:nt], T) and np.array_equal(hV[:nv], V)
    assert np.array_equal(hN[:nv], N, equal_nan=True)  # border geometry: the reference's NaN normals
    small = np.zeros((nv - 1, 3), np.float32)
    with pytest.raises(L.GMError):
        gm_ctx.update_to_host(desc, X, R, 0.02, small, None, hT)
    V2, N2, T2 = gm_ctx.mesh_download(nv, nt)
    assert np.array_equal(T2, T)


@pytest.mark.parametrize("res,mode", [(128, L.GM_REF), (256, L.GM_REF), (256, L.GM_EXACT)])
def test_update_slab_upload_equals_close_and_mesh(gm_ctx, res, mode):
    """gm_update takes the radius field in four z slabs and runs the
    dilation's y and z passes of a slab with the radius bound of the slabs
    within 128 fine voxels of it: with radii that differ strongly from slab
    to slab, the mesh equals gm_close + gm_mesh of the same inputs (one bound
    for all)."""
    import torch
    N = 2 * res
    X = synth.blob_grid(res, 150, count=60, device="cuda").cpu().numpy()
    rng = np.random.default_rng(151)
    R = np.empty((N, N, N), np.int8)  # z, y, x
    for k, top in enumerate([30, 3, 70, 5]):
        z0, z1 = k * N // 4, (k + 1) * N // 4
        R[z0:z1] = rng.integers(0, top + 1, size=(z1 - z0, N, N), dtype=np.int8)
    R = R.reshape(-1)
    desc = api.make_desc(res, cell_size=1.0 / res)
    nv, nt = gm_ctx.update(desc, X, R, 4.0 / res, mode=mode)
    V, Nn, T = gm_ctx.mesh_download(nv, nt)
    C = gm_ctx.close(desc, torch.as_tensor(X).cuda(), torch.as_tensor(R).cuda(), 0, mode)
    V2, N2, T2 = gm_ctx.mesh(desc, C, 20)
    torch.cuda.synchronize()
    assert nt > 1000
    assert np.array_equal(T, T2.view(torch.int32).cpu().numpy().view(np.uint32))
    assert np.array_equal(V, V2.cpu().numpy())
    assert np.array_equal(Nn, N2.cpu().numpy(), equal_nan=True)


def test_update_gate_skips_morphology(gm_ctx):
    # floor(2 * gs / cell) <= 1 leaves the input unchanged (GMorpho.cu:7783)
    res = 16
    X = synth.random_grid(res, 141)
    desc = api.make_desc(res, cell_size=0.01)
    nv, nt = gm_ctx.update(desc, X, None, 0.009, bilateral=False)
    V, N, T = gm_ctx.mesh_download(nv, nt)
    Vo, To = O.mc(X, res, np.array(desc.bbox_min), desc.cell_size)
    assert np.array_equal(T, To)
