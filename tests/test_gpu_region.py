"""Closing on a region of a box (gm_close_box_region): the cells of the
region are bit-identical to the whole box's closing, whatever the workspace
held before (the passes skip the tiles that cannot reach the region and
leave stale bytes there), for both modes, sphere and cube dilation, uniform
and variable radius, and regions touching every side of the box."""
import numpy as np
import pytest

from broxy_gb300 import _lib as L
from broxy_gb300 import api, synth

pytestmark = pytest.mark.gpu

RES = 128
DIMS = (128, 96, 80)  # x, y, z cells: a box cut out of a 128^3 grid


def _box_inputs(seed, variable):
    X = synth.blob_grid(RES, seed, count=120, device="cuda").view(RES, RES, RES)
    Xb = X[:DIMS[2], :DIMS[1], :DIMS[0]].contiguous()
    Rb = None
    if variable:
        n = 2 * RES
        R = synth.radius_field(RES, seed, base=2, span=20, device="cuda").view(n, n, n)
        Rb = R[:2 * DIMS[2], :2 * DIMS[1], :2 * DIMS[0]].contiguous()
    return Xb, Rb


REGIONS = [
    ((0, 0, 0), DIMS),                        # the whole box
    ((40, 30, 20), (72, 50, 44)),             # interior
    ((0, 0, 0), (17, 9, 33)),                 # low corner
    ((100, 70, 60), DIMS),                    # high corner
    ((64, 48, 40), (65, 49, 41)),             # one cell
    ((0, 10, 77), (128, 20, 80)),             # thin slab on the top z side
    ((3, 0, 0), (9, 96, 80)),                 # thin slab across y and z
]


@pytest.mark.parametrize("variable", [False, True])
@pytest.mark.parametrize("mode", [L.GM_REF, L.GM_EXACT])
def test_region_equals_whole_box(gm_ctx, variable, mode):
    import torch
    box = api.make_box(DIMS)
    X, R = _box_inputs(9100 + int(variable), variable)
    C = gm_ctx.close_box(box, X, R, 9, mode, L.GM_SE_SPHERE)
    # unrelated closing first: the workspace holds another grid's values
    X2, R2 = _box_inputs(9200, variable)
    for lo, hi in REGIONS:
        gm_ctx.close_box(box, X2, R2, 9, mode, L.GM_SE_SPHERE)
        out = torch.full_like(X, 0x5A)
        Cr = gm_ctx.close_box_region(box, X, lo, hi, R, 9, mode, L.GM_SE_SPHERE, out=out)
        torch.cuda.synchronize()
        sl = (slice(lo[2], hi[2]), slice(lo[1], hi[1]), slice(lo[0], hi[0]))
        assert torch.equal(Cr[sl], C[sl]), (lo, hi)


def test_region_cube_dilation(gm_ctx):
    import torch
    box = api.make_box(DIMS)
    X, _ = _box_inputs(9300, False)
    C = gm_ctx.close_box(box, X, None, 7, L.GM_REF, L.GM_SE_CUBE)
    lo, hi = (20, 20, 20), (60, 40, 52)
    Cr = gm_ctx.close_box_region(box, X, lo, hi, None, 7, L.GM_REF, L.GM_SE_CUBE)
    torch.cuda.synchronize()
    sl = (slice(lo[2], hi[2]), slice(lo[1], hi[1]), slice(lo[0], hi[0]))
    assert torch.equal(Cr[sl], C[sl])


def test_region_rejects_bad_regions(gm_ctx):
    import torch
    box = api.make_box(DIMS)
    X, _ = _box_inputs(9400, False)
    for lo, hi in [((0, 0, 0), (0, 5, 5)), ((-1, 0, 0), (5, 5, 5)), ((0, 0, 0), (129, 5, 5)),
                   ((5, 5, 5), (4, 9, 9))]:
        with pytest.raises(L.GMError):
            gm_ctx.close_box_region(box, X, lo, hi, None, 4)
    torch.cuda.synchronize()


def _swap_xz_bytes(C, dims):
    """Box bytes (z, y, x) -> the box with x and z exchanged, bits moved
    from x + 2y + 4z to z + 2y + 4x."""
    import torch
    lut = torch.zeros(256, dtype=torch.uint8)
    for v in range(256):
        o = 0
        for k in range(8):
            if v >> k & 1:
                x, y, z = k & 1, k >> 1 & 1, k >> 2 & 1
                o |= 1 << (z + 2 * y + 4 * x)
        lut[v] = o
    B = C.view(dims[2], dims[1], dims[0]).permute(2, 1, 0).contiguous()
    return lut.to(C.device)[B.long()].view(-1)


@pytest.mark.parametrize("mode", [L.GM_REF, L.GM_EXACT])
@pytest.mark.parametrize("rx", [1024, 2048])
def test_long_rows_equal_transposed_box(gm_ctx, mode, rx):
    """Rows of 2048 fine voxels (two 32-bit words per lane in the x passes)
    and of 4096 (the block-per-row x passes) against the same grid with x and
    z exchanged (short rows): the closing commutes with the exchange."""
    import torch
    long_dims, short_dims = (rx, 32, 32), (32, 32, rx)
    g = torch.Generator().manual_seed(9500)
    X = torch.zeros(long_dims[2], long_dims[1], long_dims[0], dtype=torch.uint8)
    # random blocks and sparse voxels away from the y / z borders
    X[6:26, 6:26, :] = torch.where(torch.rand(20, 20, rx, generator=g) < 0.08,
                                   torch.randint(0, 256, (20, 20, rx), generator=g, dtype=torch.uint8),
                                   torch.zeros(20, 20, rx, dtype=torch.uint8))
    X[10:20, 12:18, 100:180] = 0xFF
    X[8:24, 8:24, 700:705] = 0xFF
    X[9:22, 7:25, rx - 40:rx - 30] = 0xFF
    X = X.view(-1).cuda()
    Xt = _swap_xz_bytes(X, long_dims)
    C_long = gm_ctx.close_box(api.make_box(long_dims), X, None, 5, mode, L.GM_SE_SPHERE)
    C_short = gm_ctx.close_box(api.make_box(short_dims), Xt, None, 5, mode, L.GM_SE_SPHERE)
    torch.cuda.synchronize()
    assert C_long.sum().item() > 0
    assert torch.equal(_swap_xz_bytes(C_long, long_dims), C_short)
