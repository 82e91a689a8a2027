"""GPU parity of the closing (reference rows a4..a11) against the CPU oracle.

Bit-exact comparison of the packed grids: the dilation D, the dilation
contour S and the closing C, for the reference two-level algorithm (GM_REF)
and for the pure ball closing (GM_EXACT), sphere and cube dilation, uniform
and variable radius, including grids that are empty, full, and touch the
grid border.
"""
import numpy as np
import pytest

from broxy_gb300 import _lib as L
from broxy_gb300 import api, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


def _run(ctx, res, X, scale=None, uniform=4, mode=L.GM_REF, se=L.GM_SE_SPHERE, data_res=None):
    import torch
    desc = api.make_desc(res, data_res)
    Xd = _dev(X)
    Rd = _dev(scale) if scale is not None else None
    D = torch.empty_like(Xd)
    S = torch.empty_like(Xd)
    Cg = ctx.close(desc, Xd, Rd, uniform, mode, se, D=D, S=S)
    torch.cuda.synchronize()
    return D.cpu().numpy(), S.cpu().numpy(), Cg.cpu().numpy()


def _oracle(res, X, scale, uniform, mode, se, data_res=None):
    sc = scale if scale is not None else O.scale_grid(res, uniform=uniform)
    return O.close(X, res, data_res or [res] * 3, sc, mode, se)


@pytest.mark.parametrize("res,seed,r", [(16, 1, 2), (16, 2, 3), (32, 3, 4), (32, 4, 6), (64, 5, 4)])
@pytest.mark.parametrize("mode", [L.GM_REF, L.GM_EXACT])
def test_close_uniform_sphere(gm_ctx, res, seed, r, mode):
    X = synth.random_grid(res, seed)
    D, S, Cg = _run(gm_ctx, res, X, uniform=r, mode=mode)
    Do, So, Co = _oracle(res, X, None, r, mode, 0)
    assert np.array_equal(D, Do)
    assert np.array_equal(S, So)
    assert np.array_equal(Cg, Co)


@pytest.mark.parametrize("res,seed,r", [(16, 11, 2), (32, 12, 3), (32, 13, 5)])
@pytest.mark.parametrize("mode", [L.GM_REF, L.GM_EXACT])
def test_close_uniform_cube(gm_ctx, res, seed, r, mode):
    X = synth.random_grid(res, seed)
    D, S, Cg = _run(gm_ctx, res, X, uniform=r, mode=mode, se=L.GM_SE_CUBE)
    Do, So, Co = _oracle(res, X, None, r, mode, 1)
    assert np.array_equal(D, Do)
    assert np.array_equal(Cg, Co)


@pytest.mark.parametrize("mode", [L.GM_REF, L.GM_EXACT])
def test_close_large_radius(gm_ctx, mode):
    """Radii of 92 and more: the erosion's saturation 4 (r - 1)^2 no longer
    fits the packed 16-bit taps, and the wide-value passes run instead."""
    res = 32
    X = synth.random_grid(res, 31, density=0.2, blobs=3)
    D, S, Cg = _run(gm_ctx, res, X, uniform=100, mode=mode)
    Do, So, Co = _oracle(res, X, None, 100, mode, 0)
    assert np.array_equal(D, Do)
    assert np.array_equal(S, So)
    assert np.array_equal(Cg, Co)


@pytest.mark.parametrize("mode", [L.GM_REF, L.GM_EXACT])
def test_close_large_variable_radius(gm_ctx, mode):
    res = 32
    X = synth.random_grid(res, 32, density=0.2, blobs=3)
    rng = np.random.default_rng(33)
    scale = rng.integers(60, 111, size=(2 * res) ** 3).astype(np.int8)
    D, S, Cg = _run(gm_ctx, res, X, scale=scale, mode=mode)
    Do, So, Co = _oracle(res, X, scale, 0, mode, 0)
    assert np.array_equal(D, Do)
    assert np.array_equal(S, So)
    assert np.array_equal(Cg, Co)


@pytest.mark.parametrize("res,seed", [(16, 21), (32, 22), (64, 23)])
@pytest.mark.parametrize("mode", [L.GM_REF, L.GM_EXACT])
def test_close_variable_radius(gm_ctx, res, seed, mode):
    X = synth.random_grid(res, seed)
    rng = np.random.default_rng(seed)
    # radii in [-3, 9]: exercises the [2,127] clamp of the reference
    scale = rng.integers(-3, 10, size=(2 * res) ** 3).astype(np.int8)
    D, S, Cg = _run(gm_ctx, res, X, scale=scale, mode=mode)
    Do, So, Co = _oracle(res, X, scale, 0, mode, 0)
    assert np.array_equal(D, Do)
    assert np.array_equal(S, So)
    assert np.array_equal(Cg, Co)


def test_close_smooth_radius_field(gm_ctx):
    res = 32
    X = synth.blob_grid(res, 3001, count=40)
    scale = synth.radius_field(res, 3001, base=2, span=6)
    D, S, Cg = _run(gm_ctx, res, X, scale=scale)
    Do, So, Co = _oracle(res, X, scale, 0, 0, 0)
    assert np.array_equal(Cg, Co)


@pytest.mark.parametrize("fill", [0x00, 0xff])
def test_close_empty_and_full(gm_ctx, fill):
    res = 16
    X = np.full(res ** 3, fill, np.uint8)
    D, S, Cg = _run(gm_ctx, res, X, uniform=3)
    Do, So, Co = _oracle(res, X, None, 3, 0, 0)
    assert np.array_equal(D, Do) and np.array_equal(Cg, Co)


def test_close_partial_data_res(gm_ctx):
    # cells beyond data_res keep the input in the base passes (GMorpho.cu:2837-2839)
    res = 32
    X = synth.random_grid(res, 31)
    dr = [27, 30, 25]
    D, S, Cg = _run(gm_ctx, res, X, uniform=4, data_res=dr)
    Do, So, Co = _oracle(res, X, None, 4, 0, 0, data_res=dr)
    assert np.array_equal(D, Do) and np.array_equal(Cg, Co)


def test_close_touching_border(gm_ctx):
    res = 16
    N = 2 * res
    occ = np.zeros((N, N, N), bool)
    occ[:, :3, :] = True           # slab on the y = 0 face
    occ[N - 2:, N // 2, N // 2] = True  # spike reaching the z = N-1 face
    X = synth.pack_dense(occ)
    for mode in (L.GM_REF, L.GM_EXACT):
        D, S, Cg = _run(gm_ctx, res, X, uniform=3, mode=mode)
        Do, So, Co = _oracle(res, X, None, 3, mode, 0)
        assert np.array_equal(D, Do) and np.array_equal(Cg, Co)


def test_exact_mode_is_brute_force_ball_closing(gm_ctx):
    res = 16
    X = synth.random_grid(res, 41)
    sc = O.scale_grid(res, uniform=3)
    _, _, Cg = _run(gm_ctx, res, X, uniform=3, mode=L.GM_EXACT)
    assert np.array_equal(Cg, O.close_exact_brute(X, res, sc, 0))


def test_close_rejects_bad_arguments(gm_ctx):
    import torch
    desc = api.make_desc(24)  # not a power of two
    X = torch.zeros(24 ** 3, dtype=torch.uint8, device="cuda")
    with pytest.raises(L.GMError) as e:
        gm_ctx.close(desc, X, None, 4)
    assert e.value.status == L.GM_ERR_INVALID_ARGUMENT
    desc = api.make_desc(16)
    X = torch.zeros(16 ** 3 + 1, dtype=torch.uint8, device="cuda")[1:]  # misaligned
    with pytest.raises(L.GMError) as e:
        gm_ctx.close(desc, X, None, 4)
    assert e.value.status == L.GM_ERR_INVALID_ARGUMENT


def test_pyramid_matches_oracle(gm_ctx):
    import torch
    res = 32
    X = synth.random_grid(res, 51)
    rng = np.random.default_rng(51)
    scale = rng.integers(-5, 40, size=(2 * res) ** 3).astype(np.int8)
    desc = api.make_desc(res)
    pyr = gm_ctx.pyramid(desc, _dev(X), _dev(scale))
    torch.cuda.synchronize()
    got = pyr.cpu().numpy().view(np.uint64)
    assert np.array_equal(got, O.pyramid(X, res, scale))


def test_kernel_launch_counter_moves(gm_ctx):
    before = gm_ctx.kernel_launches
    _run(gm_ctx, 16, synth.random_grid(16, 61), uniform=3)
    assert gm_ctx.kernel_launches > before


def test_tma_tiles_leave_no_error_flags(gm_ctx):
    """Grids whose rows are whole 64-column boxes stage their min-plus tiles
    with TMA; after closings in every mode the kernels have recorded no
    tile-load timeout, and the grids equal the oracle's."""
    api.kernel_error_flags(clear=True)
    res = 64
    X = synth.random_grid(res, 71)
    rng = np.random.default_rng(71)
    scale = rng.integers(2, 12, size=(2 * res) ** 3).astype(np.int8)
    for mode, se in ((L.GM_REF, L.GM_SE_SPHERE), (L.GM_EXACT, L.GM_SE_SPHERE), (L.GM_REF, L.GM_SE_CUBE)):
        _, _, Co = O.close(X, res, [res] * 3, scale, mode, se)
        desc = api.make_desc(res)
        Cg = gm_ctx.close(desc, _dev(X), _dev(scale), 0, mode, se)
        assert np.array_equal(Cg.cpu().numpy(), Co), (mode, se)
    assert api.kernel_error_flags() == 0
