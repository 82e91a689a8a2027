"""The CPU oracle of the rotated-cube dilation (GMorpho::DilateByRotCubeMipmap,
GMorpho/GMorpho.cu:3058-3230) and of the frame field system
(GMorpho/FrameFieldSparseBiharmonic.cu), checked against independent
restatements:

* the frame at a lattice point (InterpolateQuaternionField, normalize,
  rotate) against a numpy float32 transliteration: bit-exact;
* the hierarchical search against an exhaustive numpy float32 evaluation of
  the separating-axis test over every occupied fine voxel: same booleans;
* an axis-aligned field ((0, 1, 0, 0), what Generate writes without
  constraints) against the oracle's cube closing in GM_EXACT: same grids;
* the frame field solution against its defining equations, and the host
  rotation -> twist conversion of the library against the oracle's.
"""
import numpy as np
import pytest

from oracle import framefield as F
from oracle import oracle as O

f32 = np.float32


def _grid(res, seed, density=0.02, blocks=3):
    rng = np.random.default_rng(seed)
    X = np.where(rng.random((res, res, res)) < density, rng.integers(1, 256, (res, res, res)), 0).astype(np.uint8)
    for _ in range(blocks):
        lo = rng.integers(2, res - 8, 3)
        ext = rng.integers(2, 6, 3)
        X[lo[2]:lo[2] + ext[2], lo[1]:lo[1] + ext[1], lo[0]:lo[0] + ext[0]] = 0xFF
    X[:1] = 0
    X[-1:] = 0
    return X.reshape(-1)


def _field(qres, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(qres ** 3, 4)).astype(np.float32)


def _lerp(a, b, t):
    s = f32(1) - t
    return s * a + t * b


def _mul(a, b):
    ax, ay, az, aw = a
    bx, by, bz, bw = b
    w = aw * bw - ax * bx - ay * by - az * bz
    x = aw * bx + ax * bw + ay * bz - az * by
    y = aw * by - ax * bz + ay * bw + az * bx
    z = aw * bz + ax * by - ay * bx + az * bw
    return (x, y, z, w)


def frame_np(Q, qres, i, res):
    """numpy float32 transliteration of the frame (GMorpho.cu:1631-1745)."""
    fq, fr = f32(qres), f32(res)
    fx, fy, fz = (fq * (f32(v) / fr) for v in i)
    jx, jy, jz = int(fx), int(fy), int(fz)
    n = qres ** 3
    b = jx + qres * jy + qres * qres * jz

    def node(k):
        return tuple(f32(v) for v in Q[min(k, n - 1)])

    tx, ty, tz = fx - f32(jx), fy - f32(jy), fz - f32(jz)

    def lq(a, c, t):
        return tuple(_lerp(u, v, t) for u, v in zip(a, c))

    sy, sz = qres, qres * qres
    q00 = lq(node(b), node(b + 1), tx)
    q01 = lq(node(b + sz), node(b + 1 + sz), tx)
    q10 = lq(node(b + sy), node(b + 1 + sy), tx)
    q11 = lq(node(b + sy + sz), node(b + 1 + sy + sz), tx)
    q = lq(lq(q00, q10, ty), lq(q01, q11, ty), tz)
    q = (-q[0], -q[1], -q[2], q[3])
    ln = np.sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3])
    q = tuple(v / ln for v in q)
    qc = (-q[0], -q[1], -q[2], q[3])
    axes = []
    for e in ((1, 0, 0), (0, 1, 0), (0, 0, 1)):
        r = _mul(qc, _mul((f32(e[0]), f32(e[1]), f32(e[2]), f32(0)), q))
        axes.append([r[0], r[1], r[2]])
    return np.array(axes, dtype=np.float32)


def overlap_all(c, ax, se, centres, hs):
    """The 15 separating-axis tests (GMorpho.cu:241-302) of one rotated cube
    against many boxes (float32, vectorised)."""
    bx, by, bz = ax
    se, hs = f32(se), f32(hs)
    t = f32(c)[None, :] - centres
    tx, ty, tz = t[:, 0], t[:, 1], t[:, 2]
    A = np.abs
    ok = A(tx) <= hs + se * (A(bx[0]) + A(by[0]) + A(bz[0]))
    ok &= A(ty) <= hs + se * (A(bx[1]) + A(by[1]) + A(bz[1]))
    ok &= A(tz) <= hs + se * (A(bx[2]) + A(by[2]) + A(bz[2]))
    for b in (bx, by, bz):
        ok &= A(tx * b[0] + ty * b[1] + tz * b[2]) <= hs * (A(b[0]) + A(b[1]) + A(b[2])) + se
    ok &= A(tz * bx[1] - ty * bx[2]) <= hs * (A(bx[2]) + A(bx[1])) + se * (A(bz[0]) + A(by[0]))
    ok &= A(tz * by[1] - ty * by[2]) <= hs * (A(by[2]) + A(by[1])) + se * (A(bz[0]) + A(bx[0]))
    ok &= A(tz * bz[1] - ty * bz[2]) <= hs * (A(bz[2]) + A(bz[1])) + se * (A(by[0]) + A(bx[0]))
    ok &= A(tx * bx[2] - tz * bx[0]) <= hs * (A(bx[2]) + A(bx[0])) + se * (A(bz[1]) + A(by[1]))
    ok &= A(tx * by[2] - tz * by[0]) <= hs * (A(by[2]) + A(by[0])) + se * (A(bz[1]) + A(bx[1]))
    ok &= A(tx * bz[2] - tz * bz[0]) <= hs * (A(bz[2]) + A(bz[0])) + se * (A(by[1]) + A(bx[1]))
    ok &= A(ty * bx[0] - tx * bx[1]) <= hs * (A(bx[1]) + A(bx[0])) + se * (A(bz[2]) + A(by[2]))
    ok &= A(ty * by[0] - tx * by[1]) <= hs * (A(by[1]) + A(by[0])) + se * (A(bz[2]) + A(bx[2]))
    ok &= A(ty * bz[0] - tx * bz[1]) <= hs * (A(bz[1]) + A(bz[0])) + se * (A(by[2]) + A(bx[2]))
    return ok


def _fine_voxels(X, res):
    g = X.reshape(res, res, res)
    z, y, x = np.nonzero(g)
    pts = []
    for k in range(8):
        m = (g[z, y, x] >> k) & 1
        pts.append(np.stack([2 * x[m == 1] + (k & 1), 2 * y[m == 1] + ((k >> 1) & 1), 2 * z[m == 1] + (k >> 2)], 1))
    return np.concatenate(pts).astype(np.float32)


@pytest.mark.parametrize("qres", [2, 3, 5])
def test_frame_matches_float32_transliteration(qres):
    Q = _field(qres, 700 + qres)
    rng = np.random.default_rng(qres)
    for res in (16, 32, 64):
        for _ in range(40):
            i = rng.integers(0, res, 3)
            got = O.rotcube_frame(Q, qres, i, res)
            want = frame_np(Q, qres, i, res)
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (res, i)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_search_matches_exhaustive_overlap(seed):
    res = 16
    X = _grid(res, 7300 + seed)
    Q = _field(3, seed)
    scale = O.scale_grid(res, uniform=2)
    pyr = O.pyramid(X, res, scale)
    leaves = _fine_voxels(X, res) + f32(0.5)
    rng = np.random.default_rng(seed)
    L = O.lib()
    qp = Q.reshape(-1)
    hits = 0
    for _ in range(300):
        p = rng.integers(0, 2 * res, 3)
        r = int(rng.integers(2, 7))
        ax = O.rotcube_frame(Q, 3, p, 2 * res)
        want = bool(overlap_all(p.astype(np.float32), ax, r, leaves, 0.5).any())
        got = bool(L.gmo_rotcube_query(O._p(pyr, O._u64p), res, O._p(qp, O._f32p), 3, int(p[0]), int(p[1]),
                                        int(p[2]), 2 * res, int(p[0]), int(p[1]), int(p[2]), r))
        assert got == want, (p, r)
        hits += got
    assert 0 < hits < 300


@pytest.mark.parametrize("uniform", [2, 4])
def test_axis_aligned_field_is_the_cube_closing(uniform):
    """The per-voxel predicate of an axis-aligned frame is the cube's closed
    box overlap, so GM_EXACT agrees with the cube closing.  (GM_REF differs
    by design: the rotated-cube path refines the conservative contour of
    GMorpho/Grid.cu:1464-1498, the cube path the tight one.)"""
    res = 32
    X = _grid(res, 7400 + uniform)
    scale = O.scale_grid(res, uniform=uniform)
    Q = np.tile(np.array([0, 1, 0, 0], np.float32), (8, 1))
    D, S, C = O.close_rotcube(X, res, [res] * 3, scale, Q, 2, 1)
    D2, S2, C2 = O.close(X, res, [res] * 3, scale, 1, 1)
    assert np.array_equal(D, D2) and np.array_equal(C, C2)
    assert C.any()
    Dr, _, Cr = O.close_rotcube(X, res, [res] * 3, scale, Q, 2, 0)
    assert not np.any(X & ~Cr)


def test_rotated_field_differs_from_cube_and_is_monotone():
    res = 32
    X = _grid(res, 7500)
    scale = O.scale_grid(res, uniform=4)
    ang = 0.6
    Q = np.tile(np.array([0, 0, np.sin(ang / 2), np.cos(ang / 2)], np.float32), (8, 1))
    D, _, C = O.close_rotcube(X, res, [res] * 3, scale, Q, 2, 0)
    Dc, _, _ = O.close(X, res, [res] * 3, scale, 0, 1)
    assert not np.array_equal(D, Dc)
    # extensive: the dilation and the closing contain the input
    assert not np.any(X & ~D)
    assert not np.any(X & ~C)


def test_frame_field_oracle_solves_its_system():
    res = 8
    pts = [((0.3, 0.4, 0.5), (0.5, 0.2, 0.1)), ((0.8, 0.1, 0.6), (0.0, 0.0, 1.0)), ((0.1, 0.9, 0.2), (0.0, 0.0, 0.0))]
    q = F.generate(res, (0, 0, 0), (1, 1, 1), pts).astype(np.float64)
    nodes, b = [], np.zeros((res ** 3, 4))
    for pos, tw in pts:
        g = F.lattice_position(pos, (0, 0, 0), (1, 1, 1), res)
        c = g[0] + res * g[1] + res * res * g[2]
        nodes.append(c)
        b[c] = F.twist_quat(tw)
    A = F.system(res, nodes)
    assert np.abs(A @ q - b).max() < 1e-5
    # a zero twist is the identity quaternion
    assert np.array_equal(F.twist_quat((0, 0, 0)), np.array([0, 0, 0, 1], np.float32))


def test_rotation_to_twist_matches_oracle():
    from broxy_gb300 import api
    rng = np.random.default_rng(5)
    for _ in range(50):
        v = rng.normal(size=3)
        v = v / np.linalg.norm(v) * rng.uniform(0.05, 3.0)
        th = np.linalg.norm(v)
        k = v / th
        K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
        R = np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K
        got = np.array(api.rotation_to_twist(R[:, 0], R[:, 1], R[:, 2]))
        want = F.rotation_to_twist(R[:, 0].astype(np.float32), R[:, 1].astype(np.float32), R[:, 2].astype(np.float32))
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-5)
        np.testing.assert_allclose(got, v, rtol=1e-4, atol=1e-4)
