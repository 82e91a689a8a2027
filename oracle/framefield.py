"""CPU restatement of the frame field's biharmonic quaternion system.

TEST INFRASTRUCTURE ONLY: used by tests/ to check gm_frame_field_generate;
the product never imports it.

Follows GMorpho/FrameFieldSparseBiharmonic.cu:
  * BuildSparseLTLMatrix (:170-312): L, row i = 1 on the diagonal and
    -(1 / deg(i)) on each in-bounds 6-neighbour, entries in float32;
  * BuildSparseSMatrix / BuildSparseBiharmonicSystem (:314-424): S = 1 on
    the diagonal of every hard-constrained node, A = L^T L + S;
  * SolveSparseBiharmonicSystem (:449-647): per component k, b_k = the
    constraint quaternion's component at its node (the last point on a node
    wins), A q_k = b_k;
  * FrameField::AddHardConstrainedPoint (GMorpho/FrameField.cu:64-77) and
    the twist -> quaternion conversion (:487-503 of the solver file).
The reference factors A in float (cusolverSp Cholesky); this oracle solves
it exactly in double (scipy's sparse LU), so it checks the GPU solver's
convergence, not the reference's float rounding: parity unpinned.
"""
import math

import numpy as np


def lattice_position(position, bbox_min, bbox_max, res):
    f32 = np.float32
    ext = [abs(f32(bbox_max[i]) - f32(bbox_min[i])) for i in range(3)]
    cell = f32(max(ext[0], max(ext[1], ext[2]))) / f32(res)
    inv = f32(1.0) / f32(cell)
    return [math.floor(f32(f32(position[i]) - f32(bbox_min[i])) * inv) for i in range(3)]


def twist_quat(twist):
    """(sin(theta/2) v, cos(theta/2)) with theta = |twist| in float and v
    the twist scaled by 1/theta (unchanged when theta is 0)."""
    f32 = np.float32
    t = [f32(v) for v in twist]
    sq = f32(f32(t[0] * t[0]) + f32(t[1] * t[1])) + f32(t[2] * t[2])
    theta = f32(math.sqrt(float(sq)))
    v = list(t)
    if theta != 0:
        inv = f32(1.0) / theta
        v = [f32(x * inv) for x in v]
    s, c = math.sin(0.5 * float(theta)), math.cos(0.5 * float(theta))
    return np.array([s * float(v[0]), s * float(v[1]), s * float(v[2]), c], dtype=np.float32)


def system(res, nodes):
    """A = L^T L + S (scipy CSR, float64 values of the float32 entries)."""
    import scipy.sparse as sp
    n = res ** 3
    idx = np.arange(n)
    x, y, z = idx % res, (idx // res) % res, idx // (res * res)
    deg = (x > 0).astype(np.int64) + (x < res - 1) + (y > 0) + (y < res - 1) + (z > 0) + (z < res - 1)
    w = (-(np.float32(1.0) / deg.astype(np.float32))).astype(np.float64)
    rows, cols, vals = [idx], [idx], [np.ones(n)]
    for d, ok in ((1, x < res - 1), (-1, x > 0), (res, y < res - 1), (-res, y > 0), (res * res, z < res - 1),
                  (-res * res, z > 0)):
        rows.append(idx[ok])
        cols.append(idx[ok] + d)
        vals.append(w[ok])
    Lm = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    s = np.zeros(n)
    s[list(nodes)] = 1.0
    return (Lm.T @ Lm + sp.diags(s)).tocsc()


def generate(res, bbox_min, bbox_max, points):
    """points: [(position, twist)]; returns (res^3, 4) float32 quaternions."""
    import scipy.sparse.linalg as sla
    n = res ** 3
    if not points:
        q = np.zeros((n, 4), np.float32)
        q[:, 1] = 1.0
        return q
    nodes, rhs = [], np.zeros((n, 4))
    for pos, tw in points:
        g = lattice_position(pos, bbox_min, bbox_max, res)
        c = g[0] + res * g[1] + res * res * g[2]
        nodes.append(c)
        rhs[c] = twist_quat(tw)
    A = system(res, nodes)
    lu = sla.splu(A)
    q = np.stack([lu.solve(rhs[:, k]) for k in range(4)], axis=1)
    return q.astype(np.float32)


def rotation_to_twist(e_x, e_y, e_z):
    """FrameField::RotationToTwistCayley (GMorpho/FrameField.cu:228-252)."""
    R = np.array([e_x, e_y, e_z], dtype=np.float64).T
    I = np.eye(3)
    C = (R - I) @ np.linalg.inv(R + I)
    axis = np.array([-C[1, 2], C[0, 2], -C[0, 1]])
    ln = np.linalg.norm(axis)
    if ln != 0:
        axis = axis / ln
    theta = math.acos(min(max((R[0, 0] + R[1, 1] + R[2, 2] - 1.0) / 2.0, -1.0), 1.0))
    return (theta * axis).astype(np.float32)
