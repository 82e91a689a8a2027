"""Generate the golden fixtures of tests/golden/ (run in a development
checkout; the fixtures are committed and the tests only read them).

    python tests/golden/gen_golden.py

There are no golden vectors in the reference (superboubek/Broxy has no
tests), so these fixtures come from a second, independent transliteration
of the reference GPU code, written here in plain Python with numpy float32
arithmetic and kept deliberately close to the reference kernels:

  * FillLevel0 / BuildMipmapFromTo texel pyramid (GMorpho/Grid.cu:733-805,
    957-998);
  * the stack traversals of DilateBySphereByTexMipmap{Base,}
    (GMorpho/GMorpho.cu:2828-3056) with HasSphereSEOverlap /
    SphereAABBSqDistance in float32 (GMorpho.cu:193-210,
    cuda_math.h:973-988), DilateByCubeByTexMipmap{Base,} with closed AABB
    overlap (GMorpho.cu:140-149, 1838-1934, 2603-2721), and the ILP erosion
    traversals ErodeBySphereTexMipmapBaseILP2 / ...PersistentWarpILP with
    their accum[] float32 sums (GMorpho.cu:4349-4647, 5041-5375);
  * the contour taggers (TagVoxelsContourBaseTight, TagVoxelsContourBase,
    TagVoxelsContourByErosion with its explicit C0..C7 tables,
    Grid.cu:1230-1327, 1499-1608) and the update sequence of
    GMorpho::Update (GMorpho.cu:7775-7817);
  * ComputeContourMCM / ComputeMCMData with the explicit MC bit tables,
    Morton sort, CompactMCMData, SplatIndices, BuildNeighbors (5-argument),
    and createTrianglesAndVertices3D (GMorpho.cu:6109-6496,
    MarchingCubesMesher.cu:1297-1500), including the case-91 slot overlap.

The CPU oracle (oracle/gm_oracle.c, integer restatement) is checked against
these fixtures by tests/test_oracle_golden.py; the CUDA path is checked
against the oracle.  The MC case tables are the ones of
broxy_gb300/csrc/mc_tables.inc.
"""
import hashlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

F = np.float32


# ------------------------------------------------------------------ tables

def mc_tables():
    src = open(os.path.join(ROOT, "broxy_gb300", "csrc", "mc_tables.inc")).read()

    def block(name):
        body = src.split("#define " + name)[1].split("}")[0]
        return [int(v, 0) for v in re.findall(r"0x[0-9a-fA-F]+|\b\d+\b", body)]

    packed = block("GM_MC_TRI_PACKED_INIT")
    count = block("GM_MC_TRI_COUNT_INIT")
    length = block("GM_MC_TRI_LEN_INIT")
    tri = []
    for c in range(256):
        tri.append([(packed[c] >> (4 * i)) & 0xF for i in range(3 * length[c])] + [-1])
    return tri, count


EDGES = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]


def edge_table(v):
    return sum(1 << e for e, (a, b) in enumerate(EDGES) if ((v >> a) & 1) != ((v >> b) & 1))


# ------------------------------------------------------------------ pyramid

def fill_level0(grid, scale, res):
    n = 2 * res
    lvl = {}
    for z in range(res):
        for y in range(res):
            for x in range(res):
                i = res * res * z + res * y + x
                pack = int(grid[i])
                for k in range(7, -1, -1):
                    fx = 2 * x + (1 if 0xaa & (1 << k) else 0)
                    fy = 2 * y + (1 if 0xcc & (1 << k) else 0)
                    fz = 2 * z + (1 if 0xf0 & (1 << k) else 0)
                    pack <<= 7
                    radius = F(int(scale[fx + n * fy + n * n * fz]))
                    radius = max(min(radius, F(127.0)), F(2.0))
                    pack |= int(radius) & 0x7f
                lvl[(x, y, z)] = pack
    return lvl


def build_mipmap(level0, res):
    levels = [level0]
    width = res
    while width != 1:
        width //= 2
        frm = levels[-1]
        to = {}
        for z in range(width):
            for y in range(width):
                for x in range(width):
                    val = [frm[(2 * x + (l & 1), 2 * y + ((l >> 1) & 1), 2 * z + (l >> 2))] for l in range(8)]
                    out = 0
                    for l in range(7, -1, -1):
                        vin = val[l]
                        m = 0
                        for k in range(8):
                            m = max(m, vin & 0x7f)
                            vin >>= 7
                        out = (out << 7) | (m & 0x7f)
                    for l in range(8):
                        if (val[l] >> 56) & 0xff:
                            out |= 1 << (56 + l)
                    to[(x, y, z)] = out
        levels.append(to)
    return levels  # levels[0] finest


# ------------------------------------------------------------------ float helpers

def sphere_aabb_sq(c, mn, mx):
    sq = F(0)
    for a in range(3):
        if c[a] < mn[a]:
            d = F(c[a] - mn[a])
            sq = F(sq + F(d * d))
        elif c[a] > mx[a]:
            d = F(c[a] - mx[a])
            sq = F(sq + F(d * d))
    return sq


def traverse_dilate(levels, max_depth, se_min, se_max, cube):
    max_res = 1 << max_depth
    stack = [(-1, 0, 0, 0)]
    node = (0, 0, 0, 0)
    occ = 0
    while True:
        depth, ix, iy, iz = node
        cell = F(max_res >> (depth + 1))
        inv = F(F(1.0) / cell)
        nmin = [F(inv * se_min[a]) for a in range(3)]
        nmax = [F(inv * se_max[a]) for a in range(3)]
        tex = levels[max_depth - depth - 1][(ix, iy, iz)]
        geo = (tex >> 56) & 0xff
        for k in range(8):
            cx, cy, cz = 2 * ix + (k & 1), 2 * iy + ((k >> 1) & 1), 2 * iz + (k >> 2)
            if not (geo & (1 << k)):
                continue
            lo = [F(cx), F(cy), F(cz)]
            hi = [F(lo[0] + F(1)), F(lo[1] + F(1)), F(lo[2] + F(1))]
            if cube:
                hit = all(nmin[a] <= hi[a] and nmax[a] >= lo[a] for a in range(3))
            else:
                q = [F(F(0.5) * F(nmin[a] + nmax[a])) for a in range(3)]
                h = F(F(0.5) * F(nmax[0] - nmin[0]))
                hit = sphere_aabb_sq(q, lo, hi) < F(h * h)
            if hit and depth + 1 != max_depth:
                stack.append((depth + 1, cx, cy, cz))
            elif hit:
                occ = 0xff
                stack.append((-1, 0, 0, 0))
        node = stack.pop()
        if node[0] == -1:
            return occ


def traverse_erode(levels, max_depth, query):
    """ILP erosion traversal: accum[] float32 sums per child (GMorpho.cu:4403-4640)."""
    max_res = 1 << max_depth
    stack = [(-1, 0, 0, 0)]
    node = (0, 0, 0, 0)
    while True:
        depth, ix, iy, iz = node
        cell = F(max_res >> (depth + 1))
        inv = F(F(1.0) / cell)
        nq = [F(inv * query[a]) for a in range(3)]
        tex = levels[max_depth - depth - 1][(ix, iy, iz)]
        geo = (tex >> 56) & 0xff
        b = [F(2 * ix), F(2 * iy), F(2 * iz)]
        sq = [F(0)] * 8
        for a in range(3):
            lo0 = F(F(nq[a] - b[a]) * F(nq[a] - b[a])) if nq[a] < b[a] else F(0)
            lo1 = F(F(nq[a] - b[a] - F(1)) * F(nq[a] - b[a] - F(1))) if nq[a] < F(b[a] + F(1)) else F(0)
            hi0 = F(F(nq[a] - b[a] - F(1)) * F(nq[a] - b[a] - F(1))) if nq[a] > F(b[a] + F(1)) else F(0)
            hi1 = F(F(nq[a] - b[a] - F(2)) * F(nq[a] - b[a] - F(2))) if nq[a] > F(b[a] + F(2)) else F(0)
            for k in range(8):
                bit = (k >> a) & 1
                sq[k] = F(sq[k] + (lo1 if bit else lo0))
            for k in range(8):
                bit = (k >> a) & 1
                sq[k] = F(sq[k] + (hi1 if bit else hi0))
        for k in range(8):
            r = (tex >> (7 * k)) & 0x7f
            t = F(F(r - 1) / cell)
            if sq[k] < F(t * t) and (geo & (1 << k)):
                if depth + 1 != max_depth:
                    stack.append((depth + 1, 2 * ix + (k & 1), 2 * iy + ((k >> 1) & 1), 2 * iz + (k >> 2)))
                else:
                    return 1
        node = stack.pop()
        if node[0] == -1:
            return 0


# ------------------------------------------------------------------ taggers

C = [1 << k for k in range(8)]


def tag_by_erosion(D, res, x, y, z):
    """TagVoxelsContourByErosion with its explicit tables (Grid.cu:1230-1327)."""
    g = lambda a, b, c: int(D[res * res * c + res * b + a])
    center = g(x, y, z)
    if center == 0xff:
        return 0
    tag = 0
    val = g(x + 1, y, z)
    for s, d in ((C[0], C[1]), (C[2], C[3]), (C[4], C[5]), (C[6], C[7])):
        tag |= d if val & s else 0
    val = g(x - 1, y, z)
    for s, d in ((C[1], C[0]), (C[3], C[2]), (C[5], C[4]), (C[7], C[6])):
        tag |= d if val & s else 0
    val = g(x, y + 1, z)
    for s, d in ((C[0], C[2]), (C[1], C[3]), (C[4], C[6]), (C[5], C[7])):
        tag |= d if val & s else 0
    val = g(x, y - 1, z)
    for s, d in ((C[2], C[0]), (C[3], C[1]), (C[6], C[4]), (C[7], C[5])):
        tag |= d if val & s else 0
    val = g(x, y, z + 1)
    for s, d in ((C[0], C[4]), (C[1], C[5]), (C[2], C[6]), (C[3], C[7])):
        tag |= d if val & s else 0
    val = g(x, y, z - 1)
    for s, d in ((C[4], C[0]), (C[5], C[1]), (C[6], C[2]), (C[7], C[3])):
        tag |= d if val & s else 0
    inner = [(C[1], C[0]), (C[2], C[0]), (C[4], C[0]), (C[0], C[1]), (C[3], C[1]), (C[5], C[1]),
             (C[0], C[2]), (C[3], C[2]), (C[6], C[2]), (C[1], C[3]), (C[2], C[3]), (C[7], C[3]),
             (C[5], C[4]), (C[6], C[4]), (C[0], C[4]), (C[4], C[5]), (C[7], C[5]), (C[1], C[5]),
             (C[4], C[6]), (C[7], C[6]), (C[2], C[6]), (C[5], C[7]), (C[6], C[7]), (C[3], C[7])]
    for s, d in inner:
        tag |= d if center & s else 0
    return tag & (~center & 0xff)


# ------------------------------------------------------------------ closing

def close_reference(X, scale, res, data_res, cube):
    """GMorpho::Update's morphology (GMorpho.cu:7775-7817), GM_REF."""
    max_depth = int(np.log2(res)) + 1
    lv = build_mipmap(fill_level0(X, scale, res), res)
    D = X.copy()
    # base dilation
    for z in range(data_res[2]):
        for y in range(data_res[1]):
            for x in range(data_res[0]):
                i = res * res * z + res * y + x
                if X[i] == 0xff:
                    continue
                r = F(lv[0][(x, y, z)] & 0x7f)
                if not cube:
                    r = F(r + F(1))
                se_min = [F(F(2 * x) - r), F(F(2 * y) - r), F(F(2 * z) - r)]
                se_max = [F(F(2 * x) + r), F(F(2 * y) + r), F(F(2 * z) + r)]
                if traverse_dilate(lv, max_depth, se_min, se_max, cube):
                    D[i] = 0xff
    # tight contour, then fine dilation
    tagged = []
    for z in range(res - 1):
        for y in range(res - 1):
            for x in range(res - 1):
                v = [D[res * res * (z + (k >> 2)) + res * (y + ((k >> 1) & 1)) + x + (k & 1)] for k in range(8)]
                ind = sum(1 << k for k in range(8) if v[k] >= 0xff)
                if ind not in (0, 0xff):
                    tagged.append(res * res * z + res * y + x)
    out = {}
    for i in tagged:
        z, rem = divmod(i, res * res)
        y, x = divmod(rem, res)
        tex = lv[0][(x, y, z)]
        occ = 0
        for k in range(8):
            fx, fy, fz = 2 * x + (k & 1), 2 * y + ((k >> 1) & 1), 2 * z + (k >> 2)
            r = F((tex >> (7 * k)) & 0x7f)
            if not cube:
                r = F(r + F(1))
            se_min = [F(F(fx) - r), F(F(fy) - r), F(F(fz) - r)]
            se_max = [F(F(fx) + r), F(F(fy) + r), F(F(fz) + r)]
            if traverse_dilate(lv, max_depth, se_min, se_max, cube):
                occ |= 1 << k
        out[i] = occ
    for i, v in out.items():
        D[i] = v
    # contour of the dilation
    S = np.zeros_like(D)
    for z in range(1, res - 1):
        for y in range(1, res - 1):
            for x in range(1, res - 1):
                S[res * res * z + res * y + x] = tag_by_erosion(D, res, x, y, z)
    ls = build_mipmap(fill_level0(S, scale, res), res)
    Cg = D.copy()
    for z in range(data_res[2]):
        for y in range(data_res[1]):
            for x in range(data_res[0]):
                i = res * res * z + res * y + x
                if D[i] == 0 or X[i] == 0xff:
                    continue
                q = [F(2 * x + 1), F(2 * y + 1), F(2 * z + 1)]
                if traverse_erode(ls, max_depth, q):
                    Cg[i] = 0
    # 6-neighbour contour of the base closing, then fine erosion
    tagged = []
    for z in range(1, res - 1):
        for y in range(1, res - 1):
            for x in range(1, res - 1):
                i = res * res * z + res * y + x
                c = Cg[i]
                if any(Cg[j] != c for j in (i - 1, i + 1, i - res, i + res, i - res * res, i + res * res)):
                    tagged.append(i)
    out = {}
    for i in tagged:
        z, rem = divmod(i, res * res)
        y, x = divmod(rem, res)
        eroded = 0xff
        for k in range(8):
            fx, fy, fz = 2 * x + (k & 1), 2 * y + ((k >> 1) & 1), 2 * z + (k >> 2)
            q = [F(fx + F(0.5)), F(fy + F(0.5)), F(fz + F(0.5))]
            if traverse_erode(ls, max_depth, q):
                eroded &= ~(1 << k) & 0xff
        out[i] = eroded
    for i, v in out.items():
        Cg[i] = v
    return D, S, Cg


# ------------------------------------------------------------------ marching cubes

def morton(x, y, z):
    m = 0
    for b in range(10):
        m |= ((x >> b) & 1) << (3 * b) | ((y >> b) & 1) << (3 * b + 1) | ((z >> b) & 1) << (3 * b + 2)
    return m


def mc_reference(Cg, res, bbox_min, cell_size, iso=0.95):
    tri, count = mc_tables()
    g = lambda x, y, z: int(Cg[res * res * z + res * y + x])
    bit = lambda v, k: (v >> k) & 1
    # ComputeContourMCM + ComputeMCMData: the eight sub-cube values, with the
    # explicit v0..v7 / C / MC mapping of GMorpho.cu:6146-6232
    cells = []
    for z in range(1, res - 1):
        for y in range(1, res - 1):
            for x in range(1, res - 1):
                v = [g(x, y, z), g(x + 1, y, z), g(x, y + 1, z), g(x + 1, y + 1, z), g(x, y, z + 1),
                     g(x + 1, y, z + 1), g(x, y + 1, z + 1), g(x + 1, y + 1, z + 1)]
                spec = [
                    [(0, 0), (0, 1), (0, 3), (0, 2), (0, 4), (0, 5), (0, 7), (0, 6)],
                    [(0, 1), (1, 0), (1, 2), (0, 3), (0, 5), (1, 4), (1, 6), (0, 7)],
                    [(0, 2), (0, 3), (2, 1), (2, 0), (0, 6), (0, 7), (2, 5), (2, 4)],
                    [(0, 3), (1, 2), (3, 0), (2, 1), (0, 7), (1, 6), (3, 4), (2, 5)],
                    [(0, 4), (0, 5), (0, 7), (0, 6), (4, 0), (4, 1), (4, 3), (4, 2)],
                    [(0, 5), (1, 4), (1, 6), (0, 7), (4, 1), (5, 0), (5, 2), (4, 3)],
                    [(0, 6), (0, 7), (2, 5), (2, 4), (4, 2), (4, 3), (6, 1), (6, 0)],
                    [(0, 7), (1, 6), (3, 4), (2, 5), (4, 3), (5, 2), (7, 0), (6, 1)],
                ]
                vals = [sum(bit(v[c], b) << j for j, (c, b) in enumerate(spec[s])) for s in range(8)]
                if any(w not in (0, 255) for w in vals):
                    cells.append((morton(x, y, z), x, y, z, vals))
    cells.sort()
    idx, vals = [], []
    for _, x, y, z, vv in cells:
        for s in range(8):
            fx, fy, fz = 2 * x + (s & 1), 2 * y + ((s >> 1) & 1), 2 * z + (s >> 2)
            if vv[s] not in (0, 255):
                idx.append(4 * res * res * fz + 2 * res * fy + fx)
                vals.append(vv[s])
    n = len(idx)
    grid_ids = {ind: i for i, ind in enumerate(idx)}  # SplatIndices
    R = 2 * res
    neigh = []
    for ind in idx:  # BuildNeighbors (5-argument)
        fz, rem = divmod(ind, R * R)
        fy, fx = divmod(rem, R)
        offs = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
        neigh.append([grid_ids.get(R * R * (fz + dz) + R * (fy + dy) + fx + dx, 0xffffffff) for dx, dy, dz in offs])
    nbv = [(1 if edge_table(v) & 1 else 0) + (1 if edge_table(v) & 8 else 0) + (1 if edge_table(v) & 256 else 0)
           for v in vals]
    nbt = [count[v] for v in vals]
    voff = np.concatenate([[0], np.cumsum(nbv)[:-1]]).astype(np.int64) if n else np.zeros(0, np.int64)
    toff = np.concatenate([[0], np.cumsum(nbt)[:-1]]).astype(np.int64) if n else np.zeros(0, np.int64)
    nV, nT = int(sum(nbv)), int(sum(nbt))
    V = np.zeros((nV, 3), np.float32)
    T = np.zeros((nT, 3), np.uint32)
    cs = F(F(0.5) * F(cell_size))
    mn = [F(b) for b in bbox_min]
    late = []
    for i in range(n):
        ind, cv = idx[i], vals[i]
        fz, rem = divmod(ind, R * R)
        fy, fx = divmod(rem, R)
        # minC + idx * cellSize, contracted into one fused multiply-add
        pt = [F(np.float64(F(c)) * np.float64(cs) + np.float64(m)) for c, m in zip((fx, fy, fz), mn)]
        e = edge_table(cv)
        v = [F(1) if (cv >> j) & 1 else F(0) for j in range(8)]
        vert = [0] * 12
        ind_v = 0

        def inter(p1, v1, p2, v2):
            t = F(F(iso) - v1)
            return [F(p1[a] + F(F(t * F(p2[a] - p1[a])) / F(v2 - v1))) for a in range(3)]

        if e & 1:
            vert[0] = int(voff[i]) + ind_v
            V[vert[0]] = inter(pt, v[0], [F(pt[0] + cs), pt[1], pt[2]], v[1])
            ind_v += 1
        nb = neigh[i]
        if e & 2 and nb[1] != 0xffffffff:
            vert[1] = int(voff[nb[1]]) + (1 if edge_table(vals[nb[1]]) & 1 else 0)
        if e & 4:
            vert[2] = int(voff[nb[3]]) if nb[3] != 0xffffffff else 0
        if e & 8:
            vert[3] = int(voff[i]) + ind_v
            V[vert[3]] = inter([pt[0], F(pt[1] + cs), pt[2]], v[3], pt, v[0])
            ind_v += 1
        if e & 16:
            vert[4] = int(voff[nb[4]]) if nb[4] != 0xffffffff else 0
        if e & 32 and nb[5] != 0xffffffff:
            vert[5] = int(voff[nb[5]]) + (1 if edge_table(vals[nb[5]]) & 1 else 0)
        if e & 64:
            vert[6] = int(voff[nb[7]]) if nb[7] != 0xffffffff else 0
        if e & 128 and nb[4] != 0xffffffff:
            vert[7] = int(voff[nb[4]]) + (1 if edge_table(vals[nb[4]]) & 1 else 0)
        if e & 256:
            vert[8] = int(voff[i]) + ind_v
            V[vert[8]] = inter(pt, v[0], [pt[0], pt[1], F(pt[2] + cs)], v[4])
            ind_v += 1
        for bitmask, k, slot in ((512, 1, 9), (1024, 2, 10), (2048, 3, 11)):
            if e & bitmask:
                e1 = edge_table(vals[nb[k]]) if nb[k] != 0xffffffff else 0
                d = (1 if e1 & 1 else 0) + (1 if e1 & 8 else 0)
                vert[slot] = int(voff[nb[k]]) + d if nb[k] != 0xffffffff else d
        tl = tri[cv]
        s = 0
        t = 0
        while tl[s] != -1:
            row = (vert[tl[s + 2]], vert[tl[s + 1]], vert[tl[s]])
            pos = int(toff[i]) + t
            if t < count[cv]:
                T[pos] = row
            elif pos < nT:
                late.append((pos, row))  # written after the others: it wins
            s += 3
            t += 1
    for pos, row in late:
        T[pos] = row
    return V, T


# ------------------------------------------------------------------ cases

def random_grid(res, seed):
    from broxy_gb300 import synth
    return synth.random_grid(res, seed)


def cases():
    out = []
    for res, seed, r, cube in [(8, 1, 2, False), (8, 2, 3, False), (16, 3, 3, False), (16, 4, 4, False),
                               (16, 5, 2, True), (16, 6, 3, True)]:
        out.append(dict(name="r%d_s%d_rad%d_%s" % (res, seed, r, "cube" if cube else "sphere"), res=res, seed=seed,
                        uniform=r, cube=cube, variable=False, data_res=[res] * 3))
    for res, seed in [(8, 11), (16, 12)]:
        out.append(dict(name="r%d_s%d_variable" % (res, seed), res=res, seed=seed, uniform=0, cube=False,
                        variable=True, data_res=[res] * 3))
    out.append(dict(name="r16_s13_datares", res=16, seed=13, uniform=3, cube=False, variable=False,
                    data_res=[13, 15, 11]))
    return out


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    manifest = {}
    for c in cases():
        res = c["res"]
        X = random_grid(res, c["seed"])
        if c["variable"]:
            rng = np.random.default_rng(c["seed"])
            scale = rng.integers(-2, 7, size=(2 * res) ** 3).astype(np.int8)
        else:
            scale = np.full((2 * res) ** 3, c["uniform"], np.int8)
        D, S, Cg = close_reference(X, scale, res, c["data_res"], c["cube"])
        V, T = mc_reference(Cg, res, [0.25, -0.5, 1.0], 0.0625)
        np.savez_compressed(os.path.join(HERE, c["name"] + ".npz"), X=X, scale=scale, D=D, S=S, C=Cg, V=V, T=T)
        manifest[c["name"]] = dict(c, D=sha(D), S=sha(S), C=sha(Cg), V=sha(V), T=sha(T), nv=len(V), nt=len(T))
        print(c["name"], int(D.sum()), int(Cg.sum()), len(V), len(T))
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
