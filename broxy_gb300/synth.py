"""Seeded synthetic inputs for the GMorpho workloads.

No dataset ships with the reference; these generators stand in for its
inputs with the shapes, sizes and value distributions named by the
benchmark configurations:

  * union of 64 level-3 icospheres (the reference's own sphere.off is a
    642-vertex / 1280-face level-3 icosphere), centres U[0.2,0.8]^3,
    radii U[0.03,0.12];
  * sum of isotropic Gaussian blobs (sigma U[0.01,0.05], weights
    U[0.5,1.5], centres U[0.2,0.8]^3) classified at level 0.5;
  * a variable radius field r = 2 + floor(30 s(x)), s a normalised sum of
    16 Gaussian RBFs clamped to [0,1], evaluated in double on the host side
    of the generator and stored as int8 per fine voxel;
  * the blob field's triangulated isosurface at level 0.5 (blob_mesh:
    marching cubes with linear interpolation on the sampled field, ~1M /
    4M / 8M triangles), which config_inputs voxelizes into the benchmark
    grids the way GMorpho::Load does (grid attributes from the mesh's box,
    conservative voxelization).

Seeds follow seed = 1000 * config + instance.
"""
import numpy as np


def icosphere(level=3):
    """Subdivided icosahedron on the unit sphere (level 3: 642 v, 1280 f)."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    faces = list(f)
    for _ in range(level):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts, dtype=np.float64), np.array(faces, dtype=np.uint32)


def spheres_mesh(seed=1000, count=64, level=3):
    """Concatenated icospheres (the configuration-1 input mesh)."""
    rng = np.random.default_rng(seed)
    V0, F0 = icosphere(level)
    centres = rng.uniform(0.2, 0.8, size=(count, 3))
    radii = rng.uniform(0.03, 0.12, size=count)
    Vs, Fs = [], []
    for i in range(count):
        Vs.append(V0 * radii[i] + centres[i])
        Fs.append(F0 + i * len(V0))
    return np.concatenate(Vs).astype(np.float32), np.concatenate(Fs).astype(np.uint32)


def blob_params(seed, count=200):
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.2, 0.8, size=(count, 3))
    sigmas = rng.uniform(0.01, 0.05, size=count)
    weights = rng.uniform(0.5, 1.5, size=count)
    return centres, sigmas, weights


def radius_params(seed, count=16):
    rng = np.random.default_rng(seed + 7)
    centres = rng.uniform(0.0, 1.0, size=(count, 3))
    widths = rng.uniform(0.05, 0.25, size=count)
    amps = rng.uniform(0.5, 1.0, size=count)
    return centres, widths, amps


def _axis(n, lo=0.0, hi=1.0):
    return lo + (np.arange(n, dtype=np.float64) + 0.5) * (hi - lo) / n


def blob_grid(res, seed, count=200, level=0.5, device=None):
    """Packed grid (uint8 res^3) of the blob solid {f >= level} sampled at the
    fine voxel centres of the unit cube.  With ``device`` (a torch device) the
    field is evaluated with torch on that device in float64 slabs."""
    N = 2 * res
    centres, sigmas, weights = blob_params(seed, count)
    if device is None:
        x = _axis(N)
        occ = np.zeros((N, N, N), dtype=bool)  # [z, y, x]
        for z0 in range(0, N, 16):
            zs = x[z0:z0 + 16]
            f = np.zeros((len(zs), N, N))
            for c, s, w in zip(centres, sigmas, weights):
                gx = np.exp(-(x - c[0]) ** 2 / (2 * s * s))
                gy = np.exp(-(x - c[1]) ** 2 / (2 * s * s))
                gz = np.exp(-(zs - c[2]) ** 2 / (2 * s * s))
                f += w * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
            occ[z0:z0 + 16] = f >= level
        return pack_dense(occ)
    import torch
    x = torch.as_tensor(_axis(N), device=device)
    occ = torch.zeros((N, N, N), dtype=torch.bool, device=device)
    c = torch.as_tensor(centres, device=device)
    s = torch.as_tensor(sigmas, device=device)
    w = torch.as_tensor(weights, device=device)
    gx = torch.exp(-(x[None, :] - c[:, 0:1]) ** 2 / (2 * s[:, None] ** 2)) * w[:, None]  # [count, N]
    gy = torch.exp(-(x[None, :] - c[:, 1:2]) ** 2 / (2 * s[:, None] ** 2))
    gz = torch.exp(-(x[None, :] - c[:, 2:3]) ** 2 / (2 * s[:, None] ** 2))
    for z0 in range(0, N, 8):
        f = torch.einsum("kz,ky,kx->zyx", gz[:, z0:z0 + 8], gy, gx)
        occ[z0:z0 + 8] = f >= level
    return pack_dense_torch(occ)


def radius_field(res, seed, base=2, span=30, count=16, device=None):
    """int8 fine radius grid r = base + floor(span * clamp(s, 0, 1))."""
    N = 2 * res
    centres, widths, amps = radius_params(seed, count)
    if device is None:
        x = _axis(N)
        out = np.empty((N, N, N), dtype=np.int8)
        for z0 in range(0, N, 16):
            zs = x[z0:z0 + 16]
            f = np.zeros((len(zs), N, N))
            for c, s, a in zip(centres, widths, amps):
                f += a * np.exp(-(zs - c[2])[:, None, None] ** 2 / (2 * s * s)) * \
                    np.exp(-(x - c[1])[None, :, None] ** 2 / (2 * s * s)) * \
                    np.exp(-(x - c[0])[None, None, :] ** 2 / (2 * s * s))
            out[z0:z0 + 16] = base + np.floor(span * np.clip(f, 0.0, 1.0)).astype(np.int8)
        return out.reshape(-1)
    import torch
    x = torch.as_tensor(_axis(N), device=device)
    c = torch.as_tensor(centres, device=device)
    s = torch.as_tensor(widths, device=device)
    a = torch.as_tensor(amps, device=device)
    gx = torch.exp(-(x[None, :] - c[:, 0:1]) ** 2 / (2 * s[:, None] ** 2)) * a[:, None]
    gy = torch.exp(-(x[None, :] - c[:, 1:2]) ** 2 / (2 * s[:, None] ** 2))
    gz = torch.exp(-(x[None, :] - c[:, 2:3]) ** 2 / (2 * s[:, None] ** 2))
    out = torch.empty((N, N, N), dtype=torch.int8, device=device)
    for z0 in range(0, N, 8):
        f = torch.einsum("kz,ky,kx->zyx", gz[:, z0:z0 + 8], gy, gx)
        out[z0:z0 + 8] = (base + torch.floor(span * f.clamp(0.0, 1.0))).to(torch.int8)
    return out.reshape(-1)


def pack_dense(occ):
    """Dense bool [z, y, x] (edge N) -> packed grid uint8[res^3] (x-fastest)."""
    N = occ.shape[0]
    res = N // 2
    o = occ.reshape(res, 2, res, 2, res, 2)  # z, zb, y, yb, x, xb
    out = np.zeros((res, res, res), dtype=np.uint8)
    for zb in range(2):
        for yb in range(2):
            for xb in range(2):
                out |= (o[:, zb, :, yb, :, xb].astype(np.uint8) << (xb + 2 * yb + 4 * zb))
    return out.reshape(-1)


def unpack_dense(grid, res):
    g = np.asarray(grid, dtype=np.uint8).reshape(res, res, res)
    occ = np.zeros((res, 2, res, 2, res, 2), dtype=bool)
    for zb in range(2):
        for yb in range(2):
            for xb in range(2):
                occ[:, zb, :, yb, :, xb] = (g >> (xb + 2 * yb + 4 * zb)) & 1
    return occ.reshape(2 * res, 2 * res, 2 * res)


def pack_dense_torch(occ):
    import torch
    N = occ.shape[0]
    res = N // 2
    o = occ.reshape(res, 2, res, 2, res, 2).to(torch.uint8)
    out = torch.zeros((res, res, res), dtype=torch.uint8, device=occ.device)
    for zb in range(2):
        for yb in range(2):
            for xb in range(2):
                out |= o[:, zb, :, yb, :, xb] << (xb + 2 * yb + 4 * zb)
    return out.reshape(-1)


def random_grid(res, seed, density=0.5, blobs=6):
    """Small random test grid: a few random spheres plus sparse noise."""
    rng = np.random.default_rng(seed)
    N = 2 * res
    z, y, x = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    occ = np.zeros((N, N, N), dtype=bool)
    for _ in range(blobs):
        c = rng.uniform(0.25 * N, 0.75 * N, size=3)
        r = rng.uniform(0.05 * N, 0.18 * N)
        occ |= (x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2 <= r * r
    noise = rng.random((N, N, N)) < 0.002 * density
    inner = np.zeros_like(occ)
    m = N // 5
    inner[m:N - m, m:N - m, m:N - m] = True
    occ |= noise & inner
    return pack_dense(occ)


def batch_instances(seed=4000, count=64, lo=64, hi=512, device=None):
    """The batching workload: `count` grids whose fine edge E is drawn
    log-uniform in [lo, hi] and padded to a multiple of 32, each embedded in
    the next power-of-two cube (data_res = E/2 cells), holding a blob solid
    scaled to its E-box, with its own uniform radius U{1..24}.  Returns a
    list of dicts (res, data_res, X, radius, edge)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        E = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        E = int(np.ceil(E / 32.0) * 32)
        N = 1
        while N < E:
            N *= 2
        res = N // 2
        radius = int(rng.integers(1, 25))
        blobs = int(max(6, min(200, 200 * (E / 512.0) ** 2)))
        X = _blob_box(res, E, seed * 100 + i, blobs, device)
        out.append(dict(res=res, data_res=[E // 2] * 3, X=X, radius=radius, edge=E))
    return out


def _blob_box(res, E, seed, count, device):
    """Blob solid with centres in [0.2, 0.8] of an E-voxel box at the grid
    origin, classified at the fine voxel centres of the res-cell grid."""
    N = 2 * res
    centres, sigmas, weights = blob_params(seed, count)
    scale = E / float(N)
    centres = centres * scale
    sigmas = sigmas * scale * 1.5
    if device is None:
        x = _axis(N)
        occ = np.zeros((N, N, N), dtype=bool)
        for z0 in range(0, N, 16):
            zs = x[z0:z0 + 16]
            f = np.zeros((len(zs), N, N))
            for c, s, w in zip(centres, sigmas, weights):
                f += w * np.exp(-(zs - c[2])[:, None, None] ** 2 / (2 * s * s)) * \
                    np.exp(-(x - c[1])[None, :, None] ** 2 / (2 * s * s)) * \
                    np.exp(-(x - c[0])[None, None, :] ** 2 / (2 * s * s))
            occ[z0:z0 + 16] = f >= 0.5
        return pack_dense(occ)
    import torch
    x = torch.as_tensor(_axis(N), device=device)
    c = torch.as_tensor(centres, device=device)
    s = torch.as_tensor(sigmas, device=device)
    w = torch.as_tensor(weights, device=device)
    gx = torch.exp(-(x[None, :] - c[:, 0:1]) ** 2 / (2 * s[:, None] ** 2)) * w[:, None]
    gy = torch.exp(-(x[None, :] - c[:, 1:2]) ** 2 / (2 * s[:, None] ** 2))
    gz = torch.exp(-(x[None, :] - c[:, 2:3]) ** 2 / (2 * s[:, None] ** 2))
    occ = torch.zeros((N, N, N), dtype=torch.bool, device=device)
    for z0 in range(0, N, 16):
        f = torch.einsum("kz,ky,kx->zyx", gz[:, z0:z0 + 16], gy, gx)
        occ[z0:z0 + 16] = f >= 0.5
    return pack_dense_torch(occ)


_MC_TABLES = None


def _mc_tables():
    """The marching-cubes triangle table (edge ids per case, x-fastest corner
    order v0=000 v1=100 v2=110 v3=010 v4=001 v5=101 v6=111 v7=011) from the
    library's generated table file."""
    global _MC_TABLES
    if _MC_TABLES is None:
        import os
        import re
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc", "mc_tables.inc")
        text = open(path).read()

        def block(name):
            body = text[text.index(name):]
            body = body[body.index("{") + 1:body.index("}")]
            return [int(v.rstrip("ULL"), 0) for v in re.findall(r"0x[0-9a-fA-F]+ULL|\b\d+\b", body)]

        packed, length = block("GM_MC_TRI_PACKED_INIT"), block("GM_MC_TRI_LEN_INIT")
        edges = np.zeros((256, 15), np.int64)
        for c in range(256):
            for k in range(15):
                edges[c, k] = (packed[c] >> (4 * k)) & 0xf
        _MC_TABLES = (edges, np.array(length, np.int64))
    return _MC_TABLES


_CORNERS = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])
_EDGES = np.array([[0, 1], [1, 2], [2, 3], [3, 0], [4, 5], [5, 6], [6, 7], [7, 4], [0, 4], [1, 5], [2, 6], [3, 7]])


def blob_mesh(n, seed, count=200, level=0.5, device="cuda"):
    """The blob field's isosurface {f = level} as a triangle mesh: marching
    cubes with linear interpolation on the field sampled at the n^3 points
    (i + 1/2)/n of the unit cube (device float32 (3m, 3) vertices, int32
    (m, 3) triangles, three vertices per triangle).  A vertex is computed
    from its edge's two samples in a fixed order, so the cubes sharing an
    edge produce the same bits and the surface is closed."""
    import torch
    edges_tab, len_tab = (torch.as_tensor(a, device=device) for a in _mc_tables())
    corners = torch.as_tensor(_CORNERS, device=device)
    edge_ab = torch.as_tensor(_EDGES, device=device)
    centres, sigmas, weights = blob_params(seed, count)
    x = torch.as_tensor(_axis(n), device=device)
    c = torch.as_tensor(centres, device=device)
    s = torch.as_tensor(sigmas, device=device)
    w = torch.as_tensor(weights, device=device)
    gx = torch.exp(-(x[None, :] - c[:, 0:1]) ** 2 / (2 * s[:, None] ** 2)) * w[:, None]
    gy = torch.exp(-(x[None, :] - c[:, 1:2]) ** 2 / (2 * s[:, None] ** 2))
    gz = torch.exp(-(x[None, :] - c[:, 2:3]) ** 2 / (2 * s[:, None] ** 2))
    f = torch.empty((n, n, n), dtype=torch.float32, device=device)  # [z, y, x]
    for z0 in range(0, n, 8):
        f[z0:z0 + 8] = torch.einsum("kz,ky,kx->zyx", gz[:, z0:z0 + 8], gy, gx).float()
    h = 1.0 / n
    tris = []
    S = 16
    for z0 in range(0, n - 1, S):
        z1 = min(z0 + S, n - 1)
        vals = [f[z0 + dz:z1 + dz, dy:n - 1 + dy, dx:n - 1 + dx] for (dx, dy, dz) in _CORNERS.tolist()]
        case = torch.zeros(vals[0].shape, dtype=torch.int64, device=device)
        for k, v in enumerate(vals):
            case |= (v >= level).long() << k
        act = torch.nonzero((case != 0) & (case != 255))
        if act.shape[0] == 0:
            continue
        cz, cy, cx = act[:, 0] + z0, act[:, 1], act[:, 2]
        cc = case[act[:, 0], act[:, 1], act[:, 2]]
        ntri = len_tab[cc]
        for t in range(5):
            sel = ntri > t
            if not bool(sel.any()):
                break
            bx, by, bz, bc = cx[sel], cy[sel], cz[sel], cc[sel]
            tri = []
            for j in range(3):
                e = edges_tab[bc, 3 * t + j]
                a, b = edge_ab[e, 0], edge_ab[e, 1]
                pa = torch.stack([bx + corners[a, 0], by + corners[a, 1], bz + corners[a, 2]], 1)
                pb = torch.stack([bx + corners[b, 0], by + corners[b, 1], bz + corners[b, 2]], 1)
                swap = (pb < pa).any(1, keepdim=True)  # the lower sample first, whichever cube asks
                p0, p1 = torch.where(swap, pb, pa), torch.where(swap, pa, pb)
                f0 = f[p0[:, 2], p0[:, 1], p0[:, 0]]
                f1 = f[p1[:, 2], p1[:, 1], p1[:, 0]]
                tt = ((level - f0) / (f1 - f0))[:, None]
                q0 = (p0.float() + 0.5) * h
                q1 = (p1.float() + 0.5) * h
                tri.append(q0 + tt * (q1 - q0))
            tris.append(torch.stack(tri, 1))
    P = torch.cat(tris, 0).reshape(-1, 3).contiguous()
    T = torch.arange(P.shape[0], dtype=torch.int32, device=device).reshape(-1, 3)
    del f
    return P, T


# Benchmark configurations with a voxelized blob mesh: (base res, field
# samples per axis of the isosurface mesh (~1M / 4M / 8M triangles), seed,
# uniform radius or 0 for the radius field r = 2 + floor(30 s)).
CONFIGS = {
    2: dict(res=256, samples=336, seed=2000, uniform=12),
    3: dict(res=512, samples=672, seed=3000, uniform=0),
    5: dict(res=1024, samples=950, seed=5000, uniform=8),
}
MESH_MARGIN = 0.05  # world units added around the mesh's box (GMorpho::Load's margin, GMorpho.cu:7735)


def mesh_samples(config, res=None):
    """Field samples per axis of a configuration's mesh, scaled with the
    grid when `res` differs from the configuration's own."""
    c = CONFIGS[config]
    if res is None or res == c["res"]:
        return c["samples"]
    return max(16, int(round(c["samples"] * res / c["res"])))


def config_inputs(ctx, config, res=None, voxelize_reps=0):
    """The inputs of benchmark configuration 2, 3 or 5 (optionally at another
    base resolution `res`, the mesh scaled with it): the blob mesh,
    voxelized like GMorpho::Load (gm_grid_attributes + gm_voxelize), and the
    fine radius field (None for a uniform radius).  Returns a dict with
    desc, X (device packed grid), R, uniform, P, T (device mesh) and, with
    voxelize_reps > 0, the voxelization's device time in ms (median of that
    many timed runs after one untimed)."""
    import torch
    from . import api
    c = CONFIGS[config]
    res = c["res"] if res is None else res
    P, T = blob_mesh(mesh_samples(config, res), c["seed"])
    desc = api.grid_attributes(P.cpu().numpy(), res, MESH_MARGIN)
    X = torch.zeros(res ** 3, dtype=torch.uint8, device=P.device)
    ctx.voxelize(desc, P, T, out=X)
    out = dict(desc=desc, X=X, P=P, T=T, res=res, uniform=c["uniform"], seed=c["seed"], config=config)
    if voxelize_reps > 0:
        times = []
        st = torch.cuda.current_stream()
        for _ in range(voxelize_reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            ctx.voxelize(desc, P, T, out=X)
            e1.record(st)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        out["voxelize_ms"] = float(np.median(times))
    if c["uniform"] == 0:
        out["R"] = radius_field(res, c["seed"], base=2, span=30, device=P.device).contiguous()
    else:
        out["R"] = None
    torch.cuda.synchronize()
    return out
