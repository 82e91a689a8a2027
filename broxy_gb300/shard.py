"""Z-slab sharding of one closing + mesh over several GPUs, one process per
GPU (no reference counterpart: the reference runs on one GPU).

Every rank owns the cells [z0, z1) of the grid and receives, up front, its
slab of the input grid (and radius field) with a halo on each cut side.  It
closes the slab as a box grid (``gm_close_box_region``; the closing is local, so a
slab cut with rmax + 8 cells of margin is exact on its owned cells) and
meshes it with a window in global coordinates (``gm_mesh_box``): triangles
of a guard band around the owned cells are kept long enough for the normals
and the bilateral filter to see every triangle their full-grid values see,
then only the triangles emitted by owned cells remain.  Stitching is one
exchange: all ranks learn each other's owned vertex counts (global vertex id
offsets) and the positions and ids of the vertices of each rank's first cell
layer, which the lower neighbour's triangles reference across the seam.
Concatenating the ranks' outputs gives the whole grid's closing and mesh.

The communication goes through a small interface (``allgather(obj)``), so
the same code runs over torch.distributed (any backend) or, for simulated
ranks in one process, over a plain list (``stitch_local``).
"""
import numpy as np

HALO_SPARE = 10  # cells past rmax: exactness margin (8) + the mesh's two cells


class Slab:
    """Cells [z0, z1) owned by `rank`; the closed box spans [zlo, zhi)."""

    def __init__(self, rank, world, res, z0, z1, zlo, zhi, guard):
        self.rank, self.world, self.res = rank, world, res
        self.z0, self.z1, self.zlo, self.zhi, self.guard = z0, z1, zlo, zhi, guard

    @property
    def depth(self):
        return self.zhi - self.zlo

    def __repr__(self):
        return "Slab(rank=%d, own=[%d,%d), box=[%d,%d))" % (self.rank, self.z0, self.z1, self.zlo, self.zhi)


def plan_slabs(res, world, rmax, bilateral_iters=20):
    """Owned ranges (multiples of 16 cells, as even as that allows) and
    boxes.  The guard band (cells of triangles kept for the normals) is
    iters + 2 cells: a vertex normal reads the triangles of its fine cube,
    and one bilateral iteration reaches one ring of neighbours, at most a
    fine-cube diagonal (< 1 cell) away."""
    if res % 16 or world < 1 or res // 16 < world:
        raise ValueError("res must be a multiple of 16 with at least 16 cells per rank")
    guard = int(bilateral_iters) + 2
    halo = rmax + HALO_SPARE + guard
    units = res // 16
    bounds = [16 * ((units * k) // world) for k in range(world + 1)]
    slabs = []
    for k in range(world):
        z0, z1 = bounds[k], bounds[k + 1]
        zlo = max(0, (z0 - halo) // 16 * 16)
        zhi = min(res, -(-(z1 + halo) // 16) * 16)
        slabs.append(Slab(k, world, res, z0, z1, zlo, zhi, guard))
    return slabs


def _lattice_z(V, bz, cs_f):
    """Fine-lattice z of each vertex's owning cube: vertices on z edges sit at
    k + 0.05 or k + 0.95 (iso 0.95 between binary corners), the others on
    the lattice plane k."""
    zf = (V[:, 2].astype(np.float64) - bz) / cs_f
    r = np.rint(zf)
    on_plane = np.abs(zf - r) < 0.01
    return np.where(on_plane, r, np.floor(zf)).astype(np.int64)


def _pos_keys(V):
    return np.ascontiguousarray(V, np.float32).view(np.uint32).reshape(-1, 3)


def local_mesh(slab, V, N, T, bbox_min_z, cell_size):
    """Keep the triangles emitted by the slab's owned cells and classify the
    vertices.  V, N, T: the window mesh of the slab (global coordinates).
    Returns a dict with the kept mesh (local ids), the owned-vertex mask and
    this rank's first-layer table (positions, local ids)."""
    cs_f = 0.5 * cell_size
    vz = _lattice_z(V, bbox_min_z, cs_f)       # cube z of each vertex
    vcell = np.floor_divide(vz, 2)              # its cell
    # emitting cube of a triangle: the smallest cube z over its vertices.
    # The reference's triangles next to untagged border cubes take vertex 0
    # for the missing edges; such triangles span more than one cube and are
    # not carried over (they are not part of a well-formed surface).
    if len(T):
        tz = vz[T]
        tcell = np.floor_divide(tz.min(axis=1), 2)
        formed = tz.max(axis=1) - tz.min(axis=1) <= 1
    else:
        tcell = np.zeros(0, np.int64)
        formed = np.zeros(0, bool)
    keep_t = (tcell >= slab.z0) & (tcell < slab.z1) & formed
    Tk = T[keep_t]
    used = np.zeros(len(V), bool)
    used[Tk.reshape(-1)] = True
    ids = np.flatnonzero(used)
    remap = np.full(len(V), -1, np.int64)
    remap[ids] = np.arange(len(ids))
    Vk, Nk, Tk = V[ids], N[ids], remap[Tk]
    cell_k = vcell[ids]
    owned = (cell_k >= slab.z0) & (cell_k < slab.z1)
    first = owned & (cell_k == slab.z0)
    dropped = int(((tcell >= slab.z0) & (tcell < slab.z1) & ~formed).sum())
    return {"V": Vk, "N": Nk, "T": Tk, "owned": owned, "cell": cell_k, "dropped": dropped,
            "first_keys": _pos_keys(Vk[first]), "first_ids": np.flatnonzero(first)}


def seam_table(part):
    """What this rank contributes to the exchange: its owned vertex count and
    the positions and owned-order ids of its first cell layer's vertices."""
    owned = part["owned"]
    own_ids = np.flatnonzero(owned)
    own_pos = np.full(len(owned), -1, np.int64)
    own_pos[own_ids] = np.arange(len(own_ids))
    return (len(own_ids), part["first_keys"], own_pos[part["first_ids"]])


def stitch_apply(slab, part, tables):
    """(V, N, T) of this rank's owned vertices with global vertex ids, from
    every rank's seam_table (the concatenation over ranks in rank order is
    the whole mesh)."""
    owned = part["owned"]
    own_ids = np.flatnonzero(owned)
    offsets = np.concatenate([[0], np.cumsum([t[0] for t in tables])])
    gid = np.full(len(owned), -1, np.int64)
    gid[own_ids] = offsets[slab.rank] + np.arange(len(own_ids))
    seam = np.flatnonzero(~owned)
    if len(seam):
        if slab.rank + 1 >= slab.world:
            raise RuntimeError("vertices past the last slab")
        _, keys_up, pos_up = tables[slab.rank + 1]
        lookup = {k.tobytes(): int(q) for k, q in zip(keys_up, pos_up)}
        for i, k in zip(seam, _pos_keys(part["V"][seam])):
            q = lookup.get(k.tobytes())
            if q is None:
                raise RuntimeError("seam vertex without owner in rank %d" % (slab.rank + 1))
            gid[i] = offsets[slab.rank + 1] + q
    return part["V"][own_ids], part["N"][own_ids], gid[part["T"]]


def stitch(slab, part, group):
    """The exchange over a group (``allgather(obj)``), then stitch_apply."""
    return stitch_apply(slab, part, group.allgather(seam_table(part)))


def stitch_local(slabs, parts):
    """All ranks in one process: the exchange is a list."""
    tables = [seam_table(p) for p in parts]
    return [stitch_apply(s, p, tables) for s, p in zip(slabs, parts)]


class TorchGroup:
    """allgather over torch.distributed (any backend)."""

    def __init__(self, group=None):
        self.group = group

    def allgather(self, obj):
        import torch.distributed as dist
        out = [None] * dist.get_world_size(self.group)
        dist.all_gather_object(out, obj, group=self.group)
        return out


def close_mesh_slab(ctx, slab, desc, X, R=None, uniform_radius=4, mode=0, se=0, bilateral_iters=20):
    """GPU work of one rank.  X (R): this rank's slab of the packed grid
    (radius field), cells [zlo, zhi) along z, whole x and y.  Returns the
    closing of the owned cells (torch, uint8 (z1-z0) * res * res) and the
    window mesh as host arrays (global coordinates)."""
    import torch
    from . import _lib as L
    from .api import make_box
    res = slab.res
    dr = [desc.data_res[0], desc.data_res[1], min(max(desc.data_res[2] - slab.zlo, 0), slab.depth)]
    box = make_box((res, res, slab.depth), dr, bbox_min=tuple(desc.bbox_min), cell_size=desc.cell_size)
    # only the mesh window and the two cells its cubes read around it are
    # closed; the rest of the box is the halo the closing reads
    zr0 = max(slab.z0 - slab.guard - 2, slab.zlo) - slab.zlo
    zr1 = min(slab.z1 + slab.guard + 2, slab.zhi) - slab.zlo
    Cb = ctx.close_box_region(box, X, (0, 0, zr0), (res, res, zr1), R, uniform_radius, mode, se)
    win = L.MeshWindow()
    win.global_res = res
    for a in range(3):
        win.origin[a] = 0 if a < 2 else slab.zlo
        win.emit_lo[a] = 0 if a < 2 else max(slab.z0 - slab.guard, 0) - slab.zlo
        win.emit_hi[a] = res if a < 2 else min(slab.z1 + slab.guard, res) - slab.zlo
    V, N, T = ctx.mesh_box(box, Cb, bilateral_iters, window=win)
    own = Cb.view(slab.depth, res, res)[slab.z0 - slab.zlo:slab.z1 - slab.zlo].clone()
    Th = T.view(torch.int32).cpu().numpy().astype(np.int64)
    return own, V.cpu().numpy(), N.cpu().numpy(), Th
