"""Functional Python API over the C ABI (include/gmorpho_gb300.h).

Device buffers are torch CUDA tensors (torch is only the allocator and the
stream provider here); every computation runs in libgmorpho_gb300.so.
"""
import ctypes as C

import numpy as np

from . import _lib as L


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class DevicePtrArray:
    """Zero-copy view of a device buffer owned by the library
    (__cuda_array_interface__), e.g. the mesh of a context."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (ptr or 0, False),
                                         "version": 3, "strides": None}


def kernel_error_flags(clear=False):
    """Error bits this library's kernels recorded on the current device
    (bit 0: a TMA tile load not complete within its poll limit)."""
    f = C.c_uint32(0)
    L.check(None, L.load().gm_kernel_error_flags(C.byref(f), 1 if clear else 0))
    return int(f.value)


def make_desc(res, data_res=None, bbox_min=(0.0, 0.0, 0.0), cell_size=None):
    d = L.GridDesc()
    cs = cell_size if cell_size is not None else 1.0 / res
    for a in range(3):
        d.bbox_min[a] = bbox_min[a]
        d.bbox_max[a] = bbox_min[a] + cs * res
        d.data_res[a] = res if data_res is None else int(data_res[a])
    d.res = res
    d.cell_size = cs
    return d


def make_box(dims, data_res=None, bbox_min=(0.0, 0.0, 0.0), cell_size=1.0):
    b = L.BoxDesc()
    for a in range(3):
        b.bbox_min[a] = bbox_min[a]
        b.dims[a] = int(dims[a])
        b.data_res[a] = int(dims[a] if data_res is None else data_res[a])
    b.cell_size = cell_size
    return b


def grid_attributes(points, base_res, margin):
    P = np.ascontiguousarray(points, dtype=np.float32)
    d = L.GridDesc()
    st = L.load().gm_grid_attributes(P.ctypes.data_as(C.c_void_p), len(P), base_res, margin, C.byref(d))
    L.check(None, st)
    return d


class Context:
    """One device context (cached workspaces + last mesh)."""

    def __init__(self, device=0):
        import torch
        torch.cuda.init()
        self.lib = L.load()
        self.ctx = C.c_void_p()
        st = self.lib.gm_ctx_create(device, C.byref(self.ctx))
        if st != L.GM_OK:
            raise L.GMError(st, "gm_ctx_create(%d)" % device)
        self.device = device

    def close_ctx(self):
        if self.ctx:
            self.lib.gm_ctx_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close_ctx()
        except Exception:
            pass

    @property
    def kernel_launches(self):
        return int(self.lib.gm_ctx_kernel_launches(self.ctx))

    def _check(self, st):
        L.check(self.ctx, st)

    def profile(self, enable=True):
        """Per-kernel CUDA-event timing of every launch on this context."""
        self._check(self.lib.gm_ctx_profile(self.ctx, 1 if enable else 0))

    def profile_reset(self):
        self._check(self.lib.gm_ctx_profile_reset(self.ctx))

    def profile_read(self):
        import json
        n = self.lib.gm_ctx_profile_read(self.ctx, None, 0)
        buf = C.create_string_buffer(int(n))
        self.lib.gm_ctx_profile_read(self.ctx, buf, n)
        return json.loads(buf.value.decode())

    # a5..a11
    def close(self, desc, X, R=None, uniform_radius=4, mode=L.GM_REF, se=L.GM_SE_SPHERE, out=None, D=None, S=None):
        import torch
        if out is None:
            out = torch.empty_like(X)
        st = self.lib.gm_close(self.ctx, C.byref(desc), _ptr(X), _ptr(R), int(uniform_radius), mode, se, _ptr(out),
                               _ptr(D), _ptr(S), _stream())
        self._check(st)
        return out

    # f2: GMorpho::Update with a frame field
    def close_rotcube(self, desc, X, quats, quat_res, R=None, uniform_radius=4, mode=L.GM_REF, out=None, D=None,
                      S=None):
        """Rotated-cube dilation under the quaternion field `quats` (device,
        (quat_res^3, 4) float32 x y z w, e.g. FrameField.quats()) then the
        sphere erosion."""
        import torch
        if out is None:
            out = torch.empty_like(X)
        self._check(self.lib.gm_close_rotcube(self.ctx, C.byref(desc), _ptr(X), _ptr(R), int(uniform_radius),
                                              _ptr(quats), int(quat_res), mode, _ptr(out), _ptr(D), _ptr(S),
                                              _stream()))
        return out

    # a8
    def contour(self, desc, grid, mode=L.GM_REF, inplace=False):
        import torch
        out = grid if inplace else torch.empty_like(grid)
        self._check(self.lib.gm_contour(self.ctx, C.byref(desc), _ptr(grid), _ptr(out), mode, _stream()))
        return out

    # box grids (slabs, crops, non-power-of-two instances)
    def close_box(self, box, X, R=None, uniform_radius=4, mode=L.GM_REF, se=L.GM_SE_SPHERE, out=None):
        import torch
        if out is None:
            out = torch.empty_like(X)
        self._check(self.lib.gm_close_box(self.ctx, C.byref(box), _ptr(X), _ptr(R), int(uniform_radius), mode, se,
                                          _ptr(out), _stream()))
        return out

    def close_box_region(self, box, X, roi_lo, roi_hi, R=None, uniform_radius=4, mode=L.GM_REF,
                         se=L.GM_SE_SPHERE, out=None):
        """The closing on cells [roi_lo, roi_hi) of the box only (other cells
        of `out` are unspecified)."""
        import torch
        if out is None:
            out = torch.empty_like(X)
        lo = (C.c_int32 * 3)(*[int(v) for v in roi_lo])
        hi = (C.c_int32 * 3)(*[int(v) for v in roi_hi])
        self._check(self.lib.gm_close_box_region(self.ctx, C.byref(box), _ptr(X), _ptr(R), int(uniform_radius), mode,
                                                 se, lo, hi, _ptr(out), _stream()))
        return out

    def mesh_box(self, box, Cg, bilateral_iters=20, window=None):
        """window: None or L.MeshWindow.  Returns zero-copy (V, N, T) owned by
        the context until the next mesh-producing call."""
        import torch
        mv = L.MeshView()
        wp = C.byref(window) if window is not None else None
        self._check(self.lib.gm_mesh_box(self.ctx, C.byref(box), _ptr(Cg), wp, int(bilateral_iters), C.byref(mv),
                                         _stream()))
        nv, nt = mv.num_vertices, mv.num_triangles
        V = torch.as_tensor(DevicePtrArray(mv.vertices, (nv, 3), "<f4"), device="cuda")
        N = torch.as_tensor(DevicePtrArray(mv.normals, (nv, 3), "<f4"), device="cuda")
        T = torch.as_tensor(DevicePtrArray(mv.triangles, (nt, 3), "<u4"), device="cuda")
        return V, N, T

    # a12..a16
    def mesh(self, desc, Cg, bilateral_iters=20):
        """Returns (V, N, T) as zero-copy device arrays owned by the context
        (valid until the next mesh-producing call) and the counts."""
        import torch
        mv = L.MeshView()
        st = self.lib.gm_mesh(self.ctx, C.byref(desc), _ptr(Cg), int(bilateral_iters), C.byref(mv), _stream())
        self._check(st)
        nv, nt = mv.num_vertices, mv.num_triangles
        V = torch.as_tensor(DevicePtrArray(mv.vertices, (nv, 3), "<f4"), device="cuda")
        N = torch.as_tensor(DevicePtrArray(mv.normals, (nv, 3), "<f4"), device="cuda")
        T = torch.as_tensor(DevicePtrArray(mv.triangles, (nt, 3), "<u4"), device="cuda")
        return V, N, T

    def mesh_download(self, nv, nt):
        V = np.empty((nv, 3), np.float32)
        N = np.empty((nv, 3), np.float32)
        T = np.empty((nt, 3), np.uint32)
        st = self.lib.gm_mesh_download(self.ctx, V.ctypes.data_as(C.c_void_p), N.ctypes.data_as(C.c_void_p),
                                       T.ctypes.data_as(C.c_void_p), _stream())
        self._check(st)
        return V, N, T

    # a17
    def update(self, desc, h_X, h_R=None, global_scale=0.0, asymmetric=False, bilateral=True, mode=L.GM_REF):
        """GMorpho::Update from host buffers (numpy arrays or pinned tensors)."""
        o = L.UpdateOpts(1 if asymmetric else 0, 1 if bilateral else 0, mode)
        nv = C.c_int64(0)
        nt = C.c_int64(0)
        hx = C.c_void_p(h_X.data_ptr()) if hasattr(h_X, "data_ptr") else h_X.ctypes.data_as(C.c_void_p)
        hr = None
        if h_R is not None:
            hr = C.c_void_p(h_R.data_ptr()) if hasattr(h_R, "data_ptr") else h_R.ctypes.data_as(C.c_void_p)
        st = self.lib.gm_update(self.ctx, C.byref(desc), hx, hr, float(global_scale), C.byref(o), C.byref(nv),
                                C.byref(nt), _stream())
        self._check(st)
        return nv.value, nt.value

    def update_to_host(self, desc, h_X, h_R, global_scale, hV, hN, hT, asymmetric=False, bilateral=True,
                       mode=L.GM_REF):
        """Update from host buffers straight into host mesh buffers (pinned
        tensors or numpy arrays of shape (cap, 3)); returns (nv, nt)."""
        o = L.UpdateOpts(1 if asymmetric else 0, 1 if bilateral else 0, mode)
        nv = C.c_int64(0)
        nt = C.c_int64(0)

        def ptr(a):
            if a is None:
                return None
            return C.c_void_p(a.data_ptr()) if hasattr(a, "data_ptr") else a.ctypes.data_as(C.c_void_p)

        vcap = hV.shape[0] if hV is not None else (hN.shape[0] if hN is not None else 0)
        tcap = hT.shape[0] if hT is not None else 0
        st = self.lib.gm_update_to_host(self.ctx, C.byref(desc), ptr(h_X), ptr(h_R), float(global_scale), C.byref(o),
                                        ptr(hV), ptr(hN), ptr(hT), vcap, tcap, C.byref(nv), C.byref(nt), _stream())
        self._check(st)
        return nv.value, nt.value

    # a4
    def pyramid(self, desc, grid, R=None, uniform_radius=4):
        import torch
        n = self.lib.gm_pyramid_texels(desc.res)
        out = torch.empty(n, dtype=torch.int64, device=grid.device)
        st = self.lib.gm_pyramid_build(self.ctx, C.byref(desc), _ptr(grid), _ptr(R), int(uniform_radius), _ptr(out),
                                       _stream())
        self._check(st)
        return out

    # a3
    def scale_fill(self, R, value):
        self._check(self.lib.gm_scalefield_fill(self.ctx, _ptr(R), R.numel(), int(value), _stream()))

    def scale_brush(self, R, fine_res, bbox_min, cell_size, position, scale, support, global_scale, mode):
        bm = (C.c_float * 3)(*bbox_min)
        pos = (C.c_float * 3)(*position)
        self._check(self.lib.gm_scalefield_brush(self.ctx, _ptr(R), fine_res, bm, float(cell_size), pos, float(scale),
                                                 float(support), float(global_scale), int(mode), _stream()))

    # a2
    def voxelize(self, desc, P, T, out=None):
        import torch
        if out is None:
            out = torch.zeros(desc.res ** 3, dtype=torch.uint8, device=P.device)
        st = self.lib.gm_voxelize(self.ctx, C.byref(desc), _ptr(P), P.shape[0], _ptr(T), T.shape[0], _ptr(out),
                                  _stream())
        self._check(st)
        return out

    # batched closing + meshing of uneven grids
    def batch_close_mesh(self, items, mode=L.GM_REF, se=L.GM_SE_SPHERE, bilateral_iters=20, lanes=0, mesh=True):
        """items: list of (desc, X, R or None, uniform_radius, out).  Returns a
        list of (V, N, T) zero-copy device arrays (or None when mesh=False)."""
        import torch
        n = len(items)
        arr = (L.BatchItem * n)()
        for i, (desc, X, R, r, out) in enumerate(items):
            arr[i].desc = desc
            arr[i].d_input = X.data_ptr()
            arr[i].d_scale = R.data_ptr() if R is not None else None
            arr[i].uniform_radius = int(r)
            arr[i].d_closing = out.data_ptr()
        views = (L.MeshView * n)() if mesh else None
        self._check(self.lib.gm_batch_close_mesh(self.ctx, n, arr, mode, se, int(bilateral_iters), int(lanes),
                                                 views, _stream()))
        if not mesh:
            return None
        res = []
        for v in views:
            res.append((torch.as_tensor(DevicePtrArray(v.vertices, (v.num_vertices, 3), "<f4"), device="cuda"),
                        torch.as_tensor(DevicePtrArray(v.normals, (v.num_vertices, 3), "<f4"), device="cuda"),
                        torch.as_tensor(DevicePtrArray(v.triangles, (v.num_triangles, 3), "<u4"), device="cuda")))
        return res

    @property
    def batch_lanes(self):
        return int(self.lib.gm_batch_lanes(self.ctx))

    # a18
    def bvh_build(self, desc, sites):
        h = C.c_void_p()
        n = C.c_int64(0)
        self._check(self.lib.gm_bvh_build(self.ctx, C.byref(desc), _ptr(sites), C.byref(h), C.byref(n), _stream()))
        return BVH(self, h, n.value)

    def erode_bvh(self, desc, X, D, radius, out=None):
        import torch
        if out is None:
            out = torch.empty_like(D)
        self._check(self.lib.gm_erode_bvh(self.ctx, C.byref(desc), _ptr(X), _ptr(D), int(radius), _ptr(out),
                                          _stream()))
        return out

    def zwords_to_packed(self, res, zw, out):
        self._check(self.lib.gm_layout_zwords_to_packed(self.ctx, res, _ptr(zw), _ptr(out), _stream()))
        return out

    def packed_to_zwords(self, res, grid, out):
        self._check(self.lib.gm_layout_packed_to_zwords(self.ctx, res, _ptr(grid), _ptr(out), _stream()))
        return out


class BVH:
    """Handle of a device BVH (gm_bvh_*)."""

    def __init__(self, ctx, handle, n):
        self.ctx, self.handle, self.n = ctx, handle, n

    def query(self, points2, radius):
        import torch
        hits = torch.empty(points2.shape[0], dtype=torch.uint8, device=points2.device)
        self.ctx._check(self.ctx.lib.gm_bvh_query(self.ctx.ctx, self.handle, _ptr(points2), points2.shape[0],
                                                  int(radius), _ptr(hits), _stream()))
        return hits

    def leaves(self):
        import torch
        keys = torch.empty(max(self.n, 1), dtype=torch.int64, device="cuda")
        self.ctx._check(self.ctx.lib.gm_bvh_leaves(self.ctx.ctx, self.handle, _ptr(keys), _stream()))
        return keys[:self.n]

    def destroy(self):
        if self.handle:
            self.ctx.lib.gm_bvh_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class FrameField:
    """FrameField with the BiHarmonicSystem method (gm_frame_field_*): a
    quaternion per node of a res^3 lattice over the box, interpolating up to
    20 hard-constrained rotations."""

    def __init__(self, ctx, bbox_min, bbox_max, res):
        self.ctx = ctx
        self.res = int(res)
        h = C.c_void_p()
        lo = (C.c_float * 3)(*[float(v) for v in bbox_min])
        hi = (C.c_float * 3)(*[float(v) for v in bbox_max])
        ctx._check(ctx.lib.gm_frame_field_create(ctx.ctx, lo, hi, self.res, C.byref(h)))
        self.h = h

    def add_point(self, position, twist):
        p = (C.c_float * 3)(*[float(v) for v in position])
        t = (C.c_float * 3)(*[float(v) for v in twist])
        self.ctx._check(self.ctx.lib.gm_frame_field_add_point(self.h, p, t))

    def update_point(self, i, twist):
        t = (C.c_float * 3)(*[float(v) for v in twist])
        self.ctx._check(self.ctx.lib.gm_frame_field_update_point(self.h, int(i), t))

    def num_points(self):
        return int(self.ctx.lib.gm_frame_field_num_points(self.h))

    def point(self, i):
        g = (C.c_float * 3)()
        t = (C.c_float * 3)()
        self.ctx._check(self.ctx.lib.gm_frame_field_get_point(self.h, int(i), g, t))
        return tuple(g), tuple(t)

    def generate(self):
        """Solve the field; returns the solver's iteration count."""
        it = C.c_int32()
        self.ctx._check(self.ctx.lib.gm_frame_field_generate(self.h, C.byref(it), _stream()))
        return it.value

    def quats(self):
        """Zero-copy (res^3, 4) float32 device array, valid until the next
        generate or destroy."""
        import torch
        p = C.c_void_p()
        r = C.c_int32()
        self.ctx._check(self.ctx.lib.gm_frame_field_quats(self.h, C.byref(p), C.byref(r)))
        n = r.value ** 3
        return torch.as_tensor(DevicePtrArray(p.value, (n, 4), "<f4"), device="cuda")

    def destroy(self):
        if self.h:
            self.ctx.lib.gm_frame_field_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def rotation_to_twist(e_x, e_y, e_z):
    """FrameField::RotationToTwistCayley (gm_rotation_to_twist)."""
    lib = L.load()
    a = [(C.c_float * 3)(*[float(v) for v in e]) for e in (e_x, e_y, e_z)]
    out = (C.c_float * 3)()
    st = lib.gm_rotation_to_twist(a[0], a[1], a[2], out)
    if st != L.GM_OK:
        raise L.GMError(st, "gm_rotation_to_twist")
    return tuple(out)


class Server:
    """Resident-grid edit server (gm_server_*): brush edits with exact local
    re-closing and re-meshing, continuous batching over `slots`."""

    def __init__(self, desc, X, R, slots=4, max_crop_res=256, rmax=32, mode=L.GM_REF, bilateral_iters=0):
        """max_crop_res: largest crop edge in cells (a multiple of 16, or
        desc.res); an edit needing more is answered with GM_ERR_CAPACITY."""
        self.lib = L.load()
        self.desc, self.X, self.R = desc, X, R  # keep the device buffers alive
        opts = L.ServerOpts(slots, max_crop_res, rmax, mode, bilateral_iters)
        self.h = C.c_void_p()
        st = self.lib.gm_server_create(C.byref(desc), _ptr(X), _ptr(R), C.byref(opts), C.byref(self.h))
        if st != L.GM_OK:
            raise L.GMError(st, "gm_server_create")

    def submit(self, center, scale, support, global_scale=0.0, mode=L.GM_BRUSH_MAX):
        e = L.Edit((C.c_float * 3)(*center), float(scale), float(support), float(global_scale), int(mode))
        t = C.c_uint64(0)
        st = self.lib.gm_server_submit(self.h, C.byref(e), C.byref(t))
        if st != L.GM_OK:
            raise L.GMError(st, "gm_server_submit")
        return t.value

    def poll(self, cap=256):
        """Finished edits; a result's patch (device mesh) stays valid until the
        next poll."""
        arr = (L.EditResult * cap)()
        n = C.c_int32(0)
        st = self.lib.gm_server_poll(self.h, arr, cap, C.byref(n))
        if st != L.GM_OK:
            raise L.GMError(st, "gm_server_poll")
        out = []
        for r in arr[:n.value]:
            out.append(dict(ticket=r.ticket, status=r.status, latency_ms=r.latency_ms, device_ms=r.device_ms,
                            dirty_lo=tuple(r.dirty_lo), dirty_hi=tuple(r.dirty_hi), crop_res=r.crop_res,
                            patch_vertices=r.patch.num_vertices, patch_triangles=r.patch.num_triangles,
                            patch=r.patch))
        return out

    @property
    def pending(self):
        return int(self.lib.gm_server_pending(self.h))

    def drain(self):
        out = []
        while self.pending > 0:
            out += self.poll()
        out += self.poll()
        return out

    def closing(self):
        import torch
        p = self.lib.gm_server_closing(self.h)
        return torch.as_tensor(DevicePtrArray(p, (self.desc.res ** 3,), "|u1"), device="cuda")

    @property
    def kernel_launches(self):
        return int(self.lib.gm_server_kernel_launches(self.h))

    def set_admission(self, budget_bytes=0, timeout_ms=0.0):
        """Memory budget of the edits on the GPU (<= 0: keep) and the queue
        timeout in ms (0: none)."""
        st = self.lib.gm_server_set_admission(self.h, int(budget_bytes), float(timeout_ms))
        if st != L.GM_OK:
            raise L.GMError(st, "gm_server_set_admission")

    def memory(self):
        """(bytes of crop buffers of the edits on the GPU, budget)."""
        a, b = C.c_int64(0), C.c_int64(0)
        st = self.lib.gm_server_memory(self.h, C.byref(a), C.byref(b))
        if st != L.GM_OK:
            raise L.GMError(st, "gm_server_memory")
        return a.value, b.value

    def inject_alloc_failures(self, count):
        st = self.lib.gm_server_inject_alloc_failures(self.h, int(count))
        if st != L.GM_OK:
            raise L.GMError(st, "gm_server_inject_alloc_failures")

    def snapshot(self):
        """Host copies (closed grid, radius field) of the resident state."""
        n = self.desc.res ** 3
        C_ = np.empty(n, np.uint8)
        R_ = np.empty(8 * n, np.int8)
        st = self.lib.gm_server_snapshot(self.h, C_.ctypes.data, R_.ctypes.data)
        if st != L.GM_OK:
            raise L.GMError(st, "gm_server_snapshot")
        return C_, R_

    def restore(self, closing, scale):
        closing = np.ascontiguousarray(closing, np.uint8)
        scale = np.ascontiguousarray(scale, np.int8)
        st = self.lib.gm_server_restore(self.h, closing.ctypes.data, scale.ctypes.data)
        if st != L.GM_OK:
            raise L.GMError(st, "gm_server_restore")

    def export_patch(self, result, path, drop_unused=True):
        """Write an edit's patch (a poll() result) as OFF / PN / PLY."""
        import torch
        p = result["patch"]
        nv, nt = p.num_vertices, p.num_triangles

        def host(ptr, shape, typestr, dtype):
            if shape[0] == 0:
                return np.empty(shape, dtype)
            return torch.as_tensor(DevicePtrArray(ptr, shape, typestr), device="cuda").cpu().numpy().view(dtype)

        V = host(p.vertices, (nv, 3), "<f4", np.float32)
        N = host(p.normals, (nv, 3), "<f4", np.float32)
        T = host(p.triangles, (nt, 3), "<i4", np.uint32)
        store_mesh(path, V, N, T, drop_unused=drop_unused)

    def profile(self, enable=True):
        st = self.lib.gm_server_profile(self.h, 1 if enable else 0)
        if st != L.GM_OK:
            raise L.GMError(st, "gm_server_profile")

    def profile_read(self):
        import json
        need = self.lib.gm_server_profile_read(self.h, None, 0)
        buf = C.create_string_buffer(int(need))
        self.lib.gm_server_profile_read(self.h, buf, need)
        return json.loads(buf.value.decode())

    def destroy(self):
        if self.h:
            self.lib.gm_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def store_mesh(path, V, N, T, drop_unused=False):
    """Write a host mesh (float32 V/N (n, 3), uint32 T (m, 3)) as OFF, PN or
    PLY, by extension (gm_mesh_store)."""
    lib = L.load()
    V = np.ascontiguousarray(V, np.float32)
    T = np.ascontiguousarray(T, np.uint32)
    Np = None
    if N is not None:
        N = np.ascontiguousarray(N, np.float32)
        Np = N.ctypes.data
    st = lib.gm_mesh_store(str(path).encode(), V.ctypes.data if V.size else None, Np, V.shape[0],
                           T.ctypes.data if T.size else None, T.shape[0], 1 if drop_unused else 0)
    if st != L.GM_OK:
        raise L.GMError(st, "gm_mesh_store")
