"""Python loader of the CPU oracle (gm_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU baseline leg of bench.py, never by the product package.  See gm_oracle.h
for what each function restates and its parity status (pinned to the
reference GMorpho built from its own sources, tests/test_oracle_ref.py, and
to a float transliteration of the reference traversal kernels on small
grids).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgmoracle.so")
SRC = os.path.join(HERE, "gm_oracle.c")
HDR = os.path.join(HERE, "gm_oracle.h")
TABLES = os.path.join(os.path.dirname(HERE), "broxy_gb300", "csrc", "mc_tables.inc")


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    deps = [SRC, HDR, TABLES]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(d) > os.path.getmtime(LIB) for d in deps):
        cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-o", LIB, SRC, "-lm"]
        subprocess.run(cmd, check=True)
    return LIB


_lib = None
_u8p = C.POINTER(C.c_uint8)
_i8p = C.POINTER(C.c_int8)
_u64p = C.POINTER(C.c_uint64)
_f32p = C.POINTER(C.c_float)
_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.gmo_pyramid_size.restype = C.c_int64
        L.gmo_pyramid_size.argtypes = [C.c_int]
        L.gmo_pyramid_build.argtypes = [_u8p, _i8p, C.c_int, _u64p]
        L.gmo_dilate_query.argtypes = [_u64p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.gmo_erode_query2.argtypes = [_u64p, C.c_int, C.c_int, C.c_int, C.c_int]
        L.gmo_dilate_query_brute.argtypes = [_u8p, _i8p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.gmo_erode_query2_brute.argtypes = [_u8p, _i8p, C.c_int, C.c_int, C.c_int, C.c_int]
        L.gmo_close.argtypes = [_u8p, _i8p, C.c_int, _i32p, C.c_int, C.c_int, _u8p, _u8p, _u8p]
        L.gmo_close_lists.argtypes = [_u8p, _i8p, C.c_int, _i32p, C.c_int, C.c_int, _u8p, _u8p, _u8p, _i64p]
        L.gmo_close_exact_brute.argtypes = [_u8p, _i8p, C.c_int, C.c_int, _u8p]
        L.gmo_mc.argtypes = [_u8p, C.c_int, _f32p, C.c_float, C.c_float, _f32p, C.c_int64, _u32p, C.c_int64,
                             _i64p, _i64p]
        L.gmo_normals.argtypes = [_f32p, C.c_int64, _u32p, C.c_int64, C.c_int, _f32p]
        L.gmo_scale_brush.argtypes = [_i8p, C.c_int, _f32p, C.c_float, _f32p, C.c_float, C.c_float, C.c_float,
                                      C.c_int]
        L.gmo_grid_attributes.argtypes = [_f32p, C.c_int64, C.c_int, C.c_float, _f32p, _f32p, _f32p, _i32p]
        L.gmo_voxelize.argtypes = [_f32p, C.c_int64, _u32p, C.c_int64, C.c_int, _f32p, C.c_float, _u8p]
        L.gmo_rotcube_frame.argtypes = [_f32p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _f32p]
        L.gmo_rotcube_query.argtypes = [_u64p, C.c_int, _f32p, C.c_int] + [C.c_int] * 8
        L.gmo_close_rotcube.argtypes = [_u8p, _i8p, C.c_int, _i32p, _f32p, C.c_int, C.c_int, _u8p, _u8p, _u8p]
        L.gmo_morton3.restype = C.c_uint32
        L.gmo_morton3.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def scale_grid(res, scale=None, uniform=None):
    n = 2 * res
    if scale is not None:
        return _c(scale, np.int8).reshape(-1)
    return np.full(n * n * n, uniform, dtype=np.int8)


def pyramid(grid, res, scale):
    out = np.zeros(lib().gmo_pyramid_size(res), dtype=np.uint64)
    lib().gmo_pyramid_build(_p(_c(grid, np.uint8), _u8p), _p(_c(scale, np.int8), _i8p), res, _p(out, _u64p))
    return out


def close(X, res, data_res, scale, mode=0, se=0):
    """GM_REF (mode 0) or GM_EXACT (mode 1) closing; returns (D, S, C)."""
    X = _c(X, np.uint8).reshape(-1)
    scale = _c(scale, np.int8).reshape(-1)
    D = np.zeros(res ** 3, np.uint8)
    S = np.zeros(res ** 3, np.uint8)
    Cg = np.zeros(res ** 3, np.uint8)
    dr = np.asarray(data_res, dtype=np.int32)
    rc = lib().gmo_close(_p(X, _u8p), _p(scale, _i8p), res, _p(dr, _i32p), mode, se, _p(D, _u8p), _p(S, _u8p),
                         _p(Cg, _u8p))
    assert rc == 0
    return D, S, Cg


def close_lists(X, res, data_res, scale, se=0):
    """GM_REF closing; returns (D, S, C, (tight dilation list size, base
    erosion list size)): the work lists of the reference's refinement
    kernels."""
    X = _c(X, np.uint8).reshape(-1)
    scale = _c(scale, np.int8).reshape(-1)
    D = np.zeros(res ** 3, np.uint8)
    S = np.zeros(res ** 3, np.uint8)
    Cg = np.zeros(res ** 3, np.uint8)
    lists = np.zeros(2, np.int64)
    dr = np.asarray(data_res, dtype=np.int32)
    rc = lib().gmo_close_lists(_p(X, _u8p), _p(scale, _i8p), res, _p(dr, _i32p), 0, se, _p(D, _u8p), _p(S, _u8p),
                               _p(Cg, _u8p), _p(lists, _i64p))
    assert rc == 0
    return D, S, Cg, (int(lists[0]), int(lists[1]))


def close_rotcube(X, res, data_res, scale, quats, qres, mode=0):
    """Rotated-cube dilation under the quaternion field `quats` ((qres^3, 4)
    float32, x y z w) then the sphere erosion; returns (D, S, C)."""
    X = _c(X, np.uint8).reshape(-1)
    scale = _c(scale, np.int8).reshape(-1)
    Q = _c(quats, np.float32).reshape(-1)
    assert Q.size == 4 * qres ** 3
    D = np.zeros(res ** 3, np.uint8)
    S = np.zeros(res ** 3, np.uint8)
    Cg = np.zeros(res ** 3, np.uint8)
    dr = np.asarray(data_res, dtype=np.int32)
    rc = lib().gmo_close_rotcube(_p(X, _u8p), _p(scale, _i8p), res, _p(dr, _i32p), _p(Q, _f32p), qres, mode,
                                 _p(D, _u8p), _p(S, _u8p), _p(Cg, _u8p))
    assert rc == 0
    return D, S, Cg


def rotcube_frame(quats, qres, i, res):
    """The rotated axes (3, 3) = b_x, b_y, b_z at lattice point i of a grid
    of `res` points per axis."""
    Q = _c(quats, np.float32).reshape(-1)
    out = np.zeros(9, np.float32)
    lib().gmo_rotcube_frame(_p(Q, _f32p), qres, int(i[0]), int(i[1]), int(i[2]), res, _p(out, _f32p))
    return out.reshape(3, 3)


def close_exact_brute(X, res, scale, se=0):
    X = _c(X, np.uint8).reshape(-1)
    scale = _c(scale, np.int8).reshape(-1)
    Cg = np.zeros(res ** 3, np.uint8)
    assert lib().gmo_close_exact_brute(_p(X, _u8p), _p(scale, _i8p), res, se, _p(Cg, _u8p)) == 0
    return Cg


def mc(Cgrid, res, bbox_min, cell_size, iso=0.95):
    Cgrid = _c(Cgrid, np.uint8).reshape(-1)
    bm = _c(bbox_min, np.float32)
    nv = C.c_int64(0)
    nt = C.c_int64(0)
    L = lib()
    L.gmo_mc(_p(Cgrid, _u8p), res, _p(bm, _f32p), cell_size, iso, None, 0, None, 0, C.byref(nv), C.byref(nt))
    V = np.zeros((max(nv.value, 1), 3), np.float32)
    T = np.zeros((max(nt.value, 1), 3), np.uint32)
    rc = L.gmo_mc(_p(Cgrid, _u8p), res, _p(bm, _f32p), cell_size, iso, _p(V, _f32p), nv.value, _p(T, _u32p),
                  nt.value, C.byref(nv), C.byref(nt))
    assert rc == 0
    return V[:nv.value], T[:nt.value]


def normals(V, T, iters):
    V = _c(V, np.float32)
    T = _c(T, np.uint32)
    N = np.zeros_like(V)
    lib().gmo_normals(_p(V, _f32p), len(V), _p(T, _u32p), len(T), iters, _p(N, _f32p))
    return N


def scale_brush(scale, n, bbox_min, cell_size, pos, value, support, global_scale, mode):
    out = _c(scale, np.int8).copy()
    lib().gmo_scale_brush(_p(out, _i8p), n, _p(_c(bbox_min, np.float32), _f32p), cell_size,
                          _p(_c(pos, np.float32), _f32p), value, support, global_scale, mode)
    return out


def grid_attributes(P, base_res, margin):
    P = _c(P, np.float32)
    bmin = np.zeros(3, np.float32)
    bmax = np.zeros(3, np.float32)
    cell = np.zeros(1, np.float32)
    dr = np.zeros(3, np.int32)
    lib().gmo_grid_attributes(_p(P, _f32p), len(P), base_res, margin, _p(bmin, _f32p), _p(bmax, _f32p),
                              _p(cell, _f32p), _p(dr, _i32p))
    return bmin, bmax, float(cell[0]), dr


def voxelize(P, T, res, bbox_min, cell_size):
    P = _c(P, np.float32)
    T = _c(T, np.uint32)
    g = np.zeros(res ** 3, np.uint8)
    lib().gmo_voxelize(_p(P, _f32p), len(P), _p(T, _u32p), len(T), res, _p(_c(bbox_min, np.float32), _f32p),
                       cell_size, _p(g, _u8p))
    return g


def morton3(x, y, z):
    return lib().gmo_morton3(x, y, z)


def dilate_query(pyr, res, se, p, radius):
    return lib().gmo_dilate_query(_p(pyr, _u64p), res, se, int(p[0]), int(p[1]), int(p[2]), radius)


def erode_query2(pyr, res, q2):
    return lib().gmo_erode_query2(_p(pyr, _u64p), res, int(q2[0]), int(q2[1]), int(q2[2]))


def dilate_query_brute(grid, scale, res, se, p, radius):
    return lib().gmo_dilate_query_brute(_p(_c(grid, np.uint8), _u8p), _p(_c(scale, np.int8), _i8p), res, se,
                                        int(p[0]), int(p[1]), int(p[2]), radius)


def erode_query2_brute(grid, scale, res, q2):
    return lib().gmo_erode_query2_brute(_p(_c(grid, np.uint8), _u8p), _p(_c(scale, np.int8), _i8p), res,
                                        int(q2[0]), int(q2[1]), int(q2[2]))
