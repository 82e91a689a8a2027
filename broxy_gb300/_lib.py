"""ctypes binding of the C ABI in include/gmorpho_gb300.h.

The library is the product: there is no Python or CPU fallback.  Loading
fails loudly when ``libgmorpho_gb300.so`` has not been built.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libgmorpho_gb300.so")

GM_OK = 0
GM_ERR_INVALID_ARGUMENT = 1
GM_ERR_CUDA = 2
GM_ERR_OUT_OF_MEMORY = 3
GM_ERR_UNSUPPORTED = 4
GM_ERR_CAPACITY = 5
GM_ERR_NOT_READY = 6

GM_REF, GM_EXACT = 0, 1
GM_SE_SPHERE, GM_SE_CUBE = 0, 1
GM_BATCH_GROUPED = -1  # batch form: one persistent launch per min-plus pass for all grids
GM_BRUSH_MAX, GM_BRUSH_MIN, GM_BRUSH_ZERO = 1, 2, 3


class GridDesc(C.Structure):
    _fields_ = [("bbox_min", C.c_float * 3), ("bbox_max", C.c_float * 3), ("res", C.c_int32),
                ("data_res", C.c_int32 * 3), ("cell_size", C.c_float)]


class MeshView(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("normals", C.c_void_p), ("triangles", C.c_void_p),
                ("num_vertices", C.c_int64), ("num_triangles", C.c_int64)]


class BoxDesc(C.Structure):
    _fields_ = [("bbox_min", C.c_float * 3), ("cell_size", C.c_float), ("dims", C.c_int32 * 3),
                ("data_res", C.c_int32 * 3)]


class MeshWindow(C.Structure):
    _fields_ = [("origin", C.c_int32 * 3), ("global_res", C.c_int32), ("emit_lo", C.c_int32 * 3),
                ("emit_hi", C.c_int32 * 3)]


class BatchItem(C.Structure):
    _fields_ = [("desc", GridDesc), ("d_input", C.c_void_p), ("d_scale", C.c_void_p), ("uniform_radius", C.c_int32),
                ("d_closing", C.c_void_p)]


class ServerOpts(C.Structure):
    _fields_ = [("slots", C.c_int32), ("max_crop_res", C.c_int32), ("rmax", C.c_int32), ("mode", C.c_int32),
                ("bilateral_iters", C.c_int32)]


class Edit(C.Structure):
    _fields_ = [("center", C.c_float * 3), ("scale", C.c_float), ("support", C.c_float),
                ("global_scale", C.c_float), ("mode", C.c_int32)]


class EditResult(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("status", C.c_int32), ("latency_ms", C.c_float), ("device_ms", C.c_float),
                ("dirty_lo", C.c_int32 * 3), ("dirty_hi", C.c_int32 * 3), ("crop_res", C.c_int32),
                ("patch", MeshView)]


class UpdateOpts(C.Structure):
    _fields_ = [("use_asymmetric_closing", C.c_int32), ("bilateral_filtering", C.c_int32), ("mode", C.c_int32)]


# name -> (restype, argtypes); every symbol of gmorpho_gb300.h
_P = C.c_void_p
PROTOTYPES = {
    "gm_status_string": (C.c_char_p, [C.c_int]),
    "gm_abi_version": (C.c_int, []),
    "gm_ctx_create": (C.c_int, [C.c_int, C.POINTER(_P)]),
    "gm_ctx_destroy": (C.c_int, [_P]),
    "gm_ctx_last_error": (C.c_char_p, [_P]),
    "gm_ctx_kernel_launches": (C.c_longlong, [_P]),
    "gm_kernel_error_flags": (C.c_int, [C.POINTER(C.c_uint32), C.c_int32]),
    "gm_ctx_profile": (C.c_int, [_P, C.c_int32]),
    "gm_ctx_profile_reset": (C.c_int, [_P]),
    "gm_ctx_profile_read": (C.c_int64, [_P, C.c_char_p, C.c_int64]),
    "gm_grid_attributes": (C.c_int, [_P, C.c_int64, C.c_int32, C.c_float, C.POINTER(GridDesc)]),
    "gm_voxelize": (C.c_int, [_P, C.POINTER(GridDesc), _P, C.c_int64, _P, C.c_int64, _P, _P]),
    "gm_scalefield_fill": (C.c_int, [_P, _P, C.c_int64, C.c_int32, _P]),
    "gm_scalefield_brush": (C.c_int, [_P, _P, C.c_int32, _P, C.c_float, _P, C.c_float, C.c_float, C.c_float,
                                      C.c_int, _P]),
    "gm_pyramid_texels": (C.c_int64, [C.c_int32]),
    "gm_pyramid_build": (C.c_int, [_P, C.POINTER(GridDesc), _P, _P, C.c_int32, _P, _P]),
    "gm_close": (C.c_int, [_P, C.POINTER(GridDesc), _P, _P, C.c_int32, C.c_int, C.c_int, _P, _P, _P, _P]),
    "gm_close_noalloc": (C.c_int, [C.POINTER(GridDesc), _P, _P, C.c_int32, C.c_int, C.c_int, _P, _P, _P, _P]),
    "gm_contour": (C.c_int, [_P, C.POINTER(GridDesc), _P, _P, C.c_int, _P]),
    "gm_mesh": (C.c_int, [_P, C.POINTER(GridDesc), _P, C.c_int32, C.POINTER(MeshView), _P]),
    "gm_update": (C.c_int, [_P, C.POINTER(GridDesc), _P, _P, C.c_float, C.POINTER(UpdateOpts),
                            C.POINTER(C.c_int64), C.POINTER(C.c_int64), _P]),
    "gm_update_to_host": (C.c_int, [_P, C.POINTER(GridDesc), _P, _P, C.c_float, C.POINTER(UpdateOpts), _P, _P, _P,
                                    C.c_int64, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64), _P]),
    "gm_mesh_download": (C.c_int, [_P, _P, _P, _P, _P]),
    "gm_batch_close_mesh": (C.c_int, [_P, C.c_int32, C.POINTER(BatchItem), C.c_int, C.c_int, C.c_int32, C.c_int32,
                                       C.POINTER(MeshView), _P]),
    "gm_batch_lanes": (C.c_int32, [_P]),
    "gm_batch_inject_alloc_failures": (C.c_int, [_P, C.c_int32]),
    "gm_server_create": (C.c_int, [C.POINTER(GridDesc), _P, _P, C.POINTER(ServerOpts), C.POINTER(_P)]),
    "gm_server_destroy": (C.c_int, [_P]),
    "gm_server_submit": (C.c_int, [_P, C.POINTER(Edit), C.POINTER(C.c_uint64)]),
    "gm_server_poll": (C.c_int, [_P, C.POINTER(EditResult), C.c_int32, C.POINTER(C.c_int32)]),
    "gm_server_pending": (C.c_int32, [_P]),
    "gm_server_closing": (C.c_void_p, [_P]),
    "gm_server_kernel_launches": (C.c_longlong, [_P]),
    "gm_server_set_admission": (C.c_int, [_P, C.c_int64, C.c_float]),
    "gm_server_memory": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "gm_server_inject_alloc_failures": (C.c_int, [_P, C.c_int32]),
    "gm_server_profile": (C.c_int, [_P, C.c_int32]),
    "gm_server_snapshot": (C.c_int, [_P, _P, _P]),
    "gm_server_restore": (C.c_int, [_P, _P, _P]),
    "gm_close_box": (C.c_int, [_P, C.POINTER(BoxDesc), _P, _P, C.c_int32, C.c_int, C.c_int, _P, _P]),
    "gm_close_box_region": (C.c_int, [_P, C.POINTER(BoxDesc), _P, _P, C.c_int32, C.c_int, C.c_int,
                                      C.POINTER(C.c_int32), C.POINTER(C.c_int32), _P, _P]),
    "gm_mesh_box": (C.c_int, [_P, C.POINTER(BoxDesc), _P, C.POINTER(MeshWindow), C.c_int32, C.POINTER(MeshView), _P]),
    "gm_mesh_store": (C.c_int, [C.c_char_p, _P, _P, C.c_int64, _P, C.c_int64, C.c_int32]),
    "gm_server_profile_read": (C.c_int64, [_P, C.c_char_p, C.c_int64]),
    "gm_bvh_build": (C.c_int, [_P, C.POINTER(GridDesc), _P, C.POINTER(_P), C.POINTER(C.c_int64), _P]),
    "gm_bvh_destroy": (C.c_int, [_P]),
    "gm_bvh_query": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int32, _P, _P]),
    "gm_bvh_leaves": (C.c_int, [_P, _P, _P, _P]),
    "gm_erode_bvh": (C.c_int, [_P, C.POINTER(GridDesc), _P, _P, C.c_int32, _P, _P]),
    "gm_layout_zwords_to_packed": (C.c_int, [_P, C.c_int32, _P, _P, _P]),
    "gm_layout_packed_to_zwords": (C.c_int, [_P, C.c_int32, _P, _P, _P]),
    "gm_close_rotcube": (C.c_int, [_P, C.POINTER(GridDesc), _P, _P, C.c_int32, _P, C.c_int32, C.c_int, _P, _P, _P,
                                   _P]),
    "gm_frame_field_create": (C.c_int, [_P, _P, _P, C.c_int32, C.POINTER(_P)]),
    "gm_frame_field_destroy": (C.c_int, [_P]),
    "gm_frame_field_add_point": (C.c_int, [_P, _P, _P]),
    "gm_frame_field_update_point": (C.c_int, [_P, C.c_int32, _P]),
    "gm_frame_field_num_points": (C.c_int32, [_P]),
    "gm_frame_field_get_point": (C.c_int, [_P, C.c_int32, _P, _P]),
    "gm_frame_field_generate": (C.c_int, [_P, C.POINTER(C.c_int32), _P]),
    "gm_frame_field_quats": (C.c_int, [_P, C.POINTER(_P), C.POINTER(C.c_int32)]),
    "gm_rotation_to_twist": (C.c_int, [_P, _P, _P, _P]),
}

_lib = None


def load(path=LIB_PATH):
    """Load the CUDA library once; raise when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libgmorpho_gb300.so is not built (%s); run __graft_entry__.build() "
                           "or python broxy_gb300/build.py" % path)
    lib = C.CDLL(path)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class GMError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (status %d): %s" % (load().gm_status_string(status).decode(), status, msg))
        self.status = status


def check(ctx, status):
    if status != GM_OK:
        msg = load().gm_ctx_last_error(ctx).decode() if ctx else ""
        raise GMError(status, msg)
