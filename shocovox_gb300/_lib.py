"""ctypes loader of libsvo.so (built in-tree by shocovox_gb300/build.py).

Loading fails loudly: if the library cannot be built or loaded, every entry
point raises; nothing falls back to a CPU path.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

OP_DTYPE = np.dtype([("x", "<u2"), ("y", "<u2"), ("z", "<u2"), ("op", "u1"), ("kind", "u1"),
                     ("size", "<u4"), ("rgba", "<u4"), ("user", "<u4")])
assert OP_DTYPE.itemsize == 20

HIT_FIELDS = {
    "status": np.uint8, "brick_octant": np.uint8, "entry_kind": np.uint8, "node_key": np.uint32,
    "voxel_index": np.uint32, "pix": np.uint32, "albedo": np.uint32, "user": np.uint32,
    "px": np.float32, "py": np.float32, "pz": np.float32, "nx": np.float32, "ny": np.float32,
    "nz": np.float32, "node_visits": np.uint32, "child_reads": np.uint32, "voxel_reads": np.uint32,
    "run_visits": np.uint32,
}


class Rays(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in ("ox", "oy", "oz", "dx", "dy", "dz")]


class Hits(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in HIT_FIELDS]


class Viewport(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_float * 3), ("direction", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("width", ctypes.c_float), ("height", ctypes.c_float), ("fov", ctypes.c_float),
                ("light", ctypes.c_float * 3), ("background", ctypes.c_uint32)]


class SceneStats(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_uint64), ("reserved_nodes", ctypes.c_uint64), ("parted_bricks", ctypes.c_uint64),
                ("colors", ctypes.c_uint64), ("datas", ctypes.c_uint64), ("device_bytes", ctypes.c_uint64),
                ("size", ctypes.c_uint32), ("brick_dim", ctypes.c_uint32)]


class SceneRecipe(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("size", ctypes.c_uint32), ("brick_dim", ctypes.c_uint32),
                ("seed", ctypes.c_uint64), ("occupancy", ctypes.c_float), ("spheres", ctypes.c_uint32),
                ("octaves", ctypes.c_uint32), ("base_freq", ctypes.c_float), ("height_lo", ctypes.c_float),
                ("height_hi", ctypes.c_float), ("cave_threshold", ctypes.c_float)]


class LaunchConfig(ctypes.Structure):
    _fields_ = [("block", ctypes.c_uint32), ("rays_per_chunk", ctypes.c_uint32), ("blocks_per_sm", ctypes.c_uint32),
                ("block_shape", ctypes.c_uint32), ("sort_key", ctypes.c_uint32), ("staging_depth", ctypes.c_uint32),
                ("refill_below", ctypes.c_uint32)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("budget_bytes", ctypes.c_uint64), ("max_batch_requests", ctypes.c_uint32),
                ("max_batch_rays", ctypes.c_uint32), ("max_inflight", ctypes.c_uint32), ("launch", LaunchConfig)]


class Request(ctypes.Structure):
    _fields_ = [("scene_id", ctypes.c_uint32), ("eye", ctypes.c_float * 3), ("target", ctypes.c_float * 3),
                ("fov_deg", ctypes.c_float), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("hits", Hits)]


class RequestResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("submit_s", ctypes.c_double), ("start_s", ctypes.c_double),
                ("done_s", ctypes.c_double), ("batch_requests", ctypes.c_uint32)]


class ServerStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_uint64) for k in ("requests_done", "rays_done", "launches", "uploads", "evictions",
                                                "resident_bytes")]


class BatchItem(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_void_p), ("rays", Rays), ("n", ctypes.c_uint64), ("hits", Hits),
                ("row_length", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


# name -> (restype, argtypes); every symbol of include/svo.h is listed here
_U32, _U64, _I32, _VP, _F = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_float
_P = ctypes.POINTER
SIGNATURES = {
    "svo_last_error": (ctypes.c_char_p, []),
    "svo_version": (_I32, []),
    "svo_scene_create": (_I32, [_U32, _U32, _P(_VP)]),
    "svo_scene_destroy": (None, [_VP]),
    "svo_set_auto_simplify": (_I32, [_VP, _I32]),
    "svo_insert": (_I32, [_VP, _U32, _U32, _U32, _U32, _U32, _U32]),
    "svo_update": (_I32, [_VP, _U32, _U32, _U32, _U32, _U32, _U32]),
    "svo_insert_at_lod": (_I32, [_VP, _U32, _U32, _U32, _U32, _U32, _U32, _U32]),
    "svo_clear": (_I32, [_VP, _U32, _U32, _U32]),
    "svo_clear_at_lod": (_I32, [_VP, _U32, _U32, _U32, _U32]),
    "svo_apply_ops": (_I32, [_VP, _VP, _U64, _P(_U64)]),
    "svo_insert_dense": (_I32, [_VP, _U32, _U32, _U32, _U32, _U32, _U32, _VP, _VP, _P(_U64)]),
    "svo_get": (_I32, [_VP, _U32, _U32, _U32, _P(_U32), _P(_U32), _P(_U32)]),
    "svo_scene_stats_get": (_I32, [_VP, _P(SceneStats)]),
    "svo_node_record": (_I32, [_VP, _U64, _P(_U64)]),
    "svo_scene_to_bytes": (_I32, [_VP, _VP, _U64, _P(_U64)]),
    "svo_scene_from_bytes": (_I32, [_VP, _U64, _P(_VP)]),
    "svo_scene_save": (_I32, [_VP, ctypes.c_char_p]),
    "svo_scene_load": (_I32, [ctypes.c_char_p, _P(_VP)]),
    "svo_scene_from_vox": (_I32, [_VP, _U64, _U32, _P(_VP)]),
    "svo_scene_load_vox": (_I32, [ctypes.c_char_p, _U32, _P(_VP)]),
    "svo_vox_tree_size": (_I32, [_VP, _U64, _P(_U32)]),
    "svo_vox_insert": (_I32, [_VP, _VP, _U64]),
    "svo_vox_rotation": (_I32, [ctypes.c_uint8, _P(ctypes.c_int8)]),
    "svo_mip_switch": (_I32, [_VP, _I32]),
    "svo_mip_set_method": (_I32, [_VP, _U32, _U32, ctypes.c_float]),
    "svo_mip_set_color_threshold": (_I32, [_VP, _U32, ctypes.c_float]),
    "svo_mip_recalculate": (_I32, [_VP]),
    "svo_mip_sample_root": (_I32, [_VP, _U32, _U32, _U32, _U32, _P(_U32), _P(_U32), _P(_U32)]),
    "svo_palette": (_U64, [_VP, _I32, _VP, _U64]),
    "svo_scene_upload": (_I32, [_VP, _VP]),
    "svo_scene_sync": (_I32, [_VP, _VP]),
    "svo_scene_release_device": (_I32, [_VP]),
    "svo_set_device_allocator": (_I32, [_VP, _VP, _VP]),
    "svo_cast": (_I32, [_VP, _P(Rays), _U64, _P(Hits), _VP]),
    "svo_cast_host": (_I32, [_VP, _P(Rays), _U64, _P(Hits), _VP]),
    "svo_cast_lod": (_I32, [_VP, _P(Rays), _U64, _P(Hits), ctypes.c_float, _VP]),
    "svo_cast_rows": (_I32, [_VP, _P(Rays), _U64, _U32, _P(Hits), _VP]),
    "svo_cast_host_rows": (_I32, [_VP, _P(Rays), _U64, _U32, _P(Hits), _VP]),
    "svo_cast_lod_rows": (_I32, [_VP, _P(Rays), _U64, _U32, _P(Hits), ctypes.c_float, _VP]),
    "svo_render_viewport": (_I32, [_VP, _P(Viewport), _U32, _U32, _VP, _VP, _VP]),
    "svo_render_viewports": (_I32, [_VP, _P(Viewport), _U32, _U32, _U32, _VP, _VP, _VP]),
    "svo_batch_workspace_create": (_I32, [_P(_VP)]),
    "svo_batch_workspace_destroy": (None, [_VP]),
    "svo_cast_batched": (_I32, [_VP, _P(BatchItem), _U32, _P(LaunchConfig), _VP]),
    "svo_cast_batched_noalloc": (_I32, [_P(BatchItem), _U32, _P(LaunchConfig), _VP]),
    "svo_server_create": (_I32, [_P(ServerConfig), _P(_VP)]),
    "svo_server_destroy": (None, [_VP]),
    "svo_server_add_scene": (_I32, [_VP, _VP, _P(_U32)]),
    "svo_server_submit": (_I32, [_VP, _P(Request), _P(_U64)]),
    "svo_server_wait": (_I32, [_VP, _U64, ctypes.c_double, _P(RequestResult)]),
    "svo_server_stats_get": (_I32, [_VP, _P(ServerStats)]),
    "svo_server_now": (ctypes.c_double, [_VP]),
    "svo_gen_scene": (_I32, [_P(SceneRecipe), _VP, _U64, _P(_U64)]),
    "svo_gen_camera_rays": (_I32, [_P(_F), _P(_F), _F, _U32, _U32, _VP, _VP, _VP, _VP, _VP, _VP]),
    "svo_gen_sphere_rays": (_I32, [_P(_F), _F, _U64, _U64, _VP, _VP, _VP, _VP, _VP, _VP]),
    "svo_selftest_luts": (_I32, [_P(_U64), _P(_U32), _P(_U64)]),
    "svo_set_cast_mode": (_I32, [_I32]),
    "svo_set_host_transfer": (_I32, [_I32]),
    "svo_set_staging_depth": (_I32, [_I32]),
    "svo_set_refill": (_I32, [_I32]),
}


def lib_path():
    return _build.LIB


def lib():
    """Loads (building first if needed) libsvo.so and declares its signatures."""
    global _lib
    if _lib is None:
        path = _build.build()
        if not os.path.exists(path):
            raise RuntimeError("libsvo.so missing at %s" % path)
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)  # AttributeError here means the library lacks a declared entry point
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class SvoError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (svo_status %d)" % (msg, code))
        self.code = code


def check(rc):
    if rc != 0:
        raise SvoError(rc, lib().svo_last_error().decode(errors="replace"))
    return rc
