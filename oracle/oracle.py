"""ctypes binding of the CPU oracle library (TEST INFRASTRUCTURE ONLY).

The oracle is a plain CPU restatement of shocovox-rs v0.11.1's octree and
`Octree::get_by_ray` (see svo_oracle.cpp).  The tests compare the GB300
product library against it, and the bench times it as the CPU baseline;
nothing in the product path imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libsvo_oracle.so")
_lib = None

OK, INVALID_SIZE, INVALID_BRICK_DIM, INVALID_STRUCTURE, INVALID_POSITION, REFERENCE_PANIC, ARGUMENT = range(7)

OP_DTYPE = np.dtype([("x", "<u2"), ("y", "<u2"), ("z", "<u2"), ("op", "u1"), ("kind", "u1"),
                     ("size", "<u4"), ("rgba", "<u4"), ("user", "<u4")])
assert OP_DTYPE.itemsize == 20


class Viewport(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_float * 3), ("direction", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("width", ctypes.c_float), ("height", ctypes.c_float), ("fov", ctypes.c_float),
                ("light", ctypes.c_float * 3), ("background", ctypes.c_uint32)]


def viewport_struct(vp):
    """vp: dict with origin, direction, up, width, height, fov, light (3-sequences / floats), background."""
    f3 = ctypes.c_float * 3
    return Viewport(f3(*vp["origin"]), f3(*vp["direction"]), f3(*vp["up"]), vp["width"], vp["height"], vp["fov"],
                    f3(*vp["light"]), vp["background"])


class Recipe(ctypes.Structure):
    """orc_recipe: a seeded synthetic scene (layout of the product's svo_scene_recipe)."""
    _fields_ = [("kind", ctypes.c_uint32), ("size", ctypes.c_uint32), ("brick_dim", ctypes.c_uint32),
                ("seed", ctypes.c_uint64), ("occupancy", ctypes.c_float), ("spheres", ctypes.c_uint32),
                ("octaves", ctypes.c_uint32), ("base_freq", ctypes.c_float), ("height_lo", ctypes.c_float),
                ("height_hi", ctypes.c_float), ("cave_threshold", ctypes.c_float)]


class Hits(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in (
        "status", "brick_octant", "entry_kind", "node_key", "voxel_index", "pix", "albedo", "user",
        "px", "py", "pz", "nx", "ny", "nz", "node_visits", "child_reads", "voxel_reads")]


HIT_FIELDS = {
    "status": np.uint8, "brick_octant": np.uint8, "entry_kind": np.uint8, "node_key": np.uint32,
    "voxel_index": np.uint32, "pix": np.uint32, "albedo": np.uint32, "user": np.uint32,
    "px": np.float32, "py": np.float32, "pz": np.float32, "nx": np.float32, "ny": np.float32,
    "nz": np.float32, "node_visits": np.uint32, "child_reads": np.uint32, "voxel_reads": np.uint32,
}


def build(force=False):
    """Compiles the oracle with its Makefile (g++, no GPU needed)."""
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(os.path.join(_HERE, f))
                                               for f in ("svo_oracle.cpp", "workloads.cpp", "svo_oracle.h",
                                                         "Makefile")):
        subprocess.check_call(["make", "-s", "-C", _HERE])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        u32, u64, vp, i = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_int
        L.orc_new.argtypes = [u32, u32, ctypes.POINTER(vp)]
        L.orc_free.argtypes = [vp]
        L.orc_set_auto_simplify.argtypes = [vp, i]
        L.orc_insert.argtypes = [vp, u32, u32, u32, u32, u32, u32]
        L.orc_update.argtypes = [vp, u32, u32, u32, u32, u32, u32]
        L.orc_insert_at_lod.argtypes = [vp, u32, u32, u32, u32, u32, u32, u32]
        L.orc_clear.argtypes = [vp, u32, u32, u32]
        L.orc_clear_at_lod.argtypes = [vp, u32, u32, u32, u32]
        L.orc_apply_ops.argtypes = [vp, vp, u64, ctypes.POINTER(u64)]
        L.orc_get.argtypes = [vp, u32, u32, u32, ctypes.POINTER(u32)]
        L.orc_cast.argtypes = [vp, u64, vp, vp, vp, vp, vp, vp, ctypes.POINTER(Hits), i]
        L.orc_cast_lod.argtypes = [vp, u64, vp, vp, vp, vp, vp, vp, ctypes.c_float, ctypes.POINTER(Hits), i]
        L.orc_mip_switch.argtypes = [vp, i]
        L.orc_mip_set_method.argtypes = [vp, u32, u32, ctypes.c_float]
        L.orc_mip_set_color_threshold.argtypes = [vp, u32, ctypes.c_float]
        L.orc_mip_recalculate.argtypes = [vp]
        L.orc_mip_sample_root.argtypes = [vp, u32, u32, u32, u32, ctypes.POINTER(u32)]
        L.orc_node_mip.argtypes = [vp, u64, ctypes.POINTER(u32), vp]
        L.orc_render_viewport.argtypes = [vp, ctypes.POINTER(Viewport), u32, u32, vp, ctypes.POINTER(u64), i]
        L.orc_node_count.argtypes = [vp]
        L.orc_node_count.restype = u64
        L.orc_node_record.argtypes = [vp, u64, ctypes.POINTER(u64)]
        L.orc_palette.argtypes = [vp, i, vp, u64]
        L.orc_palette.restype = u64
        L.orc_luts.argtypes = [vp, vp, vp, vp, vp]
        L.orc_intersect_ray.argtypes = [vp, vp, ctypes.POINTER(ctypes.c_float)]
        L.orc_cube_impact_normal.argtypes = [vp, vp, vp]
        L.orc_hash_region.argtypes = [vp, ctypes.c_float]
        L.orc_hash_region.restype = u32
        L.orc_position_in_bitmap.argtypes = [u64, u64, u64, u64]
        L.orc_position_in_bitmap.restype = u64
        L.orc_set_occupancy.argtypes = [u64, u64, u64, u64, u64, i, u64]
        L.orc_set_occupancy.restype = u64
        L.orc_plane_line_intersection.argtypes = [vp, vp, vp, vp, ctypes.POINTER(ctypes.c_float)]
        L.orc_child_bounds.argtypes = [vp, u32, vp]
        L.orc_dda_step.argtypes = [vp, vp, vp, vp]
        L.orc_flat_projection.argtypes = [u64, u64, u64, u64]
        L.orc_flat_projection.restype = u64
        L.orc_brick_empty_throughout.argtypes = [vp, u32, u32, u32, ctypes.c_int32, vp, u32, vp, u32]
        L.orc_stack_new.argtypes = [u32]
        L.orc_stack_new.restype = vp
        L.orc_stack_free.argtypes = [vp]
        L.orc_stack_push.argtypes = [vp, ctypes.c_int32]
        L.orc_stack_pop.argtypes = [vp, ctypes.POINTER(ctypes.c_int32)]
        L.orc_stack_last.argtypes = [vp, ctypes.POINTER(ctypes.c_int32)]
        L.orc_stack_add_last.argtypes = [vp, ctypes.c_int32]
        L.orc_stack_is_empty.argtypes = [vp]
        fp = ctypes.POINTER(ctypes.c_float)
        L.orc_gen_scene.argtypes = [ctypes.POINTER(Recipe), vp, u64, ctypes.POINTER(u64)]
        L.orc_gen_camera_rays.argtypes = [fp, fp, ctypes.c_float, u32, u32, vp, vp, vp, vp, vp, vp]
        L.orc_gen_camera_rays_strided.argtypes = [fp, fp, ctypes.c_float, u32, u32, u64, u64, u64, vp, vp, vp, vp, vp,
                                                  vp]
        L.orc_gen_sphere_rays.argtypes = [fp, ctypes.c_float, u64, u64, vp, vp, vp, vp, vp, vp]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def f32arr(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float32))


class OracleError(RuntimeError):
    def __init__(self, code, what):
        super().__init__("%s failed with oracle status %d" % (what, code))
        self.code = code


class Tree:
    """Oracle octree: construction, update, get and the CPU cast."""

    def __init__(self, size, brick_dim):
        h = ctypes.c_void_p()
        rc = lib().orc_new(size, brick_dim, ctypes.byref(h))
        if rc != OK:
            raise OracleError(rc, "Octree::new(%d, %d)" % (size, brick_dim))
        self._h = h
        self.size, self.brick_dim = size, brick_dim

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_free(self._h)
            self._h = None

    def set_auto_simplify(self, on):
        lib().orc_set_auto_simplify(self._h, 1 if on else 0)

    @staticmethod
    def _entry(albedo=None, user=None):
        kind = (1 if albedo is not None else 0) | (2 if user is not None else 0)
        return kind, (albedo or 0) & 0xFFFFFFFF, (user or 0) & 0xFFFFFFFF

    def insert(self, pos, albedo=None, user=None):
        k, a, u = self._entry(albedo, user)
        return lib().orc_insert(self._h, pos[0], pos[1], pos[2], k, a, u)

    def update(self, pos, albedo=None, user=None):
        k, a, u = self._entry(albedo, user)
        return lib().orc_update(self._h, pos[0], pos[1], pos[2], k, a, u)

    def insert_at_lod(self, pos, size, albedo=None, user=None):
        k, a, u = self._entry(albedo, user)
        return lib().orc_insert_at_lod(self._h, pos[0], pos[1], pos[2], size, k, a, u)

    def clear(self, pos):
        return lib().orc_clear(self._h, pos[0], pos[1], pos[2])

    def clear_at_lod(self, pos, size):
        return lib().orc_clear_at_lod(self._h, pos[0], pos[1], pos[2], size)

    def apply_ops(self, ops):
        ops = np.ascontiguousarray(ops, dtype=OP_DTYPE)
        done = ctypes.c_uint64()
        rc = lib().orc_apply_ops(self._h, _ptr(ops), len(ops), ctypes.byref(done))
        if rc != OK:
            raise OracleError(rc, "apply_ops at op %d" % done.value)

    def get(self, pos):
        out = (ctypes.c_uint32 * 3)()
        rc = lib().orc_get(self._h, pos[0], pos[1], pos[2], out)
        if rc != OK:
            raise OracleError(rc, "get")
        return tuple(out)  # (kind, rgba, user)

    def cast(self, origins, directions, threads=1, viewing_distance=None):
        """origins/directions: (n,3) float32.  Returns a dict of per-ray numpy arrays.  With a viewing
        distance the cast is get_by_ray_at_lod."""
        o = f32arr(origins).reshape(-1, 3)
        d = f32arr(directions).reshape(-1, 3)
        n = o.shape[0]
        cols = [np.ascontiguousarray(o[:, k]) for k in range(3)] + [np.ascontiguousarray(d[:, k]) for k in range(3)]
        out = {k: np.zeros(n, dtype=t) for k, t in HIT_FIELDS.items()}
        h = Hits(**{k: out[k].ctypes.data for k in HIT_FIELDS})
        if viewing_distance is None:
            rc = lib().orc_cast(self._h, n, *[_ptr(c) for c in cols], ctypes.byref(h), threads)
        else:
            rc = lib().orc_cast_lod(self._h, n, *[_ptr(c) for c in cols], viewing_distance, ctypes.byref(h), threads)
        if rc != OK:
            raise OracleError(rc, "cast")
        return out

    def render_viewport(self, vp, width, height, threads=1):
        """One frame of examples/cpu_render.rs.  Returns (rgba (height, width, 4) uint8, unshaded pixel count)."""
        img = np.zeros((height, width, 4), dtype=np.uint8)
        bad = ctypes.c_uint64(0)
        rc = lib().orc_render_viewport(self._h, ctypes.byref(viewport_struct(vp)), width, height, img.ctypes.data,
                                       ctypes.byref(bad), threads)
        if rc != OK:
            raise OracleError(rc, "render_viewport")
        return img, bad.value

    # ---- MIP maps (octree/mipmap.rs) ----
    BOX, POINT, POINT_BD, POSTERIZE, POSTERIZE_BD = range(5)

    def mip_switch(self, enabled):
        self._check(lib().orc_mip_switch(self._h, int(bool(enabled))), "mip_switch")

    def mip_set_method(self, level, method, thr=0.0):
        self._check(lib().orc_mip_set_method(self._h, level, method, thr), "mip_set_method")

    def mip_set_color_threshold(self, level, thr):
        self._check(lib().orc_mip_set_color_threshold(self._h, level, thr), "mip_set_color_threshold")

    def mip_recalculate(self):
        self._check(lib().orc_mip_recalculate(self._h), "mip_recalculate")

    def mip_sample_root(self, octant, pos):
        out = (ctypes.c_uint32 * 3)()
        self._check(lib().orc_mip_sample_root(self._h, octant, pos[0], pos[1], pos[2], out), "mip_sample_root")
        return tuple(out)  # (kind, rgba, user)

    def node_mip(self, key, brick_dim):
        """(kind, values): kind 0 empty, 1 solid, 2 parted, 3 past node_mips."""
        kind = ctypes.c_uint32(0)
        vals = np.zeros(max(1, brick_dim ** 3), dtype=np.uint32)
        self._check(lib().orc_node_mip(self._h, key, ctypes.byref(kind), vals.ctypes.data), "node_mip")
        return kind.value, vals

    def _check(self, rc, what):
        if rc != OK:
            raise OracleError(rc, what)

    def cast_one(self, origin, direction):
        r = self.cast([origin], [direction])
        return {k: v[0] for k, v in r.items()}

    def node_count(self):
        return lib().orc_node_count(self._h)

    def node_record(self, key):
        rec = (ctypes.c_uint64 * 40)()
        lib().orc_node_record(self._h, key, rec)
        return tuple(rec)

    def records(self):
        return [self.node_record(k) for k in range(self.node_count())]

    def palette(self, which):
        n = lib().orc_palette(self._h, which, None, 0)
        out = np.zeros(n, dtype=np.uint32)
        lib().orc_palette(self._h, which, _ptr(out), n)
        return out


def luts():
    rtn = np.zeros(512, dtype=np.uint64)
    step = np.zeros(27, dtype=np.uint32)
    mask = np.zeros(8, dtype=np.uint64)
    idx = np.zeros(64, dtype=np.uint8)
    off = np.zeros(24, dtype=np.float32)
    lib().orc_luts(_ptr(rtn), _ptr(step), _ptr(mask), _ptr(idx), _ptr(off))
    return {"RAY_TO_NODE_OCCUPANCY_BITMASK_LUT": rtn, "OCTANT_STEP_RESULT_LUT": step,
            "BITMAP_MASK_FOR_OCTANT_LUT": mask, "BITMAP_INDEX_LUT": idx,
            "OCTANT_OFFSET_REGION_LUT": off.reshape(8, 3)}


def intersect_ray(cube, ray):
    d = ctypes.c_float()
    k = lib().orc_intersect_ray(_ptr(f32arr(cube)), _ptr(f32arr(ray)), ctypes.byref(d))
    if k == 0:
        return None
    return ("inside", None) if k == 1 else ("hit", d.value)


def cube_impact_normal(cube, point):
    out = np.zeros(3, dtype=np.float32)
    lib().orc_cube_impact_normal(_ptr(f32arr(cube)), _ptr(f32arr(point)), _ptr(out))
    return out


def hash_region(offset, size_half):
    return lib().orc_hash_region(_ptr(f32arr(offset)), size_half)


def position_in_bitmap(x, y, z, bs):
    return lib().orc_position_in_bitmap(x, y, z, bs)


def set_occupancy(pos, size, brick_dim, occupied, bitmap):
    return lib().orc_set_occupancy(pos[0], pos[1], pos[2], size, brick_dim, 1 if occupied else 0, bitmap)


def plane_line_intersection(pp, pn, lo, ld):
    out = ctypes.c_float()
    ok = lib().orc_plane_line_intersection(_ptr(f32arr(pp)), _ptr(f32arr(pn)), _ptr(f32arr(lo)), _ptr(f32arr(ld)),
                                           ctypes.byref(out))
    return out.value if ok else None


def child_bounds(cube, octant):
    out = np.zeros(4, dtype=np.float32)
    lib().orc_child_bounds(_ptr(f32arr(cube)), octant, _ptr(out))
    return out


def flat_projection(x, y, z, size):
    return lib().orc_flat_projection(x, y, z, size)


def brick_empty_throughout(kind, pix, dim, octant, colors, datas, part=-1):
    """BrickData::is_empty_throughout (part < 0) or is_part_empty_throughout(octant, part) of a brick of
    kind 0 Empty, 1 Solid (pix[0]) or 2 Parted (dim^3 values) against the given palettes."""
    p = np.ascontiguousarray(np.asarray(pix if len(pix) else [0], dtype=np.uint32))
    c = np.ascontiguousarray(np.asarray(colors if len(colors) else [0], dtype=np.uint32))
    d = np.ascontiguousarray(np.asarray(datas if len(datas) else [0], dtype=np.uint32))
    rc = lib().orc_brick_empty_throughout(_ptr(p), dim, kind, octant, part, _ptr(c), len(colors), _ptr(d), len(datas))
    if rc not in (0, 1):
        raise OracleError(rc, "brick_empty_throughout")
    return rc == 1


class Stack:
    """NodeStack<i32, size> harness."""

    def __init__(self, size):
        self._h = lib().orc_stack_new(size)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_stack_free(self._h)

    def push(self, v):
        lib().orc_stack_push(self._h, v)

    def pop(self):
        o = ctypes.c_int32()
        return o.value if lib().orc_stack_pop(self._h, ctypes.byref(o)) else None

    def last(self):
        o = ctypes.c_int32()
        return o.value if lib().orc_stack_last(self._h, ctypes.byref(o)) else None

    def add_last(self, d):
        return bool(lib().orc_stack_add_last(self._h, d))

    def is_empty(self):
        return bool(lib().orc_stack_is_empty(self._h))


# ---- the benchmark's seeded workloads (workloads.cpp), with the product generators' signatures ----
def gen_scene(kind, size, brick_dim, seed, occupancy=0.1, spheres=0, octaves=2, base_freq=1.0 / 32,
              height_lo=0.0, height_hi=96.0, cave_threshold=0.55):
    """Construction ops (OP_DTYPE) of a seeded synthetic scene."""
    r = Recipe(kind, size, brick_dim, seed, occupancy, spheres, octaves, base_freq, height_lo, height_hi,
               cave_threshold)
    n = ctypes.c_uint64()
    if lib().orc_gen_scene(ctypes.byref(r), None, 0, ctypes.byref(n)) != OK:
        raise OracleError(ARGUMENT, "gen_scene")
    ops = np.zeros(n.value, dtype=OP_DTYPE)
    if lib().orc_gen_scene(ctypes.byref(r), _ptr(ops), n.value, ctypes.byref(n)) != OK:
        raise OracleError(ARGUMENT, "gen_scene")
    return ops


def gen_camera_rays(eye, target, fov_deg, width, height):
    """Pinhole camera rays in raster order: (origins (n,3), directions (n,3)) float32."""
    cols = [np.zeros(width * height, dtype=np.float32) for _ in range(6)]
    e, t = (ctypes.c_float * 3)(*eye), (ctypes.c_float * 3)(*target)
    if lib().orc_gen_camera_rays(e, t, fov_deg, width, height, *[_ptr(c) for c in cols]) != OK:
        raise OracleError(ARGUMENT, "gen_camera_rays")
    return np.stack(cols[:3], axis=1), np.stack(cols[3:], axis=1)


def gen_camera_rays_strided(eye, target, fov_deg, width, height, first, stride):
    """The rays of pixels first, first + stride, ... of a camera image (raster order)."""
    n = max(0, (width * height - first + stride - 1) // stride)
    cols = [np.zeros(n, dtype=np.float32) for _ in range(6)]
    e, t = (ctypes.c_float * 3)(*eye), (ctypes.c_float * 3)(*target)
    if lib().orc_gen_camera_rays_strided(e, t, fov_deg, width, height, first, stride, n, *[_ptr(c) for c in cols]) != OK:
        raise OracleError(ARGUMENT, "gen_camera_rays_strided")
    return np.stack(cols[:3], axis=1), np.stack(cols[3:], axis=1)


def gen_sphere_rays(center, radius, n, seed):
    """Origins uniform on a sphere, directions uniform on S^2: (origins (n,3), directions (n,3)) float32."""
    cols = [np.zeros(n, dtype=np.float32) for _ in range(6)]
    c = (ctypes.c_float * 3)(*center)
    if lib().orc_gen_sphere_rays(c, radius, n, seed, *[_ptr(a) for a in cols]) != OK:
        raise OracleError(ARGUMENT, "gen_sphere_rays")
    return np.stack(cols[:3], axis=1), np.stack(cols[3:], axis=1)
