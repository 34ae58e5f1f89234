"""shocovox_gb300 -- GB300-native sparse voxel octree ray caster.

Python mirror of the reference crate's API for the ray-cast path
(shocovox-rs v0.11.1): ``Octree(size, brick_dim)`` with ``insert``,
``insert_at_lod``, ``update``, ``clear``, ``clear_at_lod`` and ``get``
(src/octree/**), and ``get_by_ray`` (src/raytracing/raytracing_on_cpu.rs:316)
plus batched casts.  All work runs in libsvo (C++ host code and sm_103a CUDA
kernels behind the C ABI in include/svo.h); this module only marshals
arguments.  There is no CPU fallback: without libsvo nothing here works.
"""
import ctypes
import os

import numpy as np

from ._lib import (HIT_FIELDS, OP_DTYPE, Hits, LaunchConfig, Rays, Request, RequestResult, SceneRecipe, ServerConfig,
                   ServerStats, Viewport, check, lib)

__all__ = ["Octree", "OctreeError", "OP_DTYPE", "HIT_FIELDS", "gen_scene", "gen_camera_rays", "gen_sphere_rays",
           "SceneRecipe", "LaunchConfig", "BatchWorkspace", "Server", "viewport", "orbit_viewport", "lib"]

OK, INVALID_SIZE, INVALID_BRICK_DIM, INVALID_STRUCTURE, INVALID_POSITION = 0, 1, 2, 3, 4


class OctreeError(RuntimeError):
    """An svo_status other than SVO_OK; `.code` carries it (1..4 mirror OctreeError)."""

    def __init__(self, code, msg):
        super().__init__("%s (svo_status %d)" % (msg, code))
        self.code = code


def _vp(x):
    return ctypes.c_void_p(x) if isinstance(x, int) else x


def _np_ptr(a):
    return a.ctypes.data if a is not None else 0


def _entry(albedo, user):
    kind = (1 if albedo is not None else 0) | (2 if user is not None else 0)
    return kind, (albedo or 0) & 0xFFFFFFFF, (user or 0) & 0xFFFFFFFF


class Octree:
    """A scene: host octree plus (after ``upload``) its device-resident image."""

    def __init__(self, size, brick_dim):
        h = ctypes.c_void_p()
        rc = lib().svo_scene_create(size, brick_dim, ctypes.byref(h))
        if rc != 0:
            raise OctreeError(rc, lib().svo_last_error().decode())
        self._h = h
        self.size, self.brick_dim = size, brick_dim

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().svo_scene_destroy(h)
            self._h = None

    @classmethod
    def _adopt(cls, h):
        t = cls.__new__(cls)
        t._h = h
        st = t.stats()
        t.size, t.brick_dim = st["size"], st["brick_dim"]
        return t

    # ---- persistence: Octree::to_bytes / from_bytes / save / load (src/octree/mod.rs:138-168) ----
    def to_bytes(self):
        n = ctypes.c_uint64()
        check(lib().svo_scene_to_bytes(self._h, None, 0, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(max(n.value, 1))
        check(lib().svo_scene_to_bytes(self._h, buf, n.value, ctypes.byref(n)))
        return buf.raw[:n.value]

    @classmethod
    def from_bytes(cls, data):
        h = ctypes.c_void_p()
        check(lib().svo_scene_from_bytes(data, len(data), ctypes.byref(h)))
        return cls._adopt(h)

    def save(self, path):
        check(lib().svo_scene_save(self._h, os.fsencode(path)))

    @classmethod
    def load(cls, path):
        h = ctypes.c_void_p()
        check(lib().svo_scene_load(os.fsencode(path), ctypes.byref(h)))
        return cls._adopt(h)

    # ---- MagicaVoxel import: Octree::load_vox_file / MIPMapStrategy::load_vox_file
    #      (src/convert/magicavoxel.rs:204-385) ----
    @classmethod
    def from_vox(cls, data, brick_dim, configure=None):
        """The octree of a .vox file's frame 0. With `configure` (a callable taking the new, still
        empty octree, e.g. to set its MIP strategy) the size is taken from the file, `configure`
        runs, then the voxels are inserted: MIPMapStrategy::load_vox_file."""
        data = bytes(data)
        if configure is None:
            h = ctypes.c_void_p()
            check(lib().svo_scene_from_vox(data, len(data), brick_dim, ctypes.byref(h)))
            return cls._adopt(h)
        t = cls(cls.vox_tree_size(data), brick_dim)
        configure(t)
        check(lib().svo_vox_insert(t._h, data, len(data)))
        return t

    @classmethod
    def load_vox(cls, path, brick_dim, configure=None):
        if configure is None:
            h = ctypes.c_void_p()
            check(lib().svo_scene_load_vox(os.fsencode(path), brick_dim, ctypes.byref(h)))
            return cls._adopt(h)
        with open(path, "rb") as f:
            return cls.from_vox(f.read(), brick_dim, configure)

    @staticmethod
    def vox_tree_size(data):
        n = ctypes.c_uint32()
        check(lib().svo_vox_tree_size(bytes(data), len(data), ctypes.byref(n)))
        return n.value

    @staticmethod
    def vox_rotation(byte):
        """parse_rotation_matrix: the row-major 3x3 matrix of a .vox rotation byte."""
        m = (ctypes.c_int8 * 9)()
        check(lib().svo_vox_rotation(byte, m))
        return [list(m[0:3]), list(m[3:6]), list(m[6:9])]

    @property
    def handle(self):
        return self._h

    # ---- construction / update: return 0 (Ok) or an OctreeError code 1..4 ----
    def _op(self, rc):
        if rc in (0, 1, 2, 3, 4):
            return rc
        raise OctreeError(rc, lib().svo_last_error().decode())

    def set_auto_simplify(self, on):
        check(lib().svo_set_auto_simplify(self._h, 1 if on else 0))

    def insert(self, pos, albedo=None, user=None):
        k, a, u = _entry(albedo, user)
        return self._op(lib().svo_insert(self._h, pos[0], pos[1], pos[2], k, a, u))

    def update(self, pos, albedo=None, user=None):
        k, a, u = _entry(albedo, user)
        return self._op(lib().svo_update(self._h, pos[0], pos[1], pos[2], k, a, u))

    def insert_at_lod(self, pos, size, albedo=None, user=None):
        k, a, u = _entry(albedo, user)
        return self._op(lib().svo_insert_at_lod(self._h, pos[0], pos[1], pos[2], size, k, a, u))

    def clear(self, pos):
        return self._op(lib().svo_clear(self._h, pos[0], pos[1], pos[2]))

    def clear_at_lod(self, pos, size):
        return self._op(lib().svo_clear_at_lod(self._h, pos[0], pos[1], pos[2], size))

    def insert_dense(self, origin, rgba=None, user=None):
        """Bulk insert of a dense block: `rgba` and/or `user` are uint32 arrays of shape (d, h, w)
        (index [k, j, i] for voxel origin + (i, j, k)), inserted like the reference's fill loops."""
        a = np.ascontiguousarray(rgba, dtype=np.uint32) if rgba is not None else None
        u = np.ascontiguousarray(user, dtype=np.uint32) if user is not None else None
        shape = (a if a is not None else u).shape
        d, h, w = shape
        done = ctypes.c_uint64()
        rc = lib().svo_insert_dense(self._h, origin[0], origin[1], origin[2], w, h, d,
                                    _vp(a.ctypes.data) if a is not None else None,
                                    _vp(u.ctypes.data) if u is not None else None, ctypes.byref(done))
        if rc not in (0,):
            raise OctreeError(rc, "%s (after %d inserts)" % (lib().svo_last_error().decode(), done.value))
        return done.value

    def apply_ops(self, ops):
        ops = np.ascontiguousarray(ops, dtype=OP_DTYPE)
        done = ctypes.c_uint64()
        rc = lib().svo_apply_ops(self._h, _vp(_np_ptr(ops)), len(ops), ctypes.byref(done))
        if rc != 0:
            raise OctreeError(rc, "apply_ops stopped at op %d: %s" % (done.value, lib().svo_last_error().decode()))

    def get(self, pos):
        k, a, u = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        check(lib().svo_get(self._h, pos[0], pos[1], pos[2], ctypes.byref(k), ctypes.byref(a), ctypes.byref(u)))
        return (k.value, a.value, u.value)

    def stats(self):
        from ._lib import SceneStats
        s = SceneStats()
        check(lib().svo_scene_stats_get(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in SceneStats._fields_}

    def node_record(self, key):
        rec = (ctypes.c_uint64 * 40)()
        check(lib().svo_node_record(self._h, key, rec))
        return tuple(rec)

    def records(self):
        return [self.node_record(k) for k in range(self.stats()["nodes"])]

    def palette(self, which):
        n = lib().svo_palette(self._h, which, None, 0)
        out = np.zeros(n, dtype=np.uint32)
        lib().svo_palette(self._h, which, _vp(_np_ptr(out)), n)
        return out

    # ---- device image ----
    def upload(self, stream=0):
        check(lib().svo_scene_upload(self._h, _vp(stream)))

    def sync(self, stream=0):
        check(lib().svo_scene_sync(self._h, _vp(stream)))

    def release_device(self):
        check(lib().svo_scene_release_device(self._h))

    # ---- the cast ----
    def cast(self, rays, hits, n, stream=0, row_length=0):
        """Device cast: ``rays`` / ``hits`` map field names to device pointers (ints). ``row_length``:
        the rays are rows of that many rays (a camera image in raster order), see svo_cast_rows."""
        r = Rays(*[_vp(rays[k]) for k in ("ox", "oy", "oz", "dx", "dy", "dz")])
        h = Hits(**{k: _vp(hits.get(k, 0) or 0) for k in HIT_FIELDS})
        check(lib().svo_cast_rows(self._h, ctypes.byref(r), n, row_length, ctypes.byref(h), _vp(stream)))

    def cast_lod(self, rays, hits, n, viewing_distance, stream=0, row_length=0):
        """get_by_ray_at_lod on device buffers (dicts of device pointers, like cast())."""
        r = Rays(*[_vp(rays[k]) for k in ("ox", "oy", "oz", "dx", "dy", "dz")])
        h = Hits(**{k: _vp(hits.get(k, 0) or 0) for k in HIT_FIELDS})
        check(lib().svo_cast_lod_rows(self._h, ctypes.byref(r), n, row_length, ctypes.byref(h), viewing_distance,
                                      _vp(stream)))

    def cast_host(self, origins, directions, fields=tuple(HIT_FIELDS), stream=0, row_length=0):
        """Host-buffer cast (copies in, casts, copies out, synchronises)."""
        o = np.ascontiguousarray(np.asarray(origins, dtype=np.float32).reshape(-1, 3))
        d = np.ascontiguousarray(np.asarray(directions, dtype=np.float32).reshape(-1, 3))
        n = o.shape[0]
        cols = [np.ascontiguousarray(o[:, k]) for k in range(3)] + [np.ascontiguousarray(d[:, k]) for k in range(3)]
        out = {k: np.zeros(n, dtype=HIT_FIELDS[k]) for k in fields}
        r = Rays(*[_vp(c.ctypes.data) for c in cols])
        h = Hits(**{k: _vp(out[k].ctypes.data) if k in out else None for k in HIT_FIELDS})
        check(lib().svo_cast_host_rows(self._h, ctypes.byref(r), n, row_length, ctypes.byref(h), _vp(stream)))
        return out

    def cast_host_soa(self, cols, out, stream=0, row_length=0):
        """Host cast over caller-owned arrays: cols = 6 float32 arrays, out = {field: array}."""
        n = len(cols[0])
        r = Rays(*[_vp(c.ctypes.data) for c in cols])
        h = Hits(**{k: _vp(out[k].ctypes.data) if k in out else None for k in HIT_FIELDS})
        check(lib().svo_cast_host_rows(self._h, ctypes.byref(r), n, row_length, ctypes.byref(h), _vp(stream)))

    # ---- MIP maps: Octree::albedo_mip_map_resampling_strategy() (src/octree/mipmap.rs) ----
    BOX_FILTER, POINT_FILTER, POINT_FILTER_BD, POSTERIZE, POSTERIZE_BD = range(5)

    def switch_albedo_mip_maps(self, enabled):
        check(lib().svo_mip_switch(self._h, int(bool(enabled))))
        return self

    def set_mip_method(self, level, method, threshold=0.0):
        check(lib().svo_mip_set_method(self._h, level, method, threshold))
        return self

    def set_mip_color_threshold(self, level, threshold):
        check(lib().svo_mip_set_color_threshold(self._h, level, threshold))
        return self

    def recalculate_mips(self):
        check(lib().svo_mip_recalculate(self._h))
        return self

    def sample_root_mip(self, octant, pos):
        """(kind, rgba, user) of the root's MIP (octant 8) or a root child's at `pos`."""
        k, a, u = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        check(lib().svo_mip_sample_root(self._h, octant, pos[0], pos[1], pos[2], ctypes.byref(k), ctypes.byref(a),
                                        ctypes.byref(u)))
        return k.value, a.value, u.value

    def render_viewport(self, viewport, width, height, rgba, unshaded=0, stream=0):
        """Fused render of examples/cpu_render.rs's frame into device memory: `viewport` from
        viewport(), `rgba` a device pointer to height * width * 4 bytes (row-major from the top
        row), `unshaded` an optional device pointer to a u64 counter."""
        check(lib().svo_render_viewport(self._h, ctypes.byref(viewport), width, height, _vp(rgba), _vp(unshaded),
                                        _vp(stream)))

    def render_viewports(self, viewports, width, height, rgba, unshaded=0, stream=0):
        """Several viewports in one launch: frame k at rgba + k * height * width * 4."""
        from ._lib import Viewport
        arr = (Viewport * len(viewports))(*viewports)
        check(lib().svo_render_viewports(self._h, arr, len(viewports), width, height, _vp(rgba), _vp(unshaded),
                                         _vp(stream)))

    def get_by_ray(self, origin, direction):
        """Octree::get_by_ray for one ray: None or ((kind, rgba, user), point, normal)."""
        r = self.cast_host([origin], [direction])
        if r["status"][0] != 1:
            return None
        return ((int(r["entry_kind"][0]), int(r["albedo"][0]), int(r["user"][0])),
                (r["px"][0], r["py"][0], r["pz"][0]), (r["nx"][0], r["ny"][0], r["nz"][0]))


def _normalized(v):
    """V3c::normalized (vector.rs:75-81) in f32."""
    v = np.asarray(v, dtype=np.float32)
    n = np.sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2], dtype=np.float32)
    return v / n


def viewport(origin, direction, up=(0.0, 1.0, 0.0), width=4.0, height=4.0, fov=3.0, light=None,
             background=0x808080FF):
    """The viewport of examples/cpu_render.rs (its constants are the defaults; light defaults to
    normalize(0, -1, 1)).  `direction` is used as given: the example passes a unit vector."""
    f3 = ctypes.c_float * 3
    if light is None:
        light = _normalized([0.0, -1.0, 1.0])
    return Viewport(f3(*map(float, origin)), f3(*map(float, direction)), f3(*map(float, up)), width, height, fov,
                    f3(*map(float, light)), background)


def orbit_viewport(angle, radius, **kw):
    """The example's camera: origin (sin(angle) r, r, cos(angle) r) looking at the world origin."""
    a = np.float32(angle)
    r = np.float32(radius)
    origin = np.array([np.sin(a) * r, r, np.cos(a) * r], dtype=np.float32)
    return viewport(origin, _normalized(np.zeros(3, np.float32) - origin), **kw)


class BatchWorkspace:
    """Owner of the batched cast's device-side item table and work counter."""

    def __init__(self):
        h = ctypes.c_void_p()
        check(lib().svo_batch_workspace_create(ctypes.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().svo_batch_workspace_destroy(h)
            self._h = None

    def cast(self, items, cfg=None, stream=0):
        """items: list of (Octree, rays dict, n, hits dict[, row_length]) with device pointers."""
        from ._lib import BatchItem
        arr = (BatchItem * len(items))()
        for i, item in enumerate(items):
            scene, rays, n, hits = item[:4]
            arr[i].scene = scene.handle
            arr[i].rays = Rays(*[_vp(rays[k]) for k in ("ox", "oy", "oz", "dx", "dy", "dz")])
            arr[i].n = n
            arr[i].hits = Hits(**{k: _vp(hits.get(k, 0) or 0) for k in HIT_FIELDS})
            arr[i].row_length = item[4] if len(item) > 4 else 0
        c = cfg if cfg is not None else LaunchConfig()
        check(lib().svo_cast_batched(self._h, arr, len(items), ctypes.byref(c), _vp(stream)))


class Server:
    """Continuous-batching request server over resident scenes (svo_server_*)."""

    def __init__(self, budget_bytes=60 << 30, max_batch_requests=64, max_batch_rays=1 << 25, max_inflight=2,
                 launch=None):
        cfg = ServerConfig(budget_bytes, max_batch_requests, max_batch_rays, max_inflight,
                           launch if launch is not None else LaunchConfig())
        h = ctypes.c_void_p()
        check(lib().svo_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._scenes = []
        self._keep = {}

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            lib().svo_server_destroy(h)
            self._h = None
            self._keep.clear()

    def __del__(self):
        self.close()

    def add_scene(self, scene):
        sid = ctypes.c_uint32()
        check(lib().svo_server_add_scene(self._h, scene.handle, ctypes.byref(sid)))
        self._scenes.append(scene)  # keep it alive while registered
        return sid.value

    def submit(self, scene_id, eye, target, fov_deg, width, height, out):
        """out: {field: host array of width*height}; the arrays must stay alive until wait()."""
        r = Request(scene_id, (ctypes.c_float * 3)(*eye), (ctypes.c_float * 3)(*target), fov_deg, width, height,
                    Hits(**{k: _vp(out[k].ctypes.data) if k in out else None for k in HIT_FIELDS}))
        rid = ctypes.c_uint64()
        check(lib().svo_server_submit(self._h, ctypes.byref(r), ctypes.byref(rid)))
        self._keep[rid.value] = out
        return rid.value

    def wait(self, request_id, timeout_s=60.0):
        res = RequestResult()
        rc = lib().svo_server_wait(self._h, request_id, timeout_s, ctypes.byref(res))
        if rc == 12:  # SVO_ERR_BUSY: still running
            return None
        self._keep.pop(request_id, None)
        if rc != 0:
            raise OctreeError(rc, lib().svo_last_error().decode())
        return {"submit_s": res.submit_s, "start_s": res.start_s, "done_s": res.done_s,
                "batch_requests": res.batch_requests}

    def stats(self):
        st = ServerStats()
        check(lib().svo_server_stats_get(self._h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def now(self):
        return lib().svo_server_now(self._h)


def gen_scene(kind, size, brick_dim, seed, occupancy=0.1, spheres=0, octaves=2, base_freq=1.0 / 32,
              height_lo=0.0, height_hi=96.0, cave_threshold=0.55):
    """Seeded construction recipe (array of OP_DTYPE ops) of a synthetic scene."""
    r = SceneRecipe(kind, size, brick_dim, seed, occupancy, spheres, octaves, base_freq, height_lo, height_hi,
                    cave_threshold)
    n = ctypes.c_uint64()
    check(lib().svo_gen_scene(ctypes.byref(r), None, 0, ctypes.byref(n)))
    ops = np.zeros(n.value, dtype=OP_DTYPE)
    check(lib().svo_gen_scene(ctypes.byref(r), _vp(_np_ptr(ops)), n.value, ctypes.byref(n)))
    return ops


def _ray_arrays(n):
    return [np.zeros(n, dtype=np.float32) for _ in range(6)]


def gen_camera_rays(eye, target, fov_deg, width, height):
    """Pinhole camera rays; returns (origins (n,3), directions (n,3)) float32."""
    cols = _ray_arrays(width * height)
    e = (ctypes.c_float * 3)(*eye)
    t = (ctypes.c_float * 3)(*target)
    check(lib().svo_gen_camera_rays(e, t, ctypes.c_float(fov_deg), width, height, *[_vp(c.ctypes.data) for c in cols]))
    return np.stack(cols[:3], axis=1), np.stack(cols[3:], axis=1)


def gen_sphere_rays(center, radius, n, seed):
    """Origins uniform on a sphere, directions uniform on S^2."""
    cols = _ray_arrays(n)
    c = (ctypes.c_float * 3)(*center)
    check(lib().svo_gen_sphere_rays(c, ctypes.c_float(radius), n, seed, *[_vp(a.ctypes.data) for a in cols]))
    return np.stack(cols[:3], axis=1), np.stack(cols[3:], axis=1)
