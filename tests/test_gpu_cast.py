"""GPU parity: libsvo's sm_103a cast against the oracle's CPU restatement of get_by_ray.

Hit identity (status, node key, brick octant, voxel index, PaletteIndexValues,
entry kind, albedo, user data) must match exactly; impact point and normal
within 1e-4 voxel units (TOL below).  Counters of the instrumented cast
(node visits, child reads, voxel reads) must match exactly too.
"""
import json
import os
import zlib

import numpy as np
import pytest

import shocovox_gb300 as svo
from helpers import (ALBEDO, GOLDEN, INSERT, normalized, ops_from, ray_of, scene_brick_boundary, scene_dot_cube,
                     scene_floor, scene_stairs)

pytestmark = pytest.mark.gpu

TOL = 1e-4  # voxel units, impact point and normal
INT_FIELDS = ["status", "brick_octant", "entry_kind", "node_key", "voxel_index", "pix", "albedo", "user"]
FLOAT_FIELDS = ["px", "py", "pz", "nx", "ny", "nz"]
COUNTERS = ["node_visits", "child_reads", "voxel_reads"]


def assert_same_hits(gpu, cpu, counters=False, label=""):
    n = len(cpu["status"])
    for f in INT_FIELDS + (COUNTERS if counters else []):
        bad = np.nonzero(gpu[f] != cpu[f])[0]
        assert len(bad) == 0, "%s: %s differs on %d/%d rays, first %d: gpu %s cpu %s" % (
            label, f, len(bad), n, bad[0], gpu[f][bad[0]], cpu[f][bad[0]])
    for f in FLOAT_FIELDS:
        g, c = gpu[f].astype(np.float64), cpu[f].astype(np.float64)
        # identical values (also infinities) and NaN on both sides (e.g. a NaN-direction ray that the
        # reference reports as a hit) agree; everything else must be within TOL
        same = (g == c) | (np.isnan(g) & np.isnan(c))
        with np.errstate(invalid="ignore"):
            d = np.where(same, 0.0, np.abs(g - c))
        bad = np.nonzero(~(d <= TOL))[0]
        assert len(bad) == 0, "%s: %s differs on %d rays, first %d: gpu %r cpu %r" % (
            label, f, len(bad), bad[0], g[bad[0]], c[bad[0]])


def both(oracle_mod, size, dim, ops):
    o = oracle_mod.Tree(size, dim)
    o.apply_ops(ops)
    p = svo.Octree(size, dim)
    p.apply_ops(ops)
    p.upload()
    return o, p


def test_device_luts_match_reference_constants():
    import ctypes
    with open(os.path.join(GOLDEN, "luts.json")) as f:
        g = json.load(f)
    rtn = (ctypes.c_uint64 * 512)()
    step = (ctypes.c_uint32 * 27)()
    mask = (ctypes.c_uint64 * 8)()
    assert svo.lib().svo_selftest_luts(rtn, step, mask) == 0
    assert list(rtn) == [int(v, 16) for v in g["RAY_TO_NODE_OCCUPANCY_BITMASK_LUT"]]
    assert list(step) == g["OCTANT_STEP_RESULT_LUT"]
    assert list(mask) == [int(v, 16) for v in g["BITMAP_MASK_FOR_OCTANT_LUT"]]


KNOWN = [
    ("test_edge_case_unreachable", scene_stairs),
    ("test_edge_case_zero_advance", scene_stairs),
    ("test_edge_case_loop_stuck", lambda: scene_stairs(True)),
    ("test_edge_case_empty_line_in_middle", lambda: (4, 1, ops_from([(INSERT, 2, 1, 1, ALBEDO, 3, 0)]))),
    ("test_edge_case_edge_raycast", scene_floor),
    ("test_edge_case_voxel_corner", scene_floor),
    ("test_edge_case_bottom_edge", scene_floor),
    ("test_edge_case_overlapping_voxels",
     lambda: (4, 1, ops_from([(INSERT, 0, 0, 0, 2, 0, 5), (INSERT, 1, 0, 0, ALBEDO, 6, 0)]))),
    ("test_edge_case_brick_undetected", lambda: scene_floor(8, 4)),
    ("test_edge_case_brick_traversal_error", lambda: (8, 2, ops_from([(INSERT, 0, 0, 0, ALBEDO, 0xFF, 0)]))),
    ("test_edge_case_brick_boundary_error", scene_brick_boundary),
    ("test_edge_case_cube_flaps", lambda: scene_dot_cube(32, 1, True, False)),
    ("test_edge_case_context_bleed", lambda: scene_dot_cube(32, 1, False, True)),
]


@pytest.mark.parametrize("name,scene", KNOWN, ids=[k[0] for k in KNOWN])
def test_known_answer_rays(oracle_mod, name, scene):
    o, p = both(oracle_mod, *scene())
    orig, d = ray_of(name)
    # the known ray plus a fan of nearby rays through the same scene
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    dirs = np.concatenate([d[None], d[None] + rng.normal(0, 0.05, size=(255, 3)).astype(np.float32)])
    dirs = np.stack([normalized(v) for v in dirs])
    origins = np.repeat(orig[None], len(dirs), axis=0)
    assert_same_hits(p.cast_host(origins, dirs), o.cast(origins, dirs), counters=True, label=name)


def test_known_answer_expectations_on_gpu(oracle_mod):
    # tests.rs:597-628 and :731-770 asserted directly on the GPU results
    o, p = both(oracle_mod, 8, 2, ops_from([(INSERT, x, y, z, ALBEDO, z, 0)
                                             for x in range(1, 8) for y in range(1, 8) for z in range(1, 8)]))
    hit = p.get_by_ray(*ray_of("test_edge_case_detailed_brick_z_edge_error"))
    assert hit is not None and hit[0] == (1, 1, 0) and tuple(hit[2]) == (0.0, 0.0, -1.0)
    o, p = both(oracle_mod, *scene_dot_cube(32, 1, True, False))
    assert p.get_by_ray(*ray_of("test_edge_case_cube_flaps")) is None
    o, p = both(oracle_mod, 512, 1, ops_from([(INSERT, 0, 0, 0, ALBEDO, 0xEE, 0), (INSERT, 511, 511, 511, ALBEDO, 0xFF, 0)]))
    origin = np.array([0, 5, -1], dtype=np.float32)
    hit = p.get_by_ray(origin, normalized(np.array([511.5, 511.5, 511.5], dtype=np.float32) - origin))
    assert hit is not None and hit[0] == (1, 0xFF, 0)


def random_rays(rng, size, n, inside_frac=0.3):
    """Mixed rays: from outside towards the volume, from inside, and axis-aligned ones."""
    o = np.empty((n, 3), dtype=np.float32)
    d = np.empty((n, 3), dtype=np.float32)
    for i in range(n):
        if rng.random() < inside_frac:
            o[i] = rng.uniform(0, size, 3)
        else:
            o[i] = rng.uniform(-0.5 * size, 1.5 * size, 3)
        t = rng.uniform(0, size, 3)
        if rng.random() < 0.05:  # axis-aligned direction (zero components)
            v = np.zeros(3, dtype=np.float32)
            v[rng.integers(0, 3)] = rng.choice([-1.0, 1.0])
        elif rng.random() < 0.05:  # through integer lattice points (voxel corners and edges)
            o[i] = np.round(o[i])
            v = np.round(t) - o[i]
        else:
            v = t - o[i]
        if not np.any(v):
            v = np.array([0, -1, 0], dtype=np.float32)
        d[i] = normalized(v.astype(np.float32))
    # inputs outside the reference's debug preconditions still get its release-mode results:
    # NaN, infinite, zero, signed-zero and subnormal direction components
    special = np.array([[np.nan, 0.5, 0.5], [0.0, 0.0, 0.0], [np.inf, 1.0, 0.0], [-0.0, -1.0, 0.0],
                        [1e-40, -1.0, 1e-40], [0.0, -0.0, 1.0], [-np.inf, -np.inf, 0.25], [np.nan] * 3],
                       dtype=np.float32)
    k = min(len(special), n // 10)
    d[:k] = special[:k]
    return o, d


@pytest.mark.parametrize("kind,size,dim", [(0, 32, 1), (0, 64, 2), (0, 128, 4), (1, 128, 8), (2, 128, 8),
                                           (3, 64, 2), (3, 128, 4), (3, 64, 16)])
def test_generated_scenes_random_rays(oracle_mod, kind, size, dim):
    ops = svo.gen_scene(kind, size, dim, seed=77 + size + dim, occupancy=0.12, spheres=6, octaves=2,
                        base_freq=1.0 / 16, height_lo=2.0, height_hi=size * 0.4, cave_threshold=0.55)
    o, p = both(oracle_mod, size, dim, ops)
    rng = np.random.default_rng(size * 100 + dim)
    origins, dirs = random_rays(rng, size, 4000)
    assert_same_hits(p.cast_host(origins, dirs), o.cast(origins, dirs, threads=8), counters=True,
                     label="kind%d %d/%d" % (kind, size, dim))


@pytest.mark.parametrize("kind,size,dim", [(0, 64, 2), (1, 128, 8), (2, 128, 4), (3, 64, 16)])
def test_literal_form_matches_oracle(oracle_mod, kind, size, dim):
    """Mode 1 sends every ray through the literal restatement; it must match the oracle as the fast form does."""
    ops = svo.gen_scene(kind, size, dim, seed=301 + size + dim, occupancy=0.12, spheres=4, octaves=2,
                        base_freq=1.0 / 16, height_lo=2.0, height_hi=size * 0.4, cave_threshold=0.55)
    o, p = both(oracle_mod, size, dim, ops)
    origins, dirs = random_rays(np.random.default_rng(kind + size), size, 3000)
    expect = o.cast(origins, dirs, threads=8)
    assert svo.lib().svo_set_cast_mode(1) == 0
    try:
        literal = p.cast_host(origins, dirs)
    finally:
        assert svo.lib().svo_set_cast_mode(0) == 0
    assert_same_hits(literal, expect, counters=True, label="literal form")
    assert_same_hits(p.cast_host(origins, dirs), expect, counters=True, label="fast form")
    assert svo.lib().svo_set_cast_mode(7) != 0


def test_small_heightfield_camera_full_parity(oracle_mod):
    """Plain method, small workload: 128^3, brick 4, heightfield + 32 spheres, 640x480 camera (307,200 rays)."""
    ops = svo.gen_scene(0, 128, 4, seed=0x5EED0001, spheres=32, octaves=2, base_freq=1.0 / 32,
                        height_lo=0.0, height_hi=96.0)
    o, p = both(oracle_mod, 128, 4, ops)
    az = 0.7
    eye = [64 + 200 * np.cos(0.5) * np.sin(az), 64 + 200 * np.sin(0.5), 64 + 200 * np.cos(0.5) * np.cos(az)]
    origins, dirs = svo.gen_camera_rays(eye, [64, 64, 64], 60.0, 640, 480)
    g = p.cast_host(origins, dirs)
    c = o.cast(origins, dirs, threads=os.cpu_count() or 8)
    assert_same_hits(g, c, counters=True, label="heightfield 640x480")
    assert 0.2 < float(np.mean(g["status"] == 1)) < 0.99


def test_device_pointer_cast_matches_host_cast(oracle_mod):
    torch = pytest.importorskip("torch")
    ops = svo.gen_scene(3, 64, 4, seed=5, occupancy=0.1, spheres=3, octaves=2, base_freq=1.0 / 16)
    o, p = both(oracle_mod, 64, 4, ops)
    origins, dirs = random_rays(np.random.default_rng(3), 64, 5000)
    dev = torch.device("cuda:0")
    cols = {k: torch.from_numpy(np.ascontiguousarray(a[:, i])).to(dev)
            for a, names in ((origins, ("ox", "oy", "oz")), (dirs, ("dx", "dy", "dz"))) for i, k in enumerate(names)}
    out = {k: torch.zeros(len(origins), dtype=getattr(torch, np.dtype(t).name), device=dev)
           for k, t in svo.HIT_FIELDS.items()}
    s = torch.cuda.current_stream().cuda_stream
    p.cast({k: v.data_ptr() for k, v in cols.items()}, {k: v.data_ptr() for k, v in out.items()}, len(origins), s)
    torch.cuda.synchronize()
    g = {k: v.cpu().numpy() for k, v in out.items()}
    assert_same_hits(g, o.cast(origins, dirs), counters=True, label="device pointers")
    # only some outputs requested: the others are skipped, the requested ones are unchanged
    part = {k: torch.zeros(len(origins), dtype=getattr(torch, np.dtype(svo.HIT_FIELDS[k]).name), device=dev)
            for k in ("status", "albedo", "px")}
    p.cast({k: v.data_ptr() for k, v in cols.items()}, {k: v.data_ptr() for k, v in part.items()}, len(origins), s)
    torch.cuda.synchronize()
    for k, v in part.items():
        assert np.array_equal(v.cpu().numpy(), g[k])
    p.cast({k: v.data_ptr() for k, v in cols.items()}, {}, 0, s)  # n == 0 is a no-op


def test_in_place_sync_after_updates(oracle_mod):
    ops = svo.gen_scene(0, 64, 4, seed=11, spheres=4, octaves=2, base_freq=1.0 / 16, height_lo=4.0, height_hi=30.0)
    o, p = both(oracle_mod, 64, 4, ops)
    rng = np.random.default_rng(5)
    origins, dirs = random_rays(rng, 64, 3000)
    assert_same_hits(p.cast_host(origins, dirs), o.cast(origins, dirs), label="before updates")
    for step in range(3):
        upd = np.zeros(200, dtype=ops.dtype)
        for i in range(200):
            x, y, z = rng.integers(0, 64, 3)
            opk = int(rng.choice([0, 0, 3, 2, 4]))
            sz = 1 if opk in (0, 3) else int(rng.choice([2, 4, 8]))
            upd[i] = (x, y, z, opk, 3, sz, int(rng.choice([0xFF0000FF, 0x00FF00FF])), int(rng.integers(1, 9)))
        o.apply_ops(upd)
        p.apply_ops(upd)
        p.sync()
        assert_same_hits(p.cast_host(origins, dirs), o.cast(origins, dirs), counters=True, label="after sync %d" % step)
    # a full re-upload of the same host state gives the same results as the in-place synced image
    p.release_device()
    p.upload()
    assert_same_hits(p.cast_host(origins, dirs), o.cast(origins, dirs), counters=True, label="after re-upload")


def test_not_uploaded_scene_is_rejected():
    p = svo.Octree(16, 2)
    p.insert((1, 1, 1), albedo=0xFF)
    with pytest.raises(RuntimeError):
        p.cast_host([[0, 0, -1]], [[0, 0, 1]])


def test_batched_multi_scene_matches_single_scene_casts(oracle_mod):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(9)
    scenes, items, expected, keep = [], [], [], []
    # the row lengths lay the items out as images (8 x 4 ray blocks, partial blocks and bands included)
    for j, (kind, size, dim, nrays, row) in enumerate([(3, 64, 2, 3000, 50), (0, 128, 4, 5000, 0), (3, 32, 8, 0, 8),
                                                       (1, 64, 8, 2000, 33), (2, 128, 4, 4000, 7),
                                                       (3, 64, 1, 1500, 1500)]):
        ops = svo.gen_scene(kind, size, dim, seed=200 + j, occupancy=0.1, spheres=2, octaves=2, base_freq=1.0 / 16,
                            height_lo=2.0, height_hi=size * 0.3)
        o, p = both(oracle_mod, size, dim, ops)
        origins, dirs = random_rays(rng, size, nrays)
        cols = {k: torch.from_numpy(np.ascontiguousarray(a[:, i]) if nrays else np.zeros(0, np.float32)).to(dev)
                for a, names in ((origins, ("ox", "oy", "oz")), (dirs, ("dx", "dy", "dz")))
                for i, k in enumerate(names)}
        out = {k: torch.zeros(max(nrays, 1), dtype=getattr(torch, np.dtype(t).name), device=dev)
               for k, t in svo.HIT_FIELDS.items()}
        items.append((p, {k: v.data_ptr() for k, v in cols.items()}, nrays, {k: v.data_ptr() for k, v in out.items()},
                      row))
        expected.append(o.cast(origins, dirs) if nrays else None)
        scenes.append(p)
        keep.append((cols, out))
    ws = svo.BatchWorkspace()
    with pytest.raises(Exception):
        ws.cast(items, svo.LaunchConfig(0, 0, 0, 2), torch.cuda.current_stream().cuda_stream)  # no such block shape
    for cfg in (svo.LaunchConfig(0, 0, 0, 0), svo.LaunchConfig(128, 32, 1, 0), svo.LaunchConfig(64, 512, 2, 0),
                svo.LaunchConfig(96, 64, 0, 4), svo.LaunchConfig(128, 32, 0, 5)):
        for _, out in keep:
            for v in out.values():
                v.zero_()
        ws.cast(items, cfg, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        for j, ((_, out), exp) in enumerate(zip(keep, expected)):
            if exp is None:
                continue
            n = len(exp["status"])
            g = {k: v.cpu().numpy()[:n] for k, v in out.items()}
            assert_same_hits(g, exp, counters=True, label="batch item %d cfg %d/%d" % (j, cfg.block, cfg.rays_per_chunk))


def test_row_layout_casts_equal_plain_casts(oracle_mod):
    # svo_cast_rows / svo_cast_host_rows / svo_cast_lod_rows hand warps 8 x 4 blocks of an image's rays;
    # the hits (and counters) are those of the plain calls, for any row length, with partial blocks
    # at the right edge, a last band of fewer than 4 rows and batches below the work-queue size
    torch = pytest.importorskip("torch")
    ops = svo.gen_scene(0, 128, 4, seed=91, spheres=6, octaves=2, base_freq=1.0 / 32, height_lo=4.0, height_hi=80.0)
    o, p = both(oracle_mod, 128, 4, ops)
    W, H = 250, 163  # 40,750 rays: above the work-queue threshold
    origins, dirs = svo.gen_camera_rays([200.0, 150.0, 220.0], [64.0, 40.0, 64.0], 60.0, W, H)
    dev = torch.device("cuda:0")
    s = torch.cuda.current_stream().cuda_stream

    def device_cast(n, row, lod=None):
        cols = {k: torch.from_numpy(np.ascontiguousarray(a[:n, i])).to(dev)
                for a, names in ((origins, ("ox", "oy", "oz")), (dirs, ("dx", "dy", "dz"))) for i, k in enumerate(names)}
        out = {k: torch.zeros(n, dtype=getattr(torch, np.dtype(t).name), device=dev) for k, t in svo.HIT_FIELDS.items()}
        rp, hp = {k: v.data_ptr() for k, v in cols.items()}, {k: v.data_ptr() for k, v in out.items()}
        if lod is None:
            p.cast(rp, hp, n, s, row_length=row)
        else:
            p.cast_lod(rp, hp, n, lod, s, row_length=row)
        torch.cuda.synchronize()
        return {k: v.cpu().numpy() for k, v in out.items()}

    def same(a, b, label):
        for k in a:
            assert np.array_equal(a[k], b[k], equal_nan=a[k].dtype.kind == "f"), (label, k)

    n = len(origins)
    plain = device_cast(n, 0)
    assert_same_hits(plain, o.cast(origins, dirs, threads=8), counters=True, label="plain")
    for row in (W, 8, 7, 13, 64, 1000, 5000, 1 << 20):
        same(device_cast(n, row), plain, "rows %d" % row)
    for m in (n - 37, 4 * W * 9 + 5, 20000):  # partial last band; below the work-queue size
        same(device_cast(m, W), {k: v[:m] for k, v in plain.items()}, "rows %d, n %d" % (W, m))
    # host buffers: in place (Grace) and staged in chunks of whole bands
    # (with and without counters: the instrumented cast is a kernel of its own; mode 2 reads host
    # memory in place even without a row layout, where the device can)
    no_counters = [k for k in svo.HIT_FIELDS if k not in COUNTERS + ["run_visits"]]
    direct = False
    if svo.lib().svo_set_host_transfer(2) == 0:
        try:
            direct = True
            same(p.cast_host(origins, dirs), plain, "host in place, plain order")
            same(p.cast_host(origins, dirs, fields=no_counters, row_length=W), {k: plain[k] for k in no_counters},
                 "host in place, rows")
        finally:
            svo.lib().svo_set_host_transfer(0)
    # 0: rows in place as 32 x 2 blocks written row by row (where the device reads host memory), 1: staged,
    # 3: rows in place, each warp writing its own 16 x 2 block
    for mode in (0, 1) + ((3,) if direct else ()):
        assert svo.lib().svo_set_host_transfer(mode) == 0
        try:
            same(p.cast_host(origins, dirs, row_length=W), plain, "host rows, transfer mode %d" % mode)
            for m, row in ((n, W), (n - 37, W), (n, 40), (n, 31), (4 * W * 9 + 5, W)):
                got = p.cast_host(origins[:m], dirs[:m], fields=no_counters, row_length=row)
                same(got, {k: plain[k][:m] for k in no_counters}, "host rows %d, n %d, mode %d" % (row, m, mode))
        finally:
            svo.lib().svo_set_host_transfer(0)
    # the LOD cast with MIP maps
    o.mip_switch(True)
    p.switch_albedo_mip_maps(True)
    p.sync()
    lod_plain = device_cast(n, 0, lod=8.0)
    same(device_cast(n, W, lod=8.0), lod_plain, "lod rows")
    assert_same_hits(lod_plain, o.cast(origins, dirs, threads=8, viewing_distance=8.0), counters=True, label="lod")


def test_work_queue_with_rays_missing_the_root(oracle_mod):
    # batches above the work-queue size whose rays mostly miss the root box: the queue writes those
    # misses at once and packs the entering rays into full warps (NaN directions and the literal
    # mode included); every field and counter equals the oracle's
    torch = pytest.importorskip("torch")
    ops = svo.gen_scene(3, 64, 4, seed=31, occupancy=0.12, spheres=3, octaves=2, base_freq=1.0 / 16)
    o, p = both(oracle_mod, 64, 4, ops)
    rng = np.random.default_rng(77)
    n = 50000
    origins = rng.uniform(-200.0, 264.0, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    dirs = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    dirs[::997] = np.float32(np.nan)
    origins[5000:5100] = np.float32(32.0)  # a run of rays from inside: whole claims that all enter
    dev = torch.device("cuda:0")
    cols = {k: torch.from_numpy(np.ascontiguousarray(a[:, i])).to(dev)
            for a, names in ((origins, ("ox", "oy", "oz")), (dirs, ("dx", "dy", "dz"))) for i, k in enumerate(names)}
    s = torch.cuda.current_stream().cuda_stream
    want = o.cast(origins, dirs, threads=8)
    assert 0.5 < (want["node_visits"] == 0).mean() < 0.99
    for mode in (0, 1):
        assert svo.lib().svo_set_cast_mode(mode) == 0
        try:
            for with_counters in (True, False):
                out = {k: torch.zeros(n, dtype=getattr(torch, np.dtype(t).name), device=dev)
                       for k, t in svo.HIT_FIELDS.items()
                       if with_counters or k not in COUNTERS + ["run_visits"]}
                p.cast({k: v.data_ptr() for k, v in cols.items()}, {k: v.data_ptr() for k, v in out.items()}, n, s)
                torch.cuda.synchronize()
                g = {k: v.cpu().numpy() for k, v in out.items()}
                assert_same_hits(g, want, counters=with_counters, label="queue mode %d" % mode)
        finally:
            svo.lib().svo_set_cast_mode(0)


def test_in_place_host_rows_with_special_rays(oracle_mod):
    """svo_cast_host_rows read and written in place (two 16 x 2 blocks per warp, each field written row by
    row): camera rays with random rays mixed in (origins outside and inside the octree, axis-aligned and
    NaN / infinite / zero / subnormal directions, which take the literal form) equal the oracle's cast,
    for row lengths with partial blocks, odd numbers of claims and a tail of 32-ray claims."""
    ops = svo.gen_scene(3, 128, 4, seed=97, occupancy=0.1, spheres=5, octaves=2, base_freq=1.0 / 16)
    o, p = both(oracle_mod, 128, 4, ops)
    # 1,440,000 rays: enough for at least four two-block claims per resident warp (smaller batches keep
    # the per-block claims)
    W, H = 1600, 900
    origins, dirs = svo.gen_camera_rays([190.0, 140.0, 210.0], [64.0, 50.0, 64.0], 60.0, W, H)
    rng = np.random.default_rng(5)
    mixed = rng.choice(len(origins), 4000, replace=False)
    ro, rd = random_rays(rng, 128, 4000)
    origins, dirs = origins.copy(), dirs.copy()
    origins[mixed], dirs[mixed] = ro, rd
    ref = o.cast(origins, dirs, threads=8)
    fields = [k for k in svo.HIT_FIELDS if k not in COUNTERS + ["run_visits"]]
    if svo.lib().svo_set_host_transfer(2) != 0:
        pytest.skip("this device does not read host memory in place")
    try:
        for row in (W, 16, 17, 31, 33, 1000, 800_000):
            got = p.cast_host(origins, dirs, fields=fields, row_length=row)
            assert_same_hits(got, ref, label="in place, rows of %d" % row)
    finally:
        svo.lib().svo_set_host_transfer(0)
