"""GPU parity of the casts that stage the top tree levels in shared memory.

A cast with staging depth K copies each scene's Internal nodes of depth < K into shared memory and
reads them there (svo_set_staging_depth for the plain casts, svo_launch_config.staging_depth for the
batched cast).  The hits, counters included, must be the oracle's at every depth, in the plain and row
orders, the batched cast (index order, ray sort, allocation-free), with more scenes than the staged
records hold, and after in-place syncs that change the top levels.
"""
import ctypes

import numpy as np
import pytest

import shocovox_gb300 as svo
from test_gpu_cast import assert_same_hits, both, random_rays

pytestmark = pytest.mark.gpu
DEPTHS = (0, 1, 2, 3, 4)


@pytest.fixture
def staging():
    yield lambda k: svo.check(svo.lib().svo_set_staging_depth(k))
    svo.lib().svo_set_staging_depth(0)


def _scene(kind, size, dim, seed):
    return svo.gen_scene(kind, size, dim, seed=seed, occupancy=0.08, spheres=4, octaves=2, base_freq=1.0 / 16,
                         height_lo=2.0, height_hi=size * 0.35)


@pytest.mark.parametrize("kind,size,dim", [(0, 128, 4), (1, 256, 2), (3, 64, 1), (2, 512, 4)])
def test_plain_cast_at_every_staging_depth(oracle_mod, staging, kind, size, dim):
    ops = _scene(kind, size, dim, 40 + kind)
    o, p = both(oracle_mod, size, dim, ops)
    rng = np.random.default_rng(kind)
    origins, dirs = random_rays(rng, size, 40_000)  # above the work-queue threshold
    ref = o.cast(origins, dirs)
    cam_o, cam_d = svo.gen_camera_rays([1.3 * size, 0.8 * size, -0.2 * size], [size / 2, size / 4, size / 2], 60.0,
                                       256, 160)
    cam_ref = o.cast(cam_o, cam_d)
    for k in DEPTHS:
        staging(k)
        assert_same_hits(p.cast_host(origins, dirs), ref, counters=True, label="depth %d" % k)
        fields = [f for f in svo.HIT_FIELDS if f not in ("node_visits", "child_reads", "voxel_reads", "run_visits")]
        assert_same_hits(p.cast_host(origins, dirs, fields=fields), ref, label="depth %d uncounted" % k)
        assert_same_hits(p.cast_host(cam_o, cam_d, fields=fields, row_length=256), cam_ref, label="rows %d" % k)


def test_deep_sparse_tree_at_every_staging_depth(oracle_mod, staging):
    """4096^3 with brick 2: eleven levels, mostly empty; restarts cross staged and unstaged levels."""
    from helpers import INSERT, COMPLEX, ops_from
    rng = np.random.default_rng(3)
    recs = [(INSERT, int(x), int(y), int(z), COMPLEX, 0x10203040 + i, 7 + i)
            for i, (x, y, z) in enumerate(rng.integers(0, 4096, (300, 3)))]
    o, p = both(oracle_mod, 4096, 2, ops_from(recs))
    origins, dirs = random_rays(rng, 4096, 40_000, inside_frac=0.6)
    ref = o.cast(origins, dirs)
    for k in DEPTHS:
        staging(k)
        assert_same_hits(p.cast_host(origins, dirs), ref, counters=True, label="deep depth %d" % k)


def test_staging_follows_in_place_syncs(oracle_mod, staging):
    """Inserts and aligned insert_at_lod cubes up to half the octree: new Internal nodes appear at the
    top levels (in the empty sky) and others collapse under solid cubes, so the top table changes at
    every sync.  (Clears are left out: many of them reach the reference's panics, which other tests
    cover.)"""
    ops = _scene(0, 64, 2, 9)
    o, p = both(oracle_mod, 64, 2, ops)
    rng = np.random.default_rng(11)
    origins, dirs = random_rays(rng, 64, 40_000)
    staging(4)
    for step in range(4):
        upd = np.zeros(300, dtype=ops.dtype)
        for i in range(300):
            opk = int(rng.choice([0, 0, 2]))
            sz = 1 if opk == 0 else int(rng.choice([2, 4, 8, 16, 32]))
            x, y, z = rng.integers(0, 64 // sz, 3) * sz
            upd[i] = (x, y, z, opk, 3, sz, int(rng.choice([0xFF0000FF, 0x00FF00FF])), int(rng.integers(1, 9)))
        o.apply_ops(upd)
        p.apply_ops(upd)
        p.sync()
        assert_same_hits(p.cast_host(origins, dirs), o.cast(origins, dirs), counters=True, label="sync %d" % step)


def _batched(torch, scenes, rays, rows, cfg, noalloc=False):
    dev = torch.device("cuda:0")
    tmap = {np.uint8: torch.uint8, np.uint32: torch.int32, np.float32: torch.float32}
    outs, items = [], []
    for sc, (o, d), row in zip(scenes, rays, rows):
        n = len(o)
        r = {k: torch.from_numpy(np.ascontiguousarray(a[:, i])).to(dev)
             for a, ks in ((o, ("ox", "oy", "oz")), (d, ("dx", "dy", "dz"))) for i, k in enumerate(ks)}
        out = {k: torch.zeros(max(n, 1), dtype=tmap[t], device=dev) for k, t in svo.HIT_FIELDS.items()}
        outs.append((out, r))
        items.append((sc, {k: v.data_ptr() for k, v in r.items()}, n, {k: v.data_ptr() for k, v in out.items()}, row))
    if noalloc:
        from shocovox_gb300._lib import BatchItem, Hits, Rays
        arr = (BatchItem * len(items))()
        for i, (sc, rp, n, hp, row) in enumerate(items):
            arr[i].scene = sc.handle
            arr[i].rays = Rays(*[ctypes.c_void_p(rp[k]) for k in ("ox", "oy", "oz", "dx", "dy", "dz")])
            arr[i].n = n
            arr[i].hits = Hits(**{k: ctypes.c_void_p(hp[k]) for k in svo.HIT_FIELDS})
            arr[i].row_length = row
        svo.check(svo.lib().svo_cast_batched_noalloc(arr, len(items), ctypes.byref(cfg), None))
    else:
        svo.BatchWorkspace().cast(items, cfg, 0)
    torch.cuda.synchronize()
    return [{k: v[:len(o)].cpu().numpy().view(svo.HIT_FIELDS[k]) for k, v in out.items()}
            for (out, _), (o, _) in zip(outs, rays)]


@pytest.mark.parametrize("sort_key", [0, 1])
@pytest.mark.parametrize("noalloc", [False, True])
def test_batched_cast_at_every_staging_depth(oracle_mod, sort_key, noalloc):
    if noalloc and sort_key:
        pytest.skip("the allocation-free cast has no ray sort")
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(21)
    scenes, rays, rows, refs = [], [], [], []
    for j, (kind, size, dim) in enumerate([(0, 128, 4), (3, 64, 2), (2, 256, 8), (1, 128, 2)]):
        o, p = both(oracle_mod, size, dim, _scene(kind, size, dim, 60 + j))
        ro, rd = random_rays(rng, size, 3000)
        co, cd = svo.gen_camera_rays([1.4 * size, 0.9 * size, 1.1 * size], [size / 2, size / 3, size / 2], 60.0, 64, 40)
        for (a, b), row in (((ro, rd), 0), ((co, cd), 64)):
            scenes.append(p)
            rays.append((a, b))
            rows.append(row)
            refs.append(o.cast(a, b))
    for k in DEPTHS:
        cfg = svo.LaunchConfig(128, 32, 0, 0, sort_key, k)
        got = _batched(torch, scenes, rays, rows, cfg, noalloc)
        for j, (g, r) in enumerate(zip(got, refs)):
            assert_same_hits(g, r, counters=True, label="batched depth %d item %d" % (k, j))


def test_batched_staging_past_the_shared_memory_budget(oracle_mod):
    """Sixteen scenes at depth 4 hold more records than a block stages: the scenes past the budget are
    read from L1/L2, with the same results."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(31)
    scenes, rays, rows, refs = [], [], [], []
    for j in range(16):
        o, p = both(oracle_mod, 256, 2, _scene(3, 256, 2, 80 + j))
        a, b = random_rays(rng, 256, 1500)
        scenes.append(p)
        rays.append((a, b))
        rows.append(0)
        refs.append(o.cast(a, b))
    got = _batched(torch, scenes, rays, rows, svo.LaunchConfig(96, 64, 0, 0, 0, 4))
    for j, (g, r) in enumerate(zip(got, refs)):
        assert_same_hits(g, r, counters=True, label="item %d" % j)


def test_staging_depth_is_checked():
    assert svo.lib().svo_set_staging_depth(5) == 6
    assert svo.lib().svo_set_staging_depth(-1) == 6
    assert svo.lib().svo_set_staging_depth(0) == 0
