"""GPU parity of get_by_ray_at_lod with MIP maps (svo_cast_lod) against the oracle's restatement
(src/raytracing/raytracing_on_cpu.rs:325-565, src/octree/mipmap.rs): every field, counters included,
over viewing distances from near (MIPs read at the top levels) to f32::MAX (MIPs read only where the
level counter has drifted through ring-stack restarts)."""
import numpy as np
import pytest

import shocovox_gb300 as svo
from helpers import ALBEDO, INSERT, ops_from
from test_gpu_cast import COUNTERS, FLOAT_FIELDS, INT_FIELDS, random_rays

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
FLT_MAX = float(np.finfo(np.float32).max)


def cast_lod(tree, origins, dirs, vd):
    dev = torch.device("cuda:0")
    cols = {k: torch.from_numpy(np.ascontiguousarray(a[:, i])).to(dev)
            for a, names in ((origins, ("ox", "oy", "oz")), (dirs, ("dx", "dy", "dz"))) for i, k in enumerate(names)}
    out = {k: torch.zeros(len(origins), dtype=getattr(torch, np.dtype(t).name), device=dev)
           for k, t in svo.HIT_FIELDS.items()}
    tree.cast_lod({k: v.data_ptr() for k, v in cols.items()}, {k: v.data_ptr() for k, v in out.items()}, len(origins),
                  vd, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


def assert_equal(gpu, cpu, label):
    for f in INT_FIELDS + COUNTERS:
        bad = np.nonzero(gpu[f] != cpu[f])[0]
        assert len(bad) == 0, "%s: %s differs on %d rays, first %d: gpu %s cpu %s" % (
            label, f, len(bad), bad[0], gpu[f][bad[0]], cpu[f][bad[0]])
    for f in FLOAT_FIELDS:
        g, c = gpu[f], cpu[f]
        same = (g.view(np.uint32) == c.view(np.uint32)) | (np.isnan(g) & np.isnan(c))
        bad = np.nonzero(~same)[0]
        assert len(bad) == 0, "%s: %s differs on %d rays, first %d: gpu %r cpu %r" % (
            label, f, len(bad), bad[0], g[bad[0]], c[bad[0]])


def pair(oracle_mod, size, dim, ops, configure):
    o = oracle_mod.Tree(size, dim)
    p = svo.Octree(size, dim)
    configure(o, p)
    o.apply_ops(ops)
    p.apply_ops(ops)
    return o, p


def enable_after(method=None):
    def configure(o, p):
        if method is not None:
            for level in (1, 2, 3, 4, 5):
                o.mip_set_method(level, method, 0.25)
                p.set_mip_method(level, method, 0.25)
    return configure


@pytest.mark.parametrize("method", [None, 0, 1, 3])
def test_lod_cast_heightfield(oracle_mod, method):
    ops = svo.gen_scene(0, 128, 4, seed=0x5EED0001 + (method or 0), spheres=8, octaves=2, base_freq=1.0 / 32,
                        height_lo=0.0, height_hi=96.0)
    o, p = pair(oracle_mod, 128, 4, ops, enable_after(method))
    o.mip_switch(True)
    p.switch_albedo_mip_maps(True)
    p.upload()
    origins, dirs = random_rays(np.random.default_rng(9), 128, 4000)
    cam_o, cam_d = svo.gen_camera_rays([300.0, 200.0, 280.0], [64.0, 40.0, 64.0], 60.0, 64, 48)
    origins, dirs = np.concatenate([origins, cam_o]), np.concatenate([dirs, cam_d])
    mip_hits = 0
    for vd in (2.0, 16.0, 128.0, 1e4, FLT_MAX):
        cpu = o.cast(origins, dirs, threads=8, viewing_distance=vd)
        assert_equal(cast_lod(p, origins, dirs, vd), cpu, "heightfield vd=%g" % vd)
        mip_hits += int((cpu["brick_octant"] == 8).sum())
    assert mip_hits > 100


def test_lod_cast_deep_tree_level_drift(oracle_mod):
    # a deep tree: ring-stack restarts let the level counter drift below 1, where even f32::MAX reads MIPs
    size = 1024
    rng = np.random.default_rng(4)
    pts = rng.integers(0, size, size=(300, 3))
    ops = ops_from([(INSERT, int(x), int(y), int(z), ALBEDO, int(0x10203000 + 0x11 * i) | 0xFF, 0, 1)
                    for i, (x, y, z) in enumerate(pts)])
    o, p = pair(oracle_mod, size, 2, ops, enable_after(0))
    o.mip_switch(True)
    p.switch_albedo_mip_maps(True)
    p.upload()
    origins = rng.uniform(-0.2 * size, 1.2 * size, size=(len(pts), 3)).astype(np.float32)
    targets = pts.astype(np.float32) + np.float32(0.5)
    d = targets - origins
    dirs = (d / np.sqrt((d * d).sum(1, keepdims=True))).astype(np.float32)
    o2, d2 = random_rays(np.random.default_rng(5), size, 2000)
    origins, dirs = np.concatenate([origins, o2]), np.concatenate([dirs, d2])
    for vd in (64.0, FLT_MAX):
        assert_equal(cast_lod(p, origins, dirs, vd), o.cast(origins, dirs, threads=8, viewing_distance=vd),
                     "deep vd=%g" % vd)


def test_lod_cast_after_edits_and_sync(oracle_mod):
    # MIPs maintained by inserts and clears while enabled, then written to the device in place
    ops = svo.gen_scene(3, 64, 4, seed=21, occupancy=0.12, spheres=2, octaves=2, base_freq=1.0 / 16)
    o, p = pair(oracle_mod, 64, 4, ops, enable_after(0))
    o.mip_switch(True)
    p.switch_albedo_mip_maps(True)
    p.upload()
    rng = np.random.default_rng(8)
    edits = ops_from([(INSERT, int(x), int(y), int(z), ALBEDO, 0xC0FFEEFF, 0, 1)
                      for x, y, z in rng.integers(0, 64, size=(200, 3))])
    o.apply_ops(edits)
    p.apply_ops(edits)
    p.sync()
    origins, dirs = random_rays(np.random.default_rng(6), 64, 3000)
    for vd in (4.0, 32.0):
        assert_equal(cast_lod(p, origins, dirs, vd), o.cast(origins, dirs, threads=8, viewing_distance=vd),
                     "edited vd=%g" % vd)


def test_lod_cast_without_mips_is_the_plain_cast(oracle_mod):
    ops = svo.gen_scene(0, 64, 4, seed=3, spheres=2, octaves=2, base_freq=1.0 / 16, height_lo=4.0, height_hi=40.0)
    o, p = pair(oracle_mod, 64, 4, ops, enable_after(None))
    p.upload()
    origins, dirs = random_rays(np.random.default_rng(7), 64, 2000)
    assert_equal(cast_lod(p, origins, dirs, 1.0), o.cast(origins, dirs, threads=8), "no mips")
