"""GPU parity of restart runs: when the 4-entry node stack empties, get_by_ray moves the point by
direction * 0.1 and restarts at the root (src/raytracing/raytracing_on_cpu.rs:548-562); the device
cast takes runs of restarts whose root test fails in closed form.  These cases make such runs long
(empty trees, rays through empty root cells, tiny and zero direction components, runs that reach the
work cap) and require every output, counters included, to equal the oracle's bit for bit."""
import numpy as np
import pytest

import shocovox_gb300 as svo
from helpers import ALBEDO, INSERT, normalized, ops_from
from test_gpu_cast import INT_FIELDS, COUNTERS, FLOAT_FIELDS, both

pytestmark = pytest.mark.gpu


def assert_bit_exact(gpu, cpu, label):
    n = len(cpu["status"])
    for f in INT_FIELDS + COUNTERS:
        bad = np.nonzero(gpu[f] != cpu[f])[0]
        assert len(bad) == 0, "%s: %s differs on %d/%d rays, first %d: gpu %s cpu %s" % (
            label, f, len(bad), n, bad[0], gpu[f][bad[0]], cpu[f][bad[0]])
    # the visits counted in closed form are part of node_visits, and zero where the counters are
    assert np.all(gpu["run_visits"] <= gpu["node_visits"]), label
    for f in FLOAT_FIELDS:
        g, c = gpu[f], cpu[f]
        same = (g.view(np.uint32) == c.view(np.uint32)) | (np.isnan(g) & np.isnan(c))
        bad = np.nonzero(~same)[0]
        assert len(bad) == 0, "%s: %s differs on %d rays, first %d: gpu %r cpu %r" % (
            label, f, len(bad), bad[0], g[bad[0]], c[bad[0]])


def restart_rays(rng, size, n):
    """Rays from inside and outside, with zero, negative-zero and tiny direction components."""
    o = np.where(rng.random((n, 1)) < 0.5, rng.uniform(0, size, (n, 3)),
                 rng.uniform(-0.3 * size, 1.3 * size, (n, 3))).astype(np.float32)
    d = np.stack([normalized(v) for v in rng.normal(size=(n, 3)).astype(np.float32)])
    k = np.arange(n)
    d[k % 9 == 1, 1] = 0.0
    d[k % 13 == 2, 0] = -0.0
    d[k % 11 == 3, 2] = np.float32(1e-7)
    d[k % 17 == 4, 1] = np.float32(-3e-9)
    d[k % 23 == 5] *= np.float32(1e-3)
    return o, d


@pytest.mark.parametrize("size,dim", [(64, 4), (512, 8), (4096, 8)])
def test_empty_tree_restart_runs(oracle_mod, size, dim):
    rng = np.random.default_rng(size)
    origins, dirs = restart_rays(rng, size, 1500)
    o, p = both(oracle_mod, size, dim, ops_from([]))
    gpu = p.cast_host(origins, dirs)
    assert_bit_exact(gpu, o.cast(origins, dirs, threads=8), "empty %d" % size)
    assert gpu["run_visits"].sum() > 0.9 * gpu["node_visits"].sum()


def test_sparse_corner_scene_restart_runs(oracle_mod):
    # voxels in one corner only: most root cells are empty, rays cross them in restart runs
    size = 256
    rng = np.random.default_rng(7)
    pts = rng.integers(0, 40, size=(300, 3))
    ops = ops_from([(INSERT, int(x), int(y), int(z), ALBEDO, 0x10203040 + i, 0) for i, (x, y, z) in enumerate(pts)])
    origins, dirs = restart_rays(rng, size, 3000)
    # plus rays aimed at the corner from the far side of the octree
    m = 1000
    oo = rng.uniform(0.5 * size, size, (m, 3)).astype(np.float32)
    tt = rng.uniform(0, 48, (m, 3)).astype(np.float32)
    dd = np.stack([normalized(v) for v in (tt - oo)])
    origins, dirs = np.concatenate([origins, oo]), np.concatenate([dirs, dd])
    o, p = both(oracle_mod, size, 8, ops)
    cpu = o.cast(origins, dirs, threads=8)
    assert (cpu["status"] == 1).sum() > 100
    assert_bit_exact(p.cast_host(origins, dirs), cpu, "sparse corner")


def test_horizon_camera_restart_runs(oracle_mod):
    # a heightfield seen from above the terrain with the horizon in view: the upper rays leave
    # through empty root cells
    size = 256
    ops = svo.gen_scene(0, size, 8, seed=91, spheres=0, octaves=2, base_freq=1.0 / 64, height_lo=8.0,
                        height_hi=60.0)
    origins, dirs = svo.gen_camera_rays([30.0, 110.0, 40.0], [200.0, 70.0, 220.0], 80.0, 160, 120)
    o, p = both(oracle_mod, size, 8, ops)
    cpu = o.cast(origins, dirs, threads=8)
    assert (cpu["status"] == 1).sum() > 1000 and (cpu["status"] == 0).sum() > 1000
    assert cpu["node_visits"].max() > 500  # long restart runs are present
    assert_bit_exact(p.cast_host(origins, dirs), cpu, "horizon camera")


def test_restart_runs_reaching_the_work_cap(oracle_mod):
    # directions so small that the point never moves (or moves too slowly) inside an empty tree:
    # the reference loops forever; both sides stop at the same work cap with status 2
    size = 64
    origins = np.array([[10.5, 20.25, 30.0], [1.0, 1.0, 1.0], [63.0, 0.5, 32.0], [5.0, 5.0, 5.0]], np.float32)
    dirs = np.array([[1e-30, 0.0, 0.0], [0.0, 0.0, -0.0], [-1e-9, 1e-9, 0.0], [1e-6, 0.0, 0.0]], np.float32)
    o, p = both(oracle_mod, size, 4, ops_from([]))
    cpu = o.cast(origins, dirs, threads=4)
    assert list(cpu["status"][:3]) == [2, 2, 2]
    assert_bit_exact(p.cast_host(origins, dirs), cpu, "work cap")
