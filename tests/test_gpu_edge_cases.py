"""GPU parity on edge cases: empty trees, a tree filled by one LOD insert, very deep trees (ring-stack
restarts), rays starting inside solid voxels and on node boundaries, scenes shrunk back by clears."""
import numpy as np
import pytest

import shocovox_gb300 as svo
from helpers import ALBEDO, COMPLEX, DATA, INSERT, INSERT_AT_LOD, CLEAR_AT_LOD, normalized, ops_from
from test_gpu_cast import assert_same_hits, both, random_rays

pytestmark = pytest.mark.gpu


def check(oracle_mod, size, dim, ops, origins, dirs, label):
    o, p = both(oracle_mod, size, dim, ops)
    assert_same_hits(p.cast_host(origins, dirs), o.cast(origins, dirs, threads=8), counters=True, label=label)
    return o, p


def test_empty_tree_every_ray_misses(oracle_mod):
    origins, dirs = random_rays(np.random.default_rng(1), 64, 2000)
    o, p = check(oracle_mod, 64, 4, ops_from([]), origins, dirs, "empty tree")
    assert np.all(p.cast_host(origins, dirs, fields=("status",))["status"] != 1)


@pytest.mark.parametrize("size,dim,lod", [(16, 2, 8), (64, 4, 32), (128, 8, 64)])
def test_tree_filled_by_lod_inserts(oracle_mod, size, dim, lod):
    ops = ops_from([(INSERT_AT_LOD, x, y, z, ALBEDO, 0x11223344 + x, 0, lod)
                    for x in range(0, size, lod) for y in range(0, size, lod) for z in range(0, size, lod)])
    origins, dirs = random_rays(np.random.default_rng(size), size, 3000)
    check(oracle_mod, size, dim, ops, origins, dirs, "lod-filled %d/%d" % (size, dim))


@pytest.mark.parametrize("size,dim", [(4096, 2), (2048, 1), (1024, 8)])
def test_deep_trees_with_ring_stack_restarts(oracle_mod, size, dim):
    rng = np.random.default_rng(size + dim)
    pts = rng.integers(0, size, size=(60, 3))
    ops = ops_from([(INSERT, int(x), int(y), int(z), COMPLEX, 0xAABBCCFF, int(i) + 1) for i, (x, y, z) in enumerate(pts)] +
                   [(INSERT, size - 1, size - 1, size - 1, ALBEDO, 0xFF, 0)])
    # rays aimed at the inserted voxels (deep descents) plus the deep-stack ray of tests.rs:630-655
    origins = rng.uniform(-0.2 * size, 1.2 * size, size=(len(pts), 3)).astype(np.float32)
    dirs = np.stack([normalized(t.astype(np.float32) + np.float32(0.5) - o) for t, o in zip(pts, origins)])
    o0 = np.array([0, 5, -1], dtype=np.float32)
    origins = np.concatenate([origins, o0[None]])
    dirs = np.concatenate([dirs, normalized(np.float32(size - 1) + np.float32(0.5) - o0)[None]])
    o, p = check(oracle_mod, size, dim, ops, origins, dirs, "deep %d/%d" % (size, dim))
    assert p.cast_host(origins[-1:], dirs[-1:], fields=("status",))["status"][0] == 1


def test_rays_starting_inside_solid_voxels_and_on_boundaries(oracle_mod):
    ops = svo.gen_scene(3, 64, 4, seed=44, occupancy=0.3, spheres=2, octaves=2, base_freq=1.0 / 16)
    rng = np.random.default_rng(4)
    n = 4000
    origins = np.empty((n, 3), np.float32)
    origins[: n // 2] = rng.integers(0, 64, size=(n // 2, 3)).astype(np.float32) + np.float32(0.5)  # voxel centres
    origins[n // 2:] = (rng.integers(0, 9, size=(n - n // 2, 3)) * 8).astype(np.float32)  # node corners and faces
    dirs = np.stack([normalized(v) for v in rng.normal(size=(n, 3)).astype(np.float32)])
    check(oracle_mod, 64, 4, ops, origins, dirs, "inside/boundary origins")


def test_scene_shrunk_by_clears(oracle_mod):
    base = svo.gen_scene(0, 64, 2, seed=45, spheres=3, octaves=2, base_freq=1.0 / 16, height_lo=4.0, height_hi=40.0)
    clears = ops_from([(CLEAR_AT_LOD, x, y, z, 0, 0, 0, 16) for x in range(0, 64, 16) for y in (0, 16, 32)
                       for z in range(0, 64, 32)])
    ops = np.concatenate([base, clears])
    origins, dirs = random_rays(np.random.default_rng(45), 64, 3000)
    check(oracle_mod, 64, 2, ops, origins, dirs, "after clears")
