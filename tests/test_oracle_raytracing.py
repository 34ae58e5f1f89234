"""Ports of the reference's ray-cast known-answer tests (src/raytracing/tests.rs) onto the oracle.

Hit identity follows `OctreeEntry`: entry_kind 1 = Visual(albedo),
2 = Informative(user data), 3 = Complex.  The randomized tests of the
reference (tests.rs:144-251) use an unseeded thread_rng; here they run
over fixed seeds.
"""
import numpy as np
import pytest

from helpers import (ALBEDO, DATA, INSERT, normalized, ops_from, ray_of, scene_brick_boundary, scene_dot_cube,
                     scene_floor, scene_stairs)

VISUAL, INFORMATIVE = 1, 2


def build(oracle_mod, scene):
    size, dim, ops = scene
    t = oracle_mod.Tree(size, dim)
    t.apply_ops(ops)
    return t


def cast(t, test):
    o, d = ray_of(test)
    return t.cast_one(o, d)


def test_unreachable(oracle_mod):  # tests.rs:253-294
    t = build(oracle_mod, scene_stairs())
    assert cast(t, "test_edge_case_unreachable")["status"] in (0, 1)


def test_empty_line_in_middle(oracle_mod):  # tests.rs:296-315
    t = build(oracle_mod, (4, 1, ops_from([(INSERT, 2, 1, 1, ALBEDO, 3, 0)])))
    assert cast(t, "test_edge_case_empty_line_in_middle")["status"] == 1


def test_zero_advance(oracle_mod):  # tests.rs:317-358
    t = build(oracle_mod, scene_stairs())
    assert cast(t, "test_edge_case_zero_advance")["status"] == 1


def test_ray_behind_octree(oracle_mod):  # tests.rs:360-375
    t = build(oracle_mod, (4, 1, ops_from([(INSERT, 0, 3, 0, DATA, 0, 5)])))
    assert t.get((0, 3, 0)) == (INFORMATIVE, 0, 5)
    origin = np.array([2, 2, -5], dtype=np.float32)
    h = t.cast_one(origin, normalized(np.array([0, 3, 0], dtype=np.float32) - origin))
    assert h["status"] == 1 and h["entry_kind"] == INFORMATIVE and h["user"] == 5


def test_overlapping_voxels(oracle_mod):  # tests.rs:377-402
    t = build(oracle_mod, (4, 1, ops_from([(INSERT, 0, 0, 0, DATA, 0, 5), (INSERT, 1, 0, 0, ALBEDO, 6, 0)])))
    h = cast(t, "test_edge_case_overlapping_voxels")
    assert h["status"] == 1 and h["entry_kind"] == VISUAL and h["albedo"] == 6


def test_edge_raycast(oracle_mod):  # tests.rs:404-429
    t = build(oracle_mod, scene_floor())
    h = cast(t, "test_edge_case_edge_raycast")
    assert h["status"] == 0 or (h["entry_kind"] == INFORMATIVE and h["user"] == 5)


@pytest.mark.parametrize("name", ["test_edge_case_voxel_corner", "test_edge_case_bottom_edge"])
def test_floor_hits(oracle_mod, name):  # tests.rs:431-485
    t = build(oracle_mod, scene_floor())
    h = cast(t, name)
    assert h["status"] == 1 and h["entry_kind"] == INFORMATIVE and h["user"] == 5


def test_loop_stuck(oracle_mod):  # tests.rs:487-528
    t = build(oracle_mod, scene_stairs(loop_stuck_variant=True))
    assert cast(t, "test_edge_case_loop_stuck")["status"] in (0, 1)


def test_brick_undetected(oracle_mod):  # tests.rs:530-563
    t = build(oracle_mod, scene_floor(8, 4))
    for x in range(4):
        for z in range(4):
            assert t.get((x, 0, z)) == (INFORMATIVE, 0, 5)
    h = cast(t, "test_edge_case_brick_undetected")
    assert h["status"] == 1 and h["entry_kind"] == INFORMATIVE and h["user"] == 5


def test_detailed_brick_undetected(oracle_mod):  # tests.rs:565-595
    t = build(oracle_mod, (8, 2, ops_from([(INSERT, x, y, z, DATA, 0, 5)
                                             for x in range(8) for y in range(8) for z in range(8)])))
    h = cast(t, "test_edge_case_detailed_brick_undetected")
    assert h["status"] == 1 and h["entry_kind"] == INFORMATIVE and h["user"] == 5


def test_detailed_brick_z_edge_error(oracle_mod):  # tests.rs:597-628
    t = build(oracle_mod, (8, 2, ops_from([(INSERT, x, y, z, ALBEDO, z, 0)
                                             for x in range(1, 8) for y in range(1, 8) for z in range(1, 8)])))
    h = cast(t, "test_edge_case_detailed_brick_z_edge_error")
    assert h["status"] == 1 and h["entry_kind"] == VISUAL and h["albedo"] == 1
    assert (h["nx"], h["ny"], h["nz"]) == (0.0, 0.0, -1.0)


def test_deep_stack(oracle_mod):  # tests.rs:630-655
    t = build(oracle_mod, (512, 1, ops_from([(INSERT, 0, 0, 0, ALBEDO, 0xEE, 0), (INSERT, 511, 511, 511, ALBEDO, 0xFF, 0)])))
    origin = np.array([0, 5, -1], dtype=np.float32)
    d = normalized(np.array([511, 511, 511], dtype=np.float32) + np.float32(0.5) - origin)
    h = t.cast_one(origin, d)
    assert h["status"] == 1 and h["entry_kind"] == VISUAL and h["albedo"] == 0xFF


def test_brick_traversal_error(oracle_mod):  # tests.rs:657-685
    t = build(oracle_mod, (8, 2, ops_from([(INSERT, 0, 0, 0, ALBEDO, 0xFF, 0)])))
    h = cast(t, "test_edge_case_brick_traversal_error")
    assert h["status"] == 1 and h["entry_kind"] == VISUAL and h["albedo"] == 0xFF
    assert np.linalg.norm([h["nx"], h["ny"], h["nz"]]) < 1.1


def test_brick_boundary_error(oracle_mod):  # tests.rs:687-729
    t = build(oracle_mod, scene_brick_boundary())
    assert cast(t, "test_edge_case_brick_boundary_error")["status"] == 1


def test_cube_flaps(oracle_mod):  # tests.rs:731-770 (expects a miss)
    t = build(oracle_mod, scene_dot_cube(32, 1, corner_cube=True, lattice=False))
    assert cast(t, "test_edge_case_cube_flaps")["status"] == 0


def test_context_bleed(oracle_mod):  # tests.rs:772-813
    t = build(oracle_mod, scene_dot_cube(32, 1, corner_cube=False, lattice=True))
    assert cast(t, "test_edge_case_context_bleed")["status"] == 1


def _random_fill(rng, size, dim, with_z):
    filled = []
    rec = []
    for x in range(1, 4):
        for y in range(1, 4):
            zs = range(1, 4) if with_z else (1,)
            for z in zs:
                if 10 > rng.integers(0, 20):
                    rec.append((INSERT, x, y, z, DATA, 0, 5))
                    filled.append((x, y, z))
    return (size, dim, ops_from(rec)), filled


@pytest.mark.parametrize("seed", range(16))
@pytest.mark.parametrize("size,dim,with_z,edge", [(4, 1, False, False), (4, 2, False, False),
                                                  (8, 1, True, True), (16, 1, True, False)])
def test_randomized_get_by_ray(oracle_mod, seed, size, dim, with_z, edge):  # tests.rs:144-251
    rng = np.random.default_rng(seed)
    scene, filled = _random_fill(rng, size, dim, with_z)
    if not filled:
        return
    t = build(oracle_mod, scene)
    for p in filled:
        if edge:  # make_edge_ray_point_to (tests.rs:188-198), target offset by 0.1
            origin = np.array([rng.integers(0, 8), rng.integers(0, 8), 8], dtype=np.float32)
            target = np.array(p, dtype=np.float32) + np.float32(0.1)
        else:  # make_ray_point_to (tests.rs:132-142)
            origin = rng.integers(8, 16, size=3).astype(np.float32)
            target = np.array(p, dtype=np.float32)
            if size == 16:
                assert t.get(p) == (INFORMATIVE, 0, 5)
        h = t.cast_one(origin, normalized(target - origin))
        assert h["status"] == 1 and h["entry_kind"] == INFORMATIVE and h["user"] == 5
