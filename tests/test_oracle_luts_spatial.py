"""Pins the oracle's spatial layer to the reference.

* The look-up tables the oracle regenerates with the reference's generator
  functions (src/spatial/lut.rs:7-152) must equal the constants written in
  src/spatial/lut.rs:156-896 (extracted into tests/golden/luts.json).
* Ports of src/spatial/tests.rs, src/spatial/raytracing/tests.rs and
  src/spatial/math/tests.rs.
"""
import json
import os

import numpy as np
import pytest

from helpers import GOLDEN, normalized, ray_of

SR = "src/spatial/raytracing/tests.rs"
SM = "src/spatial/math/tests.rs"


@pytest.fixture(scope="module")
def golden_luts():
    with open(os.path.join(GOLDEN, "luts.json")) as f:
        return json.load(f)


def test_luts_match_reference_constants(oracle_mod, golden_luts):
    L = oracle_mod.luts()
    g = golden_luts
    assert [int(v, 16) for v in g["RAY_TO_NODE_OCCUPANCY_BITMASK_LUT"]] == [int(v) for v in L["RAY_TO_NODE_OCCUPANCY_BITMASK_LUT"]]
    assert g["OCTANT_STEP_RESULT_LUT"] == [int(v) for v in L["OCTANT_STEP_RESULT_LUT"]]
    assert [int(v, 16) for v in g["BITMAP_MASK_FOR_OCTANT_LUT"]] == [int(v) for v in L["BITMAP_MASK_FOR_OCTANT_LUT"]]
    assert g["BITMAP_INDEX_LUT"] == [int(v) for v in L["BITMAP_INDEX_LUT"]]
    assert np.array_equal(np.array(g["OCTANT_OFFSET_REGION_LUT"], dtype=np.float32), L["OCTANT_OFFSET_REGION_LUT"])


# src/spatial/tests.rs:22-32
def test_hash_region(oracle_mod):
    h = oracle_mod.hash_region
    assert h([0, 0, 0], 5.0) == 0
    assert h([6, 0, 0], 5.0) == 1
    assert h([0, 0, 6], 5.0) == 2
    assert h([6, 0, 6], 5.0) == 3
    assert h([0, 6, 0], 5.0) == 4
    assert h([6, 6, 0], 5.0) == 5
    assert h([0, 6, 6], 5.0) == 6
    assert h([6, 6, 6], 5.0) == 7


# src/spatial/tests.rs:42-66
def test_flat_projection(oracle_mod):
    fp = oracle_mod.flat_projection
    D = 10
    assert fp(0, 0, 0, D) == 0
    assert fp(10, 0, 0, D) == D
    assert fp(0, 1, 0, D) == D
    assert fp(0, 0, 1, D) == D * D
    assert fp(0, 0, 4, D) == D * D * 4
    assert fp(3, 0, 4, D) == D * D * 4 + 3
    assert fp(3, 2, 4, D) == D * D * 4 + D * 2 + 3
    seen = {fp(x, y, z, D) for x in range(D) for y in range(D) for z in range(D)}
    assert len(seen) == D ** 3


# src/spatial/tests.rs:68-93
def test_bitmap_flat_projection(oracle_mod):
    p = oracle_mod.position_in_bitmap
    assert p(0, 0, 0, 4) == 0 and p(0, 0, 2, 4) == 32 and p(3, 3, 3, 4) == 63
    assert p(0, 0, 0, 10) == 0 and p(0, 0, 5, 10) == 32 and p(5, 5, 5, 10) == 42 and p(9, 9, 9, 10) == 63
    assert [p(1, 0, 0, 2), p(0, 1, 0, 2), p(1, 1, 0, 2), p(0, 0, 1, 2), p(1, 0, 1, 2), p(0, 1, 1, 2), p(1, 1, 1, 2)] == \
        [2, 8, 10, 32, 34, 40, 42]


# src/spatial/math/tests.rs:93-186 (the should_panic cases are debug_assert!s, absent in release builds)
def test_occupancy_bitmaps(oracle_mod):
    s = oracle_mod.set_occupancy
    m = s((0, 0, 0), 1, 4, True, 0)
    assert m == 0x1
    m = s((3, 3, 3), 1, 4, True, m)
    assert m == 0x8000000000000001
    m = s((2, 2, 2), 1, 4, True, m)
    assert m == 0x8000040000000001
    assert s((0, 0, 0), 1, 1, False, 2 ** 64 - 1) == 0
    assert s((0, 0, 0), 1, 1, True, 0) == 2 ** 64 - 1
    m = s((0, 0, 0), 1, 2, True, 0)
    assert m == 0x0000000000330033
    assert s((1, 1, 1), 1, 2, True, m) == 0xCC00CC0000330033
    assert s((0, 0, 0), 3, 4, True, 0) == 0x77707770777
    assert s((0, 0, 0), 2, 2, True, 0) == 0xFFFFFFFFFFFFFFFF
    assert s((0, 0, 0), 5, 4, True, 0) == 0xFFFFFFFFFFFFFFFF
    assert s((0, 0, 0), 3, 2, True, 0) == 0xFFFFFFFFFFFFFFFF


# src/spatial/raytracing/tests.rs:5-39 and src/spatial/math/tests.rs:11-24
def test_plane_line_intersection(oracle_mod):
    pli = oracle_mod.plane_line_intersection
    assert pli([0, 0, 0], [0, 1, 0], [0, 1, 0], [1, 0, 0]) is None
    assert pli([0, 0, 0], [0, 1, 0], [0, 1, 0], [0, -1, 0]) == 1.0
    assert pli([0, 0, 0], [0, 1, 0], [0, 0, 0], [1, 0, 0]) == 0.0
    assert pli([0, 0, 0], [0, 1, 0], [0, 1, 0], [0, 1, 0]) == -1.0


# src/spatial/raytracing/tests.rs:41-87
def test_cube_bounds(oracle_mod):
    expect = [(0, 0, 0), (5, 0, 0), (0, 0, 5), (5, 0, 5), (0, 5, 0), (5, 5, 0), (0, 5, 5), (5, 5, 5)]
    for o, e in enumerate(expect):
        b = oracle_mod.child_bounds([0, 0, 0, 10.0], o)
        assert tuple(b[:3]) == e and b[3] == 5.0


# src/spatial/raytracing/tests.rs:89-200
def test_cube_contains_ray(oracle_mod):
    cube = [0, 0, 0, 4.0]
    rays = [ray_of("test_cube_contains_ray", SR, i) for i in range(6)]
    ray_above, ray_below, ray_miss, ray_hit, corner_hit, ray_still_miss = rays
    ix = oracle_mod.intersect_ray
    assert ix(cube, np.concatenate(ray_above)) is not None
    assert ix(cube, np.concatenate(ray_below)) is not None
    assert ix(cube, np.concatenate(ray_miss)) is None
    # the (1,1,1) and (1,100,1) directions are `.normalized()` in the test
    assert ix(cube, np.concatenate([ray_hit[0], normalized(ray_hit[1])])) is not None
    assert ix(cube, np.concatenate([corner_hit[0], normalized(corner_hit[1])])) is not None
    origin = np.array([4, -1, 4], dtype=np.float32)
    d = normalized(np.array([4.055, 4.055, 4.055], dtype=np.float32) - origin)
    assert ix(cube, np.concatenate([origin, d])) is None
    assert ix(cube, np.concatenate([ray_still_miss[0], normalized(ray_still_miss[1])])) is None


# src/spatial/raytracing/tests.rs:202-278
def test_cube_intersect_edge_cases(oracle_mod):
    ix = oracle_mod.intersect_ray
    r = ray_of("test_edge_case_cube_intersect_inwards_pointing_vector", SR)
    hit = ix([0, 0, 0, 8.0], np.concatenate(r))
    assert hit == ("hit", 0.0)
    r = ray_of("test_edge_case_cube_internal_ray_targeting_corners", SR)
    assert ix([0, 0, 0, 16.0], np.concatenate(r)) == ("inside", None)
    r = ray_of("test_edge_case_cube_bottom_edge", SR)
    hit = ix([0, 2, 0, 2.0], np.concatenate(r))
    assert hit is not None and hit[0] == "hit" and hit[1] > 0.0


# src/spatial/math/tests.rs:26-51
def test_cube_top_hit(oracle_mod):
    o, d = ray_of("test_edge_case_cube_top_hit", SM)
    hit = oracle_mod.intersect_ray([2, 0, 0, 2.0], np.concatenate([o, d]))
    assert hit[0] == "hit" and abs(hit[1] - 11.077772) < 0.001
    p = o + d * np.float32(hit[1])
    assert abs(p[1] - 2.0) < 0.001


# src/spatial/math/tests.rs:53-66
def test_impact_normal(oracle_mod):
    c = [0, 0, 0, 2.0]
    n = oracle_mod.cube_impact_normal
    assert tuple(n(c, [1, 1, 2])) == (0, 0, 1)
    assert tuple(n(c, [1, 2, 1])) == (0, 1, 0)
    assert tuple(n(c, [2, 1, 1])) == (1, 0, 0)
    assert tuple(n(c, [1, 1, 0])) == (0, 0, -1)
    assert tuple(n(c, [1, 0, 1])) == (0, -1, 0)
    assert tuple(n(c, [0, 1, 1])) == (-1, 0, 0)


# src/raytracing/tests.rs:816-912 (NodeStack ring semantics)
def test_node_stack(oracle_mod):
    S = oracle_mod.Stack
    assert S(4).is_empty()
    s = S(3)
    for v in (1, 2, 3, 4):
        s.push(v)
    assert s.last() == 4 and s.pop() == 4
    assert s.last() == 3 and s.pop() == 3
    assert s.last() == 2 and s.pop() == 2
    assert s.pop() is None
    s = S(3)
    for v in (10, 20, 30):
        s.push(v)
    assert s.last() == 30
    s.push(40)
    assert s.last() == 40
    s = S(3)
    for v in (100, 200, 300):
        s.push(v)
    assert s.add_last(50) and s.last() == 350
    s = S(3)
    for v in (5, 15, 25):
        s.push(v)
    assert [s.pop(), s.pop(), s.pop(), s.pop()] == [25, 15, 5, None]


# ---- BrickData::is_empty_throughout / is_part_empty_throughout (src/octree/tests.rs:8-158) ----
# The palettes of those tests: one colour (0, 0, 0, alpha 100) and one user datum 0; a voxel holds
# colour index 0 and no datum (pix_visual(0)); the empty marker is u32::MAX.
EMPTY_MARK = 0xFFFFFFFF
PAL_C, PAL_D = [0x00000064], [0]
OCTANT_OFFSET = [(0, 0, 0), (1, 0, 0), (0, 0, 1), (1, 0, 1), (0, 1, 0), (1, 1, 0), (0, 1, 1), (1, 1, 1)]


def _brick(dim):  # every voxel pix_visual(0): colour index 0, no user datum
    return [0xFFFF << 16] * dim ** 3


def test_brick_octant_empty(oracle_mod):  # tests.rs:8-31
    for o in range(8):
        assert oracle_mod.brick_empty_throughout(0, [], 1, o, PAL_C, PAL_D)
        assert not oracle_mod.brick_empty_throughout(2, _brick(1), 1, o, PAL_C, PAL_D)


def test_brick_octant_empty_where_dim_is_2(oracle_mod):  # tests.rs:33-62
    b = _brick(2)
    assert not any(oracle_mod.brick_empty_throughout(2, b, 2, o, PAL_C, PAL_D) for o in range(8))
    x, y, z = OCTANT_OFFSET[5]
    b[oracle_mod.flat_projection(x, y, z, 2)] = EMPTY_MARK
    assert oracle_mod.brick_empty_throughout(2, b, 2, 5, PAL_C, PAL_D)


def test_brick_octant_empty_where_dim_is_4(oracle_mod):  # tests.rs:64-118
    b = _brick(4)
    assert not any(oracle_mod.brick_empty_throughout(2, b, 4, o, PAL_C, PAL_D) for o in range(8))
    ox, oy, oz = (2 * v for v in OCTANT_OFFSET[5])
    b[oracle_mod.flat_projection(ox, oy, oz, 4)] = EMPTY_MARK  # part of the octant: not yet empty
    assert not oracle_mod.brick_empty_throughout(2, b, 4, 5, PAL_C, PAL_D)
    for x in range(2):
        for y in range(2):
            for z in range(2):
                b[oracle_mod.flat_projection(ox + x, oy + y, oz + z, 4)] = EMPTY_MARK
    assert oracle_mod.brick_empty_throughout(2, b, 4, 5, PAL_C, PAL_D)


def test_brick_part_of_octant_empty(oracle_mod):  # tests.rs:120-158
    b = _brick(4)
    assert not any(oracle_mod.brick_empty_throughout(2, b, 4, i, PAL_C, PAL_D, part=j)
                   for i in range(8) for j in range(8))
    ox, oy, oz = (2 * v for v in OCTANT_OFFSET[5])
    b[oracle_mod.flat_projection(ox, oy, oz, 4)] = EMPTY_MARK
    assert oracle_mod.brick_empty_throughout(2, b, 4, 5, PAL_C, PAL_D, part=0)
    assert not oracle_mod.brick_empty_throughout(2, b, 4, 5, PAL_C, PAL_D, part=1)
