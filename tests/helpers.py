"""Shared test helpers: the reference tests' scenes as operation lists.

Each builder restates a tree that a reference test builds with
`Octree::insert` loops, as an array of construction ops (layout OP_DTYPE:
x, y, z, op, kind, size, rgba, user).  The same array feeds the oracle and
the GB300 product library, so both see identical construction calls.
"""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

OP_DTYPE = np.dtype([("x", "<u2"), ("y", "<u2"), ("z", "<u2"), ("op", "u1"), ("kind", "u1"),
                     ("size", "<u4"), ("rgba", "<u4"), ("user", "<u4")])
INSERT, UPDATE, INSERT_AT_LOD, CLEAR, CLEAR_AT_LOD = range(5)
ALBEDO, DATA, COMPLEX = 1, 2, 3


def rgba(r, g, b, a):
    """Albedo packed as Albedo::from(u32) reads it: 0xRRGGBBAA."""
    return ((int(r) & 0xFF) << 24) | ((int(g) & 0xFF) << 16) | ((int(b) & 0xFF) << 8) | (int(a) & 0xFF)


def ops_from(records):
    """records: iterable of (op, x, y, z, kind, rgba, user[, size])."""
    recs = list(records)
    a = np.zeros(len(recs), dtype=OP_DTYPE)
    for i, r in enumerate(recs):
        op, x, y, z, kind, col, user = r[:7]
        size = r[7] if len(r) > 7 else 1
        a[i] = (x, y, z, op, kind, size, col & 0xFFFFFFFF, user & 0xFFFFFFFF)
    return a


def grid_ops(size, mask, colors=None, user=None):
    """Inserts at every (x, y, z) with mask[x, y, z] true, in the reference's x->y->z loop order."""
    xs, ys, zs = np.nonzero(mask)  # C order of the (x, y, z) array == nested x, y, z loops
    a = np.zeros(len(xs), dtype=OP_DTYPE)
    a["x"], a["y"], a["z"] = xs, ys, zs
    a["op"] = INSERT
    a["size"] = 1
    kind = 0
    if colors is not None:
        a["rgba"] = colors[xs, ys, zs]
        kind |= ALBEDO
    if user is not None:
        a["user"] = user if np.isscalar(user) else user[xs, ys, zs]
        kind |= DATA
    a["kind"] = kind
    return a


def f32_color(num, den):
    """`(255 as f32 * num as f32 / den as f32) as u8` evaluated in f32."""
    v = (np.float32(255.0) * np.asarray(num, dtype=np.float32)) / np.float32(den)
    return np.floor(v).astype(np.uint8)


def known_rays():
    with open(os.path.join(GOLDEN, "known_rays.json")) as f:
        return json.load(f)


def ray_of(test, rel="src/raytracing/tests.rs", index=0):
    r = known_rays()[rel + "::" + test][index]
    return (np.array([np.float32(v) for v in r["origin"]], dtype=np.float32),
            np.array([np.float32(v) for v in r["direction"]], dtype=np.float32))


def normalized(v):
    """V3c::<f32>::normalized: v / sqrt((x*x + y*y) + z*z), every step in f32."""
    v = np.asarray(v, dtype=np.float32)
    l = np.sqrt(np.float32(v[0] * v[0]) + np.float32(v[1] * v[1]) + np.float32(v[2] * v[2]), dtype=np.float32)
    return (v / l).astype(np.float32)


# ---------------- scenes of src/raytracing/tests.rs ----------------

def scene_stairs(loop_stuck_variant=False):
    """tests.rs:255-279 (unreachable / zero_advance) and :489-513 (loop_stuck)."""
    rec = [(INSERT, 3, 0, 0, ALBEDO, 0, 0), (INSERT, 3, 3, 0, ALBEDO, 1, 0), (INSERT, 0, 3, 0, ALBEDO, 2, 0)]
    for y in range(4):
        if loop_stuck_variant:
            rec += [(INSERT, 0, y, y, ALBEDO, 3, 0), (INSERT, 1, y, y, ALBEDO, 4, 0),
                    (INSERT, 2, y, y, DATA, 0, 5), (INSERT, 3, y, y, ALBEDO, 6, 0)]
        else:
            rec += [(INSERT, x, y, y, ALBEDO, 3, 0) for x in range(4)]
    return 4, 1, ops_from(rec)


def scene_floor(size=4, dim=1):
    """tests.rs:408-414 / 435-441 / 463-469 / 534-540: user data 5 on the y == 0 plane (x, z < 4)."""
    return size, dim, ops_from([(INSERT, x, 0, z, DATA, 0, 5) for x in range(4) for z in range(4)])


def scene_brick_boundary():
    """tests.rs:689-713 (TREE_SIZE 128, BRICK_DIMENSION 8)."""
    S = 128
    x, y, z = np.meshgrid(np.arange(S), np.arange(S), np.arange(S), indexing="ij")
    m = (((x < S // 4) | (y < S // 4) | (z < S // 4)) & ((x % 2 == 0) & (y % 4 == 0) & (z % 2 == 0))) | \
        ((S // 2 <= x) & (S // 2 <= y) & (S // 2 <= z))
    r, g, b = f32_color(x % 6, 6), f32_color(y % 6, 6), f32_color(z % 6, 6)
    col = (r.astype(np.uint32) << 24) | (g.astype(np.uint32) << 16) | (b.astype(np.uint32) << 8) | 255
    return S, 8, grid_ops(S, m, colors=col)


def scene_dot_cube(S, dim, corner_cube=True, lattice=True):
    """The "dot cube" fill of tests.rs:737-797 and examples/cpu_render.rs:23-43 (colour = 255*c/S)."""
    x, y, z = np.meshgrid(np.arange(S), np.arange(S), np.arange(S), indexing="ij")
    m = np.zeros((S, S, S), dtype=bool)
    if lattice:
        m |= ((x < S // 4) | (y < S // 4) | (z < S // 4)) & ((x % 2 == 0) & (y % 4 == 0) & (z % 2 == 0))
    if corner_cube:
        m |= (S // 2 <= x) & (S // 2 <= y) & (S // 2 <= z)
    r, g, b = f32_color(x, S), f32_color(y, S), f32_color(z, S)
    col = (r.astype(np.uint32) << 24) | (g.astype(np.uint32) << 16) | (b.astype(np.uint32) << 8) | 255
    return S, dim, grid_ops(S, m, colors=col)
