"""The product library's host octree builds exactly the oracle's structure.

Node keys, node content, children, occupancy bitmaps, brick contents and
palettes are compared record by record (the canonical 40-word record of
svo_node_record / orc_node_record).  A freed node's content is never read by
the reference (every access is behind key_is_valid), so content is compared
for reserved nodes only; children entries are compared for every key.
"""
import numpy as np
import pytest

import shocovox_gb300 as svo
from helpers import OP_DTYPE, scene_brick_boundary, scene_dot_cube, scene_floor, scene_stairs

CONTENT_FIELDS = [1, 2] + list(range(13, 37))


def canon(rec):
    rec = list(rec)
    if not rec[0]:
        for i in CONTENT_FIELDS:
            rec[i] = 0
    return tuple(rec)


def compare(oracle_tree, product_tree):
    a = [canon(r) for r in oracle_tree.records()]
    b = [canon(r) for r in product_tree.records()]
    assert len(a) == len(b), "node pool lengths differ: oracle %d, product %d" % (len(a), len(b))
    for k, (ra, rb) in enumerate(zip(a, b)):
        assert ra == rb, "node %d differs:\n oracle  %s\n product %s" % (k, ra, rb)
    for which in (0, 1):
        assert np.array_equal(oracle_tree.palette(which), product_tree.palette(which))


def build_both(oracle_mod, size, dim, ops, auto_simplify=True):
    o = oracle_mod.Tree(size, dim)
    p = svo.Octree(size, dim)
    if not auto_simplify:
        o.set_auto_simplify(False)
        p.set_auto_simplify(False)
    o.apply_ops(ops)
    p.apply_ops(ops)
    return o, p


@pytest.mark.parametrize("scene", ["stairs", "stairs_loop", "floor", "floor84", "boundary", "flaps", "bleed"])
def test_reference_test_scenes(oracle_mod, scene):
    s = {"stairs": scene_stairs, "stairs_loop": lambda: scene_stairs(True), "floor": scene_floor,
         "floor84": lambda: scene_floor(8, 4), "boundary": scene_brick_boundary,
         "flaps": lambda: scene_dot_cube(32, 1, True, False), "bleed": lambda: scene_dot_cube(32, 1, False, True)}[scene]()
    o, p = build_both(oracle_mod, *s)
    compare(o, p)


@pytest.mark.parametrize("kind,size,dim", [(0, 32, 2), (0, 64, 4), (1, 64, 8), (2, 128, 4), (3, 32, 2), (3, 64, 8)])
def test_generated_scenes(oracle_mod, kind, size, dim):
    ops = svo.gen_scene(kind, size, dim, seed=1000 + size + dim, occupancy=0.15, spheres=4, octaves=2,
                        base_freq=1.0 / 16, height_lo=2.0, height_hi=size * 0.4, cave_threshold=0.55)
    assert len(ops) > 0
    o, p = build_both(oracle_mod, size, dim, ops)
    compare(o, p)


def random_ops(rng, size, n, lod_sizes=(2, 4, 8)):
    ops = np.zeros(n, dtype=OP_DTYPE)
    for i in range(n):
        r = rng.random()
        if r < 0.55:
            op, sz = 0, 1
        elif r < 0.65:
            op, sz = 1, 1
        elif r < 0.75:
            op, sz = 2, int(rng.choice(lod_sizes))
        elif r < 0.92:
            op, sz = 3, 1
        else:
            op, sz = 4, int(rng.choice(lod_sizes))
        kind = int(rng.integers(0, 4))
        col = int(rng.choice([0x000000FF, 0xFF0000FF, 0x00FF00FF, 0x11223300, 0]))
        user = int(rng.choice([0, 1, 7, 4096]))
        pos = rng.integers(0, size, size=3)
        if op in (2, 4):
            pos = (pos // sz) * sz if rng.random() < 0.7 else pos
        ops[i] = (pos[0], pos[1], pos[2], op, kind, sz, col, user)
    return ops


@pytest.mark.parametrize("seed", range(24))
@pytest.mark.parametrize("size,dim", [(8, 1), (8, 2), (16, 2), (16, 4), (32, 4), (32, 8)])
def test_random_update_sequences(oracle_mod, seed, size, dim):
    rng = np.random.default_rng(seed * 7919 + size * 31 + dim)
    ops = random_ops(rng, size, 300)
    o = oracle_mod.Tree(size, dim)
    p = svo.Octree(size, dim)
    if seed % 5 == 4:
        o.set_auto_simplify(False)
        p.set_auto_simplify(False)
    for chunk in range(0, len(ops), 50):
        part = ops[chunk:chunk + 50]
        eo = ep = None
        try:
            o.apply_ops(part)
        except oracle_mod.OracleError as e:
            eo = e.code
        try:
            p.apply_ops(part)
        except svo.OctreeError as e:
            ep = e.code
        assert eo == ep, "error status differs: oracle %s, product %s" % (eo, ep)
        if eo is not None:
            return  # the reference panicked: the tree is no longer meaningful
        compare(o, p)
        for pos in rng.integers(0, size, size=(20, 3)):
            assert o.get(tuple(int(v) for v in pos)) == p.get(tuple(int(v) for v in pos))


def test_insert_dense_equals_the_reference_fill_loops(oracle_mod):
    # svo_insert_dense: one Octree::insert per voxel in the nesting of the reference's fill loops
    # (x outermost, z innermost); empty entries insert nothing; a block past the octree stops with
    # InvalidPosition after the inserts that fit
    import shocovox_gb300 as svo
    from helpers import ALBEDO, COMPLEX, DATA, INSERT, ops_from
    rng = np.random.default_rng(41)
    for size, dim, origin, shape, which in ((32, 2, (3, 5, 1), (7, 9, 6), "rgba"), (64, 4, (10, 0, 20), (12, 5, 17), "both"),
                                            (16, 1, (0, 0, 0), (16, 16, 16), "user")):
        d, h, w = shape
        rgba = rng.choice([0, 0x10203000, 0xFF0000FF, 0x00FF00FF, 0x336699FF], size=shape).astype(np.uint32)
        user = rng.choice([0, 1, 7, 4096], size=shape).astype(np.uint32)
        a = rgba if which in ("rgba", "both") else None
        u = user if which in ("user", "both") else None
        kind = {"rgba": ALBEDO, "user": DATA, "both": COMPLEX}[which]
        recs = []
        for i in range(w):
            for j in range(h):
                for k in range(d):
                    recs.append((INSERT, origin[0] + i, origin[1] + j, origin[2] + k, kind,
                                 int(rgba[k, j, i]) if a is not None else 0, int(user[k, j, i]) if u is not None else 0))
        o = oracle_mod.Tree(size, dim)
        o.apply_ops(ops_from(recs))
        p = svo.Octree(size, dim)
        assert p.insert_dense(origin, rgba=a, user=u) == w * h * d
        assert [list(r) for r in p.records()] == [list(r) for r in o.records()], (size, dim, which)
        assert list(p.palette(0)) == list(o.palette(0)) and list(p.palette(1)) == list(o.palette(1))
    p = svo.Octree(16, 2)
    with pytest.raises(svo.OctreeError) as e:
        p.insert_dense((10, 10, 10), rgba=np.full((8, 8, 8), 0xFF0000FF, np.uint32))
    assert e.value.code == 4 and "after 6 inserts" in str(e.value)  # z = 16 is the first voxel outside
