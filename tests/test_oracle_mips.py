"""MIP maps in the oracle, pinned by the reference's own known-answer tests
(src/octree/tests.rs:155-560, mod mipmap_tests), plus the LOD cast's use of them."""
import numpy as np

RED, GREEN, BLUE = 0xFF0000FF, 0x00FF00FF, 0x0000FFFF
# gamma-corrected mixes, mip = ((a^2 + b^2 ...) / n).sqrt() (tests.rs:164-171, 404-412)
RG = (int(np.sqrt(np.float32(255.0) ** 2 / np.float32(2.0))) << 16) | \
     (int(np.sqrt(np.float32(255.0) ** 2 / np.float32(2.0))) << 24) | 0xFF
C3 = int(np.sqrt(np.float32(255.0) ** 2 / np.float32(3.0)))
RGB = (C3 << 8) | (C3 << 16) | (C3 << 24) | 0xFF
OOB = 8
MIXED6 = [((0, 0, 0), RED), ((0, 0, 1), GREEN), ((0, 1, 0), RED), ((0, 1, 1), GREEN), ((1, 0, 0), RED),
          ((1, 0, 1), GREEN)]
SECOND6 = [((8, 0, 0), RED), ((8, 0, 1), GREEN), ((8, 1, 0), BLUE), ((8, 1, 1), GREEN), ((9, 1, 0), RED),
           ((9, 0, 1), BLUE)]


def tree_with(O, size, dim, voxels, methods=(1,), mips_first=True):
    t = O.Tree(size, dim)
    t.set_auto_simplify(False)
    if mips_first:
        t.mip_switch(True)
        for level in methods:
            t.mip_set_method(level, O.Tree.BOX)
    for p, c in voxels:
        t.insert(p, albedo=c)
    return t


def albedo_of(sample):
    kind, rgba, _ = sample
    return rgba if kind & 1 else None


def test_mixed_mip_lvl1(oracle_mod):  # tests.rs:161-204
    t = tree_with(oracle_mod, 2, 1, MIXED6)
    assert albedo_of(t.mip_sample_root(OOB, (0, 0, 0))) == RG
    assert RG == 0xB4B400FF


def test_simple_solid_mip_lvl2_where_dim_is_2(oracle_mod):  # tests.rs:206-276
    t = tree_with(oracle_mod, 4, 2, [(p, RED) for p, _ in MIXED6])
    assert albedo_of(t.mip_sample_root(OOB, (0, 0, 0))) == RED
    for p in [(0, 0, 1), (0, 1, 0), (0, 1, 1), (1, 0, 0), (1, 0, 1), (1, 1, 0), (1, 1, 1)]:
        assert albedo_of(t.mip_sample_root(OOB, p)) is None


def test_mixed_mip_lvl2_where_dim_is_2(oracle_mod):  # tests.rs:278-356
    t = tree_with(oracle_mod, 4, 2, MIXED6)
    assert albedo_of(t.mip_sample_root(OOB, (0, 0, 0))) == RG
    for p in [(0, 0, 1), (0, 1, 0), (0, 1, 1), (1, 0, 0), (1, 0, 1), (1, 1, 0), (1, 1, 1)]:
        assert albedo_of(t.mip_sample_root(OOB, p)) is None


def check_dim4(t):
    sample = t.mip_sample_root if hasattr(t, "mip_sample_root") else t.sample_root_mip  # oracle / product
    assert albedo_of(sample(0, (0, 0, 0))) == RG
    assert albedo_of(sample(1, (0, 0, 0))) == RGB
    assert albedo_of(sample(OOB, (0, 0, 0))) == RG
    assert albedo_of(sample(OOB, (2, 0, 0))) == RGB


def test_mixed_mip_lvl2_where_dim_is_4(oracle_mod):  # tests.rs:358-470
    check_dim4(tree_with(oracle_mod, 16, 4, MIXED6 + SECOND6, methods=(1, 2)))


def test_mixed_mip_regeneration_lvl2_where_dim_is_4(oracle_mod):  # tests.rs:472-560
    O = oracle_mod
    t = tree_with(O, 16, 4, MIXED6 + SECOND6, mips_first=False)
    t.mip_switch(True)  # recalculates with the default strategy (PointFilter at level 1)
    t.mip_set_method(1, O.Tree.BOX)
    t.mip_set_method(2, O.Tree.BOX)
    t.mip_recalculate()
    check_dim4(t)


def test_regenerated_mips_equal_incremental_ones(oracle_mod):
    # the same scene with MIPs built while inserting and rebuilt afterwards
    O = oracle_mod
    a = tree_with(O, 16, 4, MIXED6 + SECOND6, methods=(1, 2))
    b = tree_with(O, 16, 4, MIXED6 + SECOND6, mips_first=False)
    b.mip_switch(True)
    b.mip_set_method(1, O.Tree.BOX)
    b.mip_set_method(2, O.Tree.BOX)
    b.mip_recalculate()
    for key in range(a.node_count()):
        ka, va = a.node_mip(key, 4)
        kb, vb = b.node_mip(key, 4)
        assert ka == kb
        if ka in (1, 2):
            for x, y in zip(va, vb):
                assert albedo_of(a_entry(a, x)) == albedo_of(a_entry(b, y))


def a_entry(t, pix):
    # resolve a PaletteIndexValues through the tree's colour palette (user data is never set here)
    pal = t.palette(0)
    c = pix & 0xFFFF
    return (1, int(pal[c]), 0) if c != 0xFFFF else (0, 0, 0)


def test_lod_cast_reads_mips(oracle_mod):
    # a far viewing distance keeps the voxels, a near one reads the root MIP once the ray has travelled
    O = oracle_mod
    t = tree_with(O, 16, 4, MIXED6 + SECOND6, methods=(1, 2))
    origin = np.array([[0.5, 0.5, -40.0]], np.float32)
    direction = np.array([[0.0, 0.0, 1.0]], np.float32)
    full = t.cast(origin, direction)
    assert full["status"][0] == 1 and full["brick_octant"][0] != 8
    near = t.cast(origin, direction, viewing_distance=1.0)
    assert near["status"][0] == 1 and near["brick_octant"][0] == 8 and near["albedo"][0] == RG


# ---- the product's host octree against the same known answers and the oracle's records ----
def product_tree(size, dim, voxels, methods=(1,), mips_first=True):
    import shocovox_gb300 as svo
    t = svo.Octree(size, dim)
    t.set_auto_simplify(False)
    if mips_first:
        t.switch_albedo_mip_maps(True)
        for level in methods:
            t.set_mip_method(level, svo.Octree.BOX_FILTER)
    for p, c in voxels:
        t.insert(p, albedo=c)
    return t


def test_product_mips_match_reference_known_answers():
    assert albedo_of(product_tree(2, 1, MIXED6).sample_root_mip(OOB, (0, 0, 0))) == RG
    assert albedo_of(product_tree(4, 2, MIXED6).sample_root_mip(OOB, (0, 0, 0))) == RG
    check_dim4(product_tree(16, 4, MIXED6 + SECOND6, methods=(1, 2)))
    import shocovox_gb300 as svo
    t = product_tree(16, 4, MIXED6 + SECOND6, mips_first=False)
    t.switch_albedo_mip_maps(True)
    t.set_mip_method(1, svo.Octree.BOX_FILTER).set_mip_method(2, svo.Octree.BOX_FILTER).recalculate_mips()
    check_dim4(t)


def test_product_mip_records_equal_the_oracle(oracle_mod):
    # random scenes with MIPs enabled before and after construction, every filter, inserts and clears
    import shocovox_gb300 as svo
    from helpers import ops_from, INSERT, CLEAR, INSERT_AT_LOD, ALBEDO
    rng = np.random.default_rng(11)
    for case in range(24):
        size, dim = [(16, 2), (32, 4), (64, 4), (32, 8)][case % 4]
        method = case % 5
        early = case % 2 == 0
        ops = []
        for _ in range(int(rng.integers(40, 200))):
            x, y, z = (int(v) for v in rng.integers(0, size, 3))
            r = rng.random()
            col = int(rng.choice([0xFF0000FF, 0x00FF00FF, 0x0000FFFF, 0x808080FF, 0x102030FF, 0xF0E0D0FF]))
            if r < 0.75:
                ops.append((INSERT, x, y, z, ALBEDO, col, 0, 1))
            elif r < 0.85:
                s = int(rng.choice([2, 4]))
                ops.append((INSERT_AT_LOD, x - x % s, y - y % s, z - z % s, ALBEDO, col, 0, s))
            else:
                ops.append((CLEAR, x, y, z, 0, 0, 0, 1))
        ops = ops_from(ops)
        o = oracle_mod.Tree(size, dim)
        p = svo.Octree(size, dim)
        if early:
            o.mip_switch(True)
            p.switch_albedo_mip_maps(True)
        for level in (1, 2, 3):
            o.mip_set_method(level, method, 0.3)
            p.set_mip_method(level, method, 0.3)
        # both stop at the same operation where the reference would panic (e.g. a MIP of a node
        # pushed where the reference does not grow node_mips)
        assert apply_status(o, ops) == apply_status(p, ops), "case %d" % case
        if not early:
            assert switch_status(o) == switch_status(p), "case %d" % case
        assert o.records() == p.records(), "case %d" % case
        assert list(o.palette(0)) == list(p.palette(0)), "case %d" % case


def apply_status(t, ops):
    import re
    try:
        t.apply_ops(ops)
        return (0, len(ops))
    except Exception as e:  # OracleError / OctreeError: status code and the operation it stopped at
        code = getattr(e, "code", None)
        at = int(re.search(r"op (\d+)", str(e)).group(1))
        return (code, at)


def switch_status(t):
    try:
        t.mip_switch(True) if hasattr(t, "mip_switch") else t.switch_albedo_mip_maps(True)
        return 0
    except Exception as e:
        return getattr(e, "code", -1)
