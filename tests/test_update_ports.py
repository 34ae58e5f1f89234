"""Ports of the reference's construction/update tests (src/octree/update/tests.rs).

Every test runs twice: against the oracle and against the GB300 product
library's host-side octree (libsvo, which needs no GPU for construction).
`get` results are (kind, rgba, user) with kind 0 Empty, 1 Visual,
2 Informative, 3 Complex.
"""
import pytest

from backends import make_tree

RED, GREEN, BLUE = 0xFF0000FF, 0x00FF00FF, 0x0000FFFF
OFFS = [(0, 0, 0), (1, 0, 0), (0, 0, 1), (1, 0, 1), (0, 1, 0), (1, 1, 0), (0, 1, 1), (1, 1, 1)]
E = (0, 0, 0)


def V(c):
    return (1, c, 0)


def I(u):
    return (2, 0, u)


def C(c, u):
    return (3, c, u)


@pytest.fixture(params=["oracle", "product"])
def backend(request):
    return request.param


def tree(backend, size, dim, simplify=True):
    t = make_tree(backend, size, dim)
    if not simplify:
        t.set_auto_simplify(False)
    return t


def test_simplest_insert_and_get(backend):  # tests.rs:8-17
    t = tree(backend, 2, 1, False)
    assert t.insert((0, 0, 0), albedo=0xFF000001) == 0
    assert t.get((0, 0, 0)) == V(0xFF000001)


def test_simple_insert_and_get(backend):  # tests.rs:19-46
    t = tree(backend, 2, 1, False)
    t.insert((1, 0, 0), albedo=RED)
    t.insert((0, 1, 0), albedo=GREEN)
    t.insert((0, 0, 1), albedo=BLUE)
    assert [t.get(p) for p in [(1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 1)]] == [V(RED), V(GREEN), V(BLUE), E]
    t.insert((1, 0, 0), albedo=GREEN)
    assert [t.get(p) for p in [(1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 1)]] == [V(GREEN), V(GREEN), V(BLUE), E]


def test_insert_empty(backend):  # tests.rs:48-54
    t = tree(backend, 2, 1, False)
    t.insert((0, 0, 0))
    assert t.get((0, 0, 0)) == E


def test_complex_insert_and_get(backend):  # tests.rs:56-110
    t = tree(backend, 2, 1, False)
    t.insert((1, 0, 0), albedo=RED, user=3)
    t.insert((0, 1, 0), albedo=GREEN, user=1)
    t.insert((0, 0, 1), user=2)
    assert [t.get(p) for p in [(1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 1)]] == [C(RED, 3), C(GREEN, 1), I(2), E]
    t.insert((1, 0, 0), user=3)
    assert [t.get(p) for p in [(1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 1)]] == [I(3), C(GREEN, 1), I(2), E]


def test_simple_insert_and_get_where_dim_is_2(backend):  # tests.rs:112-140
    t = tree(backend, 4, 2, False)
    for p, c in [((1, 0, 0), RED), ((0, 1, 0), GREEN), ((0, 0, 1), BLUE), ((3, 0, 0), RED), ((0, 3, 0), GREEN),
                 ((0, 0, 3), BLUE)]:
        assert t.insert(p, albedo=c) == 0
        assert t.get(p) == V(c)
    t.insert((1, 0, 0), albedo=GREEN)
    assert [t.get(p) for p in [(1, 0, 0), (0, 1, 0), (0, 0, 1)]] == [V(GREEN), V(GREEN), V(BLUE)]


@pytest.mark.parametrize("dim", [1, 2])
def test_insert_at_lod(backend, dim):  # tests.rs:142-242
    t = tree(backend, 8, dim, False)
    t.insert_at_lod((0, 0, 0), 2, albedo=RED)
    for x in range(2):
        for y in range(2):
            for z in range(2):
                assert t.get((x, y, z)) == V(RED)
    t.insert_at_lod((0, 0, 0), 4, albedo=GREEN)
    hits = [t.get((x, y, z)) for x in range(4) for y in range(4) for z in range(4)]
    assert all(h in (E, V(GREEN)) for h in hits) and sum(h != E for h in hits) == 64


@pytest.mark.parametrize("dim", [1, 2, 4])
def test_simplified_insert_separated_by_clear(backend, dim):  # tests.rs:244-358
    t = tree(backend, 8, dim)
    for x in range(8):
        for y in range(8):
            for z in range(8):
                assert t.insert((x, y, z), albedo=RED) == 0
    assert t.get((3, 3, 3)) == V(RED)
    assert t.clear((3, 3, 3)) == 0
    assert t.get((3, 3, 3)) == E
    hits = [t.get((x, y, z)) for x in range(8) for y in range(8) for z in range(8)]
    assert all(h in (E, V(RED)) for h in hits) and sum(h != E for h in hits) == 511


def test_update_color_data_empty(backend):  # tests.rs:360-401
    t = tree(backend, 2, 1, False)
    t.insert((0, 0, 0), albedo=RED, user=3)
    assert t.get((0, 0, 0)) == C(RED, 3)
    t.update((0, 0, 0), albedo=GREEN)
    assert t.get((0, 0, 0)) == C(GREEN, 3)
    t = tree(backend, 2, 1, False)
    t.insert((0, 0, 0), albedo=RED, user=3)
    t.update((0, 0, 0), user=4)
    assert t.get((0, 0, 0)) == C(RED, 4)
    t = tree(backend, 2, 1, False)
    t.insert((0, 0, 0), albedo=RED, user=3)
    t.update((0, 0, 0))
    assert t.get((0, 0, 0)) == C(RED, 3)


@pytest.mark.parametrize("mode", ["clear", "insert"])
def test_uniform_solid_leaf_separated_where_dim_is_1(backend, mode):  # tests.rs:403-460
    t = tree(backend, 2, 1)
    base = 0xFFFF00FF
    for o in OFFS:
        t.insert(o, albedo=base)
    assert t.get((0, 0, 0)) == V(base)
    if mode == "clear":
        t.clear((0, 0, 0))
        assert t.get((0, 0, 0)) == E
    else:
        t.insert((0, 0, 0), albedo=base)
        assert t.get((0, 0, 0)) == V(base)
    for o in OFFS[1:]:
        assert t.get(o) == V(base)


@pytest.mark.parametrize("mode", ["clear", "insert"])
def test_uniform_solid_leaf_separated_where_dim_is_4(backend, mode):  # tests.rs:462-567
    t = tree(backend, 8, 4)
    base = 0xFFFF00AA
    for oi, o in enumerate(OFFS):
        for x in range(2):
            for y in range(2):
                for z in range(2):
                    t.insert((o[0] * 2 + x, o[1] * 2 + y, o[2] * 2 + z), albedo=base + oi)
    assert t.get((0, 0, 0)) == V(base)
    if mode == "clear":
        t.clear((0, 0, 0))
        assert t.get((0, 0, 0)) == E
    else:
        t.insert((0, 0, 0), albedo=0x000000FF)
        assert t.get((0, 0, 0)) == V(0x000000FF)
    for oi, o in enumerate(OFFS):
        for x in range(2):
            for y in range(2):
                for z in range(2):
                    if (x, y, z, oi) == (0, 0, 0, 0):
                        continue
                    assert t.get((o[0] * 2 + x, o[1] * 2 + y, o[2] * 2 + z)) == V(base + oi)


def test_uniform_parted_brick_leaf_separated_by_clear_where_dim_is_4(backend):  # tests.rs:569-640
    t = tree(backend, 8, 4)

    def col(x, y, z):
        return ((x - x % 2) << 24) | ((y - y % 2) << 16) | ((z - z % 2) << 8) | 0xFF

    for o in OFFS:
        for x in range(4):
            for y in range(4):
                for z in range(4):
                    p = (o[0] * 4 + x, o[1] * 4 + y, o[2] * 4 + z)
                    t.insert(p, albedo=col(x, y, z))
                    assert t.get(p) == V(col(x, y, z))
    assert t.get((0, 0, 0)) == V(0x000000FF)
    t.clear((1, 1, 1))
    assert t.get((1, 1, 1)) == E
    for oi, o in enumerate(OFFS):
        for x in range(4):
            for y in range(4):
                for z in range(4):
                    p = (o[0] * 4 + x, o[1] * 4 + y, o[2] * 4 + z)
                    assert t.get(p) == (E if (x, y, z, oi) == (1, 1, 1, 0) else V(col(x, y, z)))


def test_simple_uniform_parted_brick_leaf_separated_by_insert(backend):  # tests.rs:642-692
    t = tree(backend, 4, 2)
    base = 0xF00000FF
    for oi, o in enumerate(OFFS):
        t.insert_at_lod((o[0] * 2, o[1] * 2, o[2] * 2), 2, albedo=base + 2 * oi)
    assert t.get((0, 0, 0)) == V(base)
    t.insert((0, 0, 0), albedo=0x000000FF)
    assert t.get((0, 0, 0)) == V(0x000000FF)
    for x in range(2):
        for y in range(2):
            for z in range(2):
                for oi, o in enumerate(OFFS):
                    p = (o[0] * 2 + x, o[1] * 2 + y, o[2] * 2 + z)
                    assert t.get(p) == (V(0x000000FF) if (x, y, z, oi) == (0, 0, 0, 0) else V(base + 2 * oi))


def test_insert_at_lod_with_simplify(backend):  # tests.rs:911-965
    t = tree(backend, 8, 1)
    t.insert_at_lod((4, 0, 0), 2, albedo=RED)
    for x in (4, 5):
        for y in (0, 1):
            for z in (0, 1):
                assert t.get((x, y, z)) == V(RED)
    t.insert_at_lod((0, 0, 0), 4, albedo=GREEN)
    hits = 0
    for x in range(4):
        for y in range(4):
            for z in range(4):
                h = t.get((x, y, z))
                if h != E:
                    assert h == V(GREEN)
                    hits += 1
    for x in (4, 5):
        for y in (0, 1):
            for z in (0, 1):
                h = t.get((x, y, z))
                if h != E:
                    assert h == V(RED)
                    hits += 1
    assert hits == 64 + 8


@pytest.mark.parametrize("size,dim", [(2, 1), (4, 2)])
def test_simplifyable_insert_and_clear(backend, size, dim):  # tests.rs:967-1027, 1138-1196
    t = tree(backend, size, dim)
    for x in range(size):
        for y in range(size):
            for z in range(size):
                t.insert((x, y, z), albedo=RED)
    t.insert((0, 0, 0), albedo=GREEN)
    assert t.get((0, 0, 0)) == V(GREEN)
    for x in range(1, size):
        for y in range(1, size):
            for z in range(1, size):
                assert t.get((x, y, z)) == V(RED)
    t2 = tree(backend, size, dim)
    for x in range(size):
        for y in range(size):
            for z in range(size):
                t2.insert((x, y, z), albedo=0xFFAAEEFF)
    t2.clear((0, 0, 0))
    assert t2.get((0, 0, 0)) == E
    for x in range(1, size):
        for y in range(1, size):
            for z in range(1, size):
                assert t2.get((x, y, z)) == V(0xFFAAEEFF)


@pytest.mark.parametrize("size,dim", [(2, 1), (4, 2)])
def test_simple_clear(backend, size, dim):  # tests.rs:1029-1069
    t = tree(backend, size, dim, False)
    t.insert((1, 0, 0), albedo=RED)
    t.insert((0, 1, 0), albedo=GREEN)
    t.insert((0, 0, 1), albedo=BLUE)
    t.clear((0, 0, 1))
    assert [t.get(p) for p in [(1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 1)]] == [V(RED), V(GREEN), E, E]


def test_ocbits_resolution_cases(backend):  # tests.rs:1071-1118
    t = tree(backend, 64, 8)
    t.insert((0, 1, 1), albedo=RED)
    t.insert((1, 0, 0), albedo=RED)
    assert t.get((0, 1, 1)) == V(RED) and t.get((1, 0, 0)) == V(RED)
    t.clear((1, 0, 0))
    assert t.get((1, 0, 0)) == E
    t = tree(backend, 64, 8)
    t.insert_at_lod((33, 33, 33), 2, albedo=RED)
    assert t.get((33, 33, 33)) == V(RED)
    t.clear((33, 33, 33))
    assert t.get((33, 33, 33)) == E
    t = tree(backend, 64, 8)
    t.insert((31, 31, 31), albedo=RED)
    assert t.get((31, 31, 31)) == V(RED)
    t.clear((31, 31, 31))
    assert t.get((31, 31, 31)) == E


def test_double_clear(backend):  # tests.rs:1120-1136
    t = tree(backend, 2, 1, False)
    t.insert((1, 0, 0), albedo=0x000000FF)
    t.insert((0, 1, 0), albedo=0xFFFFFFFF)
    t.insert((0, 0, 1), albedo=0xFFFFFFFF)
    t.clear((0, 0, 1))
    t.clear((0, 0, 1))
    assert t.get((1, 0, 0)) == V(0x000000FF) and t.get((0, 1, 0)) == V(0xFFFFFFFF) and t.get((0, 0, 1)) == E


def test_clear_to_nothing(backend):  # tests.rs:1198-1226
    t = tree(backend, 4, 1)
    for o in OFFS:
        t.insert(o, albedo=0xFFAAEEFF)
    t.clear_at_lod((0, 0, 0), 2)
    for o in OFFS:
        assert t.get(o) == E


def test_invalid_arguments(backend):  # octree/mod.rs:173-186 and insert.rs:106-114
    from backends import creation_error
    assert creation_error(backend, 0, 1) == 2      # InvalidBrickDimension (size 0)
    assert creation_error(backend, 8, 3) == 2      # InvalidBrickDimension
    assert creation_error(backend, 4, 8) == 1      # InvalidSize
    assert creation_error(backend, 12, 4) == 1     # InvalidSize
    assert creation_error(backend, 4, 4) == 3      # InvalidStructure
    t = tree(backend, 4, 1)
    assert t.insert((4, 0, 0), albedo=RED) == 4   # InvalidPosition
    assert t.clear((0, 9, 0)) == 4


# ---- the remaining cases of tests.rs: uniform parted leaves split by an insert, LOD inserts and clears at
# unaligned positions and sizes, whole-node clears and overwrites, and two edge cases

def cube(n, lo=0):
    return [(x, y, z) for x in range(lo, n) for y in range(lo, n) for z in range(lo, n)]


def hits_of(t, positions, value):
    """Count of non-empty entries at `positions`, each of which must equal `value`."""
    got = [t.get(p) for p in positions]
    assert all(g in (E, value) for g in got), [(p, g) for p, g in zip(positions, got) if g not in (E, value)][:4]
    return sum(g != E for g in got)


def test_uniform_parted_brick_leaf_separated_by_insert_where_dim_is_4(backend):  # tests.rs:694-771
    D = 4
    t = tree(backend, 8, D)

    def color(x, y, z):  # the brick's 2x2x2 cells share a colour: the leaf is downsampled losslessly
        return ((x - x % (D // 2)) << 24) | ((y - y % (D // 2)) << 16) | ((z - z % (D // 2)) << 8) | 0xFF

    for o in OFFS:
        for x, y, z in cube(D):
            p = (o[0] * D + x, o[1] * D + y, o[2] * D + z)
            t.insert(p, albedo=color(x, y, z))
            assert t.get(p) == V(color(x, y, z)), p
    assert t.get((0, 0, 0)) == V(0x000000FF)
    t.insert((1, 1, 1), albedo=0xFF0000FF)  # splits the uniform leaf
    assert t.get((1, 1, 1)) == V(0xFF0000FF) and t.get((0, 0, 0)) == V(0x000000FF)
    for o in OFFS:
        for x, y, z in cube(D):
            p = (o[0] * D + x, o[1] * D + y, o[2] * D + z)
            want = V(0xFF0000FF) if p == (1, 1, 1) else V(color(x, y, z))
            assert t.get(p) == want, p


@pytest.mark.parametrize("size,dim,pos,lod,region,want", [
    (8, 4, (1, 1, 1), 4, 4, 27),  # tests.rs:773-811: one brick is updated, from 1,1,1 to 3,3,3
    (8, 1, (2, 2, 2), 3, 8, 8),   # tests.rs:813-843: the size rounds down to 2
    (8, 1, (3, 3, 3), 3, 8, 1),   # tests.rs:845-876: a brick corner, one voxel
    (8, 4, (1, 1, 1), 3, 8, 27),  # tests.rs:878-910
])
def test_insert_at_lod_unaligned(backend, size, dim, pos, lod, region, want):
    t = tree(backend, size, dim, False)
    t.insert_at_lod(pos, lod, albedo=RED)
    assert t.get(pos) == V(RED)
    assert hits_of(t, cube(region), V(RED)) == want


def test_clear_edge_case(backend):  # tests.rs:1227-1278
    red = 0xFF0000FF
    t = tree(backend, 64, 16)
    t.update((1, 0, 0), user=0xFACEFEED)
    t.insert_at_lod((0, 0, 0), 32, albedo=red)
    t.clear_at_lod((5, 5, 5), 8)
    assert all(t.get(p) == E for p in cube(8, 5))
    assert all(t.get(p) == V(red) for p in cube(5))
    t.clear_at_lod((0, 0, 0), 32)
    assert all(t.get(p) == E for p in cube(32))


@pytest.mark.parametrize("dim,pos,lod,want", [
    (1, (0, 0, 0), 2, 64 - 8),  # tests.rs:1280-1313
    (2, (0, 0, 0), 2, 64 - 8),  # tests.rs:1316-1349
    (1, (0, 0, 0), 3, 64 - 8),  # tests.rs:1465-1495: the size rounds down to 2
])
def test_clear_at_lod_in_a_size_4_block(backend, dim, pos, lod, want):
    t = tree(backend, 8, dim)
    t.insert_at_lod((0, 0, 0), 4, albedo=0xFFAAEEFF)
    t.clear_at_lod(pos, lod)
    assert hits_of(t, cube(4), V(0xFFAAEEFF)) == want


def test_clear_at_lod_with_unaligned_position(backend):  # tests.rs:1352-1405
    t = tree(backend, 8, 1)
    t.insert_at_lod((0, 0, 0), 4, albedo=0xFFAAEEFF)
    t.clear_at_lod((1, 1, 1), 2)  # clears the aligned 2-cube that holds 1,1,1
    assert all(t.get(p) == E for p in cube(2))
    for p in [(0, 0, 2), (0, 2, 0), (0, 2, 2), (2, 0, 0), (2, 0, 2), (2, 2, 0), (2, 2, 2)]:
        assert t.get(p) != E, p
    assert hits_of(t, cube(4), V(0xFFAAEEFF)) == 64 - 8


def test_clear_at_lod_with_unaligned_position_where_dim_is_4(backend):  # tests.rs:1407-1463
    t = tree(backend, 16, 4)
    t.insert_at_lod((0, 0, 0), 8, albedo=0xFFAAEEFF)
    assert all(t.get(p) == V(0xFFAAEEFF) for p in cube(8))
    t.clear_at_lod((1, 1, 1), 4)  # one brick is updated: 1,1,1 to 3,3,3
    assert hits_of(t, cube(8), V(0xFFAAEEFF)) == 512 - 27


@pytest.mark.parametrize("size,set_lod,clear_lod,want_before,want_after", [
    (8, 4, 3, 64, 64 - 27),      # tests.rs:1498-1547
    (16, 8, 5, 512, 512 - 64),   # tests.rs:1549-1598: clears whole nodes
])
def test_clear_at_lod_where_dim_is_4(backend, size, set_lod, clear_lod, want_before, want_after):
    t = tree(backend, size, 4)
    t.insert_at_lod((0, 0, 0), set_lod, albedo=0xFFAAEEFF)
    assert hits_of(t, cube(8), V(0xFFAAEEFF)) == want_before
    t.clear_at_lod((0, 0, 0), clear_lod)
    assert hits_of(t, cube(8), V(0xFFAAEEFF)) == want_after


def test_overwrite_whole_nodes_where_dim_is_4(backend):  # tests.rs:1600-1655
    t = tree(backend, 16, 4)
    t.insert_at_lod((0, 0, 0), 8, albedo=RED)
    assert hits_of(t, cube(8), V(RED)) == 512
    t.insert_at_lod((0, 0, 0), 5, albedo=BLUE)
    got = [t.get(p) for p in cube(8)]
    assert E not in got
    assert sum(g == V(RED) for g in got) == 512 - 64 and sum(g == V(BLUE) for g in got) == 64


def test_edge_case_octree_set(backend):  # tests.rs:1657-1673
    t = tree(backend, 8, 1)
    for x, y, z in cube(8, 6):
        t.insert((x, y, z), albedo=x + y + z)
        assert t.get((x, y, z)) == V(x + y + z)


def test_case_inserting_empty(backend):  # tests.rs:1675-1687
    t = tree(backend, 4, 1)
    t.insert((3, 0, 0), albedo=0)
    assert t.get((3, 0, 0)) == E
