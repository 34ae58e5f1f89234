"""MagicaVoxel .vox import (Octree::load_vox_file, MIPMapStrategy::load_vox_file,
src/convert/magicavoxel.rs) against the oracle's restatement (oracle/vox.py), pinned by the
reference's own known answers: parse_rotation_matrix (magicavoxel.rs:387-414) and
convert_coordinate (src/spatial/math/tests.rs:197-234).

Scenes are written by tests/vox_writer.py; the reference's example models (assets/models/
navigate*.vox) are imported too where the SHOCOVOX_REFERENCE environment variable names a checkout
of the reference."""
import glob
import os

import numpy as np
import pytest

import shocovox_gb300 as svo
from shocovox_gb300._lib import SvoError
from oracle import vox as V
from vox_writer import VALID_ROTATIONS, group, random_scene, shape, transform, vox_file

_REF = os.environ.get("SHOCOVOX_REFERENCE", "")
ASSETS = sorted(glob.glob(os.path.join(_REF, "assets", "models", "*.vox"))) if _REF else []
PANIC, ARGUMENT = 5, 6


def records(t):
    return [list(r) for r in t.records()]


def outcome_oracle(oracle_mod, data, bd, configure=None):
    try:
        return V.build(oracle_mod, data, bd, configure)
    except V.VoxPanic:
        return "panic"
    except V.VoxFormatError:
        return "format"


def outcome_product(data, bd, configure=None):
    try:
        return svo.Octree.from_vox(data, bd, configure)
    except SvoError as e:
        return {PANIC: "panic", ARGUMENT: "format"}.get(e.code, e.code)
    except svo.OctreeError as e:  # Octree::new refused the size (MIPMapStrategy path)
        return "panic"


def assert_same_import(oracle_mod, data, bd, configure=None, pconfigure=None):
    o = outcome_oracle(oracle_mod, data, bd, configure)
    p = outcome_product(data, bd, pconfigure)
    if isinstance(o, str) or isinstance(p, str):
        assert o == p
        return None
    assert records(p) == records(o)
    assert list(p.palette(0)) == list(o.palette(0))
    assert p.size == V.plan(data)[0] == svo.Octree.vox_tree_size(data)
    return o, p


# ---- known answers --------------------------------------------------------------------------------
def test_rotation_matrix_known_answers():  # magicavoxel.rs:387-414
    ident = [[1, 0, 0], [0, 1, 0], [0, 0, 1]]
    example = [[0, 1, 0], [0, 0, -1], [-1, 0, 0]]
    byte = (1 << 0) | (2 << 2) | (0 << 4) | (1 << 5) | (1 << 6)
    for f in (V.rotation, svo.Octree.vox_rotation):
        assert f(4) == ident
        assert f(byte) == example


def test_every_rotation_byte_matches_the_oracle():
    valid = 0
    for b in range(256):
        try:
            want = V.rotation(b)
        except V.VoxPanic:
            with pytest.raises(SvoError):
                svo.Octree.vox_rotation(b)
            continue
        m = svo.Octree.vox_rotation(b)
        assert m == want
        valid += 1
        # a signed permutation: one +-1 per row and per column
        a = np.array(m)
        assert (np.abs(a).sum(0) == 1).all() and (np.abs(a).sum(1) == 1).all()
    assert valid == 2 * len(VALID_ROTATIONS)  # bit 7 is ignored


def test_coordinate_conversion_known_answers():  # src/spatial/math/tests.rs:197-234
    c = (1.0, 2.0, 3.0)
    assert V.convert_coordinate(c, "Rzup", "Rzup") == (1.0, 2.0, 3.0)
    assert V.convert_coordinate(c, "Lzup", "Ryup") == (1.0, 3.0, 2.0)
    assert V.convert_coordinate(c, "Rzup", "Ryup") == (1.0, 3.0, -2.0)
    assert V.convert_coordinate(c, "Lyup", "Ryup") == (1.0, 2.0, -3.0)
    # the pair the importer uses swaps y and z both ways
    assert V.convert_coordinate(c, "Rzup", "Lyup") == (1.0, 3.0, 2.0)
    assert V.convert_coordinate(c, "Lyup", "Rzup") == (1.0, 3.0, 2.0)


# ---- imports against the oracle -----------------------------------------------------------------------
@pytest.mark.skipif(not ASSETS, reason="the reference's example models are not present")
@pytest.mark.parametrize("path", ASSETS, ids=lambda p: os.path.basename(p))
def test_reference_example_models(oracle_mod, path):
    data = open(path, "rb").read()
    for bd in (2, 8):
        pair = assert_same_import(oracle_mod, data, bd)
        assert pair is not None
        o, p = pair
        _, voxels = V.plan(data)
        for x, y, z, c in voxels[::97]:
            assert p.get((x, y, z))[1] == c or (c & 0xFF) == 0
    # the file path entry point
    assert records(svo.Octree.load_vox(path, 8)) == records(svo.Octree.from_vox(data, 8))


@pytest.mark.parametrize("rotate", [False, True])
def test_random_scene_graphs(oracle_mod, rotate):
    # transforms with translations and rotations, nested groups, frames, models of another frame;
    # the reference's bounds arithmetic puts some voxels outside the octree (it panics there): both
    # sides must agree on which files those are
    outcomes = {"ok": 0, "panic": 0}
    for seed in range(24):
        rng = np.random.default_rng(1000 * rotate + seed)
        data = random_scene(rng, n_models=int(rng.integers(1, 7)), rotate=rotate)
        for bd in (1, 2, 4):
            pair = assert_same_import(oracle_mod, data, bd)
            outcomes["ok" if pair is not None else "panic"] += 1
    assert outcomes["ok"] >= 15


def test_mip_strategy_load(oracle_mod):
    # MIPMapStrategy::load_vox_file: the strategy is set on the empty octree, MIPs follow the inserts
    def oconf(t):
        t.mip_switch(True)
        t.mip_set_method(1, 0)
        t.mip_set_method(2, 3, 0.2)

    def pconf(t):
        t.switch_albedo_mip_maps(True)
        t.set_mip_method(1, svo.Octree.BOX_FILTER)
        t.set_mip_method(2, svo.Octree.POSTERIZE, 0.2)

    done = 0
    for seed in range(12):
        data = random_scene(np.random.default_rng(77 + seed), n_models=3, rotate=False)
        if assert_same_import(oracle_mod, data, 2, oconf, pconf) is not None:
            done += 1
    assert done >= 6


def test_frames_and_graph_quirks(oracle_mod):
    # kept from iterate_vox_tree: the root transform's own translation is not applied, a transform
    # without "_r" resets the orientation, models of frames other than 0 are skipped (the flipped
    # axis has an even size: with an odd one the reference's bounds put a voxel at -1)
    rng = np.random.default_rng(5)
    vox = np.array([[0, 0, 0, 1], [1, 0, 0, 2], [0, 2, 1, 3]], np.uint8)
    models = [((2, 4, 2), vox), ((4, 4, 4), np.array([[3, 3, 3, 4]], np.uint8))]
    nodes = [transform(0, 1, [{"_t": "500 x 500", "_r": "3"}]),  # never parsed
             group(1, [2, 4]),
             transform(2, 3, [{"_t": "4 0 0", "_r": "36"}]),  # 36: rows (0, 1, 2) with the y sign flipped
             shape(3, [(0, {}), (1, {"_f": "2"})]),
             transform(4, 5, [{"_t": "-4 1 1"}, {"_t": "9 9 9"}]),
             shape(5, [(0, {"_f": "0"})])]
    colors = [int(c) | 0xFF for c in rng.integers(1, 1 << 32, 256, dtype=np.uint64)]
    data = vox_file(models, nodes, colors)
    pair = assert_same_import(oracle_mod, data, 1)
    assert pair is not None
    size, voxels = V.plan(data)
    assert len(voxels) == 6 and size == 16


def test_malformed_and_panicking_files(oracle_mod):
    rng = np.random.default_rng(9)
    good = random_scene(rng, n_models=2, rotate=False)
    colors = [0xFF0000FF] * 256
    one = [((2, 2, 2), np.array([[0, 0, 0, 1]], np.uint8))]
    cases = {
        "format": [b"", b"VOX", b"VOX \xc8\x00\x00\x00", b"XXXX" + good[4:], good[:-7], good[:40],
                   vox_file(one, [transform(0, 1, [{}]), shape(1, [(0, {})])], None)],
        "panic": [vox_file(one, [shape(0, [(0, {})])], colors),                          # root not a transform
                  vox_file(one, [transform(0, 1, [{}]), transform(1, 2, [{"_t": "1 2"}]), shape(2, [(0, {})])], colors),
                  vox_file(one, [transform(0, 1, [{}]), transform(1, 2, [{"_t": "1  2 3"}]), shape(2, [(0, {})])],
                           colors),
                  vox_file(one, [transform(0, 1, [{}]), transform(1, 2, [{"_r": "3"}]), shape(2, [(0, {})])], colors),
                  vox_file(one, [transform(0, 1, [{}]), transform(1, 2, [{"_r": "-4"}]), shape(2, [(0, {})])], colors),
                  vox_file(one, [transform(0, 7, [{}])], colors),                             # child out of range
                  vox_file(one, [transform(0, 1, [{}]), shape(1, [(3, {})])], colors),       # model out of range
                  vox_file(one, [transform(0, 1, [{}]), transform(1, 1, [{}])], colors),      # a cycle
                  vox_file(one, [transform(0, 1, [{}]), transform(1, 2, []), shape(2, [(0, {})])], colors),
                  vox_file([], [transform(0, 1, [{}]), group(1, [])], colors)],               # nothing: size 1
    }
    for want, files in cases.items():
        for i, data in enumerate(files):
            assert outcome_oracle(oracle_mod, data, 1) == want, (want, i)
            assert outcome_product(data, 1) == want, (want, i)
    with pytest.raises(SvoError):
        svo.Octree.load_vox("/nonexistent/dir/model.vox", 8)
