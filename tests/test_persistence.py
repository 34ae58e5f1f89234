"""Scene persistence in the reference's bytecode format (Octree::to_bytes / from_bytes / save / load,
src/octree/mod.rs:138-168; format of src/convert/bytecode.rs and src/object_pool.rs:25-140).

The product's bytes are decoded here by an independent bencode reader and checked field by field
against the oracle's structure of the same scene; loading them back must give the same structure,
and corrupt input must be refused with a status code."""
import os

import numpy as np
import pytest

import shocovox_gb300 as svo
from shocovox_gb300._lib import SvoError
from helpers import ALBEDO, CLEAR, COMPLEX, DATA, INSERT, INSERT_AT_LOD, ops_from


def bdecode(data, i=0):
    """bencode -> (value, next index): ints, byte strings (bytes) and lists."""
    c = data[i:i + 1]
    if c == b"i":
        j = data.index(b"e", i)
        return int(data[i + 1:j]), j + 1
    if c == b"l":
        out, i = [], i + 1
        while data[i:i + 1] != b"e":
            v, i = bdecode(data, i)
            out.append(v)
        return out, i + 1
    j = data.index(b":", i)
    n = int(data[i:j])
    return data[j + 1:j + 1 + n], j + 1 + n


def fnv(values):  # the brick hash of the node records
    h = 1469598103934665603
    for w in values:
        for b in range(4):
            h ^= (w >> (8 * b)) & 0xFF
            h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h ^ len(values)


def brick_record(b):
    """(kind as numbered in the records, solid value, parted hash) of a decoded brick."""
    if b == b"#b":
        return 0, 0, 0
    if b[0] == b"#b#":
        return 2, b[1], 0
    assert b[0] == b"##b#" and b[-1] == b"#" and b[1] == len(b) - 3
    return 1, 0, fnv(b[2:-1])


def records_from_bytes(data):
    """Node records (the layout of svo_node_record / orc_node_record) rebuilt from decoded bytes."""
    tree, end = bdecode(data)
    assert end == len(data) and len(tree) == 9
    auto_simplify, size, dim, pool, children, mips, colours, datas, strategy = tree
    first_available, items = pool
    recs = []
    for k, (reserved, content) in enumerate(items):
        r = [0] * 40
        r[0] = reserved
        if reserved:
            if content == b"#":
                kind = 0
            else:
                kind = {b"##": 1, b"###": 2, b"##u#": 3}[content[0]]
            r[1] = kind
            if kind == 1:
                r[2] = content[1]
            bricks = content[1:9] if kind == 2 else (content[1:2] if kind == 3 else [])
            for i, b in enumerate(bricks):
                r[13 + i], r[21 + i], r[29 + i] = brick_record(b)
        c = children[k]
        if c == b"##x##":
            r[3] = 0
        elif c[0] == b"##c##":
            r[3] = 1
            r[4:12] = c[1:9]
        else:
            assert c[0] == b"##b##"
            r[3] = 2
            r[12] = c[1]
        if k < len(mips):
            r[37], r[38], r[39] = brick_record(mips[k])
        else:
            r[37] = 3
        recs.append(r)
    palette = [(r << 24) | (g << 16) | (b << 8) | a for r, g, b, a in colours]
    return recs, palette, datas, strategy, (auto_simplify, size, dim)


def scene_ops(size, seed):
    rng = np.random.default_rng(seed)
    ops = []
    for _ in range(400):
        x, y, z = (int(v) for v in rng.integers(0, size, 3))
        r = rng.random()
        if r < 0.7:
            kind = int(rng.choice([ALBEDO, DATA, COMPLEX]))
            ops.append((INSERT, x, y, z, kind, int(rng.integers(1, 1 << 32)) | 0xFF, int(rng.integers(1, 4096)), 1))
        elif r < 0.85:
            s = int(rng.choice([2, 4]))
            ops.append((INSERT_AT_LOD, x - x % s, y - y % s, z - z % s, ALBEDO, 0x336699FF, 0, s))
        else:
            ops.append((CLEAR, x, y, z, 0, 0, 0, 1))
    return ops_from(ops)


def oracle_records(o):
    return [list(r) for r in o.records()]


@pytest.mark.parametrize("size,dim,mips", [(32, 2, False), (64, 4, True), (64, 8, False)])
def test_bytes_decode_to_the_oracle_structure(oracle_mod, size, dim, mips):
    ops = scene_ops(size, size + dim)
    o = oracle_mod.Tree(size, dim)
    p = svo.Octree(size, dim)
    o.apply_ops(ops)
    p.apply_ops(ops)
    if mips:
        o.mip_switch(True)
        p.switch_albedo_mip_maps(True)
    recs, palette, datas, strategy, head = records_from_bytes(p.to_bytes())
    assert head == (1, size, dim)
    want = oracle_records(o)
    # freed nodes are written without content (the reference keeps a freed node's last content)
    for r, w in zip(recs, want):
        if not w[0]:
            w[1:3] = [0, 0]
            w[13:37] = [0] * 24
    assert recs == want
    assert palette == [int(c) for c in o.palette(0)]
    assert datas == [int(d) for d in o.palette(1)]
    # the default strategy: PointFilter at level 1, BoxFilter at 2-4, thresholds 0.1 / 0.05 / 0.02
    enabled, n = strategy[0], strategy[1]
    assert enabled == int(mips) and n == 4
    assert dict(zip(strategy[2:2 + 2 * n:2], strategy[3:3 + 2 * n:2])) == {1: 1, 2: 0, 3: 0, 4: 0}
    m = strategy[2 + 2 * n]
    assert dict(zip(strategy[3 + 2 * n::2], strategy[4 + 2 * n::2])) == {2: 100, 3: 50, 4: 20} and m == 3


def test_round_trip_keeps_structure_and_results(oracle_mod, tmp_path):
    ops = scene_ops(64, 3)
    p = svo.Octree(64, 4)
    p.apply_ops(ops)
    p.set_mip_method(2, svo.Octree.POSTERIZE, 0.25).set_mip_color_threshold(3, 0.3)
    p.switch_albedo_mip_maps(True)
    data = p.to_bytes()
    q = svo.Octree.from_bytes(data)
    assert q.records() == p.records()
    assert q.to_bytes() == data
    path = str(tmp_path / "scene.bencode")
    p.save(path)
    r = svo.Octree.load(path)
    assert r.records() == p.records() and os.path.getsize(path) == len(data)
    # the loaded scene keeps working: the same edits give the same structure (with MIPs enabled an
    # edit can reach the reference's node_mips panic: both stop at the same operation)
    more = scene_ops(64, 4)
    assert stop_of(p, more) == stop_of(r, more)
    assert r.records() == p.records()
    for pos in [(1, 2, 3), (10, 20, 30), (63, 63, 63)]:
        assert r.get(pos) == p.get(pos)


def stop_of(t, ops):
    try:
        t.apply_ops(ops)
        return None
    except svo.OctreeError as e:
        return e.code, str(e).split(":")[0]


def test_corrupt_bytes_are_refused():
    data = svo.Octree(16, 2).to_bytes()
    for bad in (b"", b"x", data[:-1], data + b"e", data.replace(b"i16e", b"i17e", 1), b"li1ei16ei2ee"):
        with pytest.raises(SvoError):
            svo.Octree.from_bytes(bad)
    with pytest.raises(SvoError):
        svo.Octree.load("/nonexistent/dir/scene.bencode")
