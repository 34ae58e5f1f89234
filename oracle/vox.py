"""MagicaVoxel .vox import restated in Python (TEST INFRASTRUCTURE ONLY).

Restates Octree::load_vox_file / MIPMapStrategy::load_vox_file of shocovox-rs
v0.11.1 (src/convert/magicavoxel.rs:61-385) over the published .vox chunk format
with the conventions of the dot_vox 5.1.1 crate the reference parses files with
(a dependency absent here): models in SIZE/XYZI order, scene nodes in order of
appearance, a voxel's colour index one less than the stored one (saturating at
0) selecting entry i of the RGBA chunk, attribute dictionaries where the last
repeated key wins.  It yields the octree size and the insert sequence; the
oracle's Tree applies them.  Where the reference panics this raises VoxPanic;
malformed bytes raise VoxFormatError.  The tests compare the product's importer
against it; the product does not import it.
"""
import math
import struct

import numpy as np

__all__ = ["VoxPanic", "VoxFormatError", "rotation", "convert_coordinate", "read", "plan", "build"]

I32_MIN, I32_MAX = -(1 << 31), (1 << 31) - 1


class VoxPanic(RuntimeError):
    """The reference panics here."""


class VoxFormatError(ValueError):
    """dot_vox refuses the bytes (the reference's expect() then panics)."""


def wrap32(v):
    return ((v + (1 << 31)) % (1 << 32)) - (1 << 31)


# ---- the chunk format -----------------------------------------------------------------------
class _Reader:
    def __init__(self, data, lo, hi):
        self.d, self.i, self.hi = data, lo, hi

    def u32(self):
        if self.hi - self.i < 4:
            raise VoxFormatError("truncated")
        v = struct.unpack_from("<I", self.d, self.i)[0]
        self.i += 4
        return v

    def i32(self):
        return wrap32(self.u32())

    def string(self):
        n = self.u32()
        if self.hi - self.i < n:
            raise VoxFormatError("truncated string")
        s = self.d[self.i:self.i + n].decode("utf-8", "surrogateescape")
        self.i += n
        return s

    def dictionary(self):
        out = {}
        for _ in range(self.u32()):
            k = self.string()
            out[k] = self.string()
        return out


def read(data):
    """bytes -> {"models": [(size (3 ints), uint8 array (n, 4))], "nodes": [...], "palette": [rgba] or None}.
    Nodes are ("T", child, [frame dicts]), ("G", [children]) or ("S", [(model id, dict)])."""
    data = bytes(data)
    if len(data) < 8 or data[:4] != b"VOX ":
        raise VoxFormatError("not a .vox file")
    if len(data) < 20 or data[8:12] != b"MAIN":
        raise VoxFormatError("no MAIN chunk")
    content, children = struct.unpack_from("<II", data, 12)
    if len(data) - 20 < content + children:
        raise VoxFormatError("truncated MAIN")
    at, end = 20 + content, 20 + content + children
    models, nodes, palette, pending = [], [], None, False
    while at < end:
        if end - at < 12:
            raise VoxFormatError("truncated chunk header")
        cid = data[at:at + 4]
        n, m = struct.unpack_from("<II", data, at + 4)
        body = at + 12
        if end - body < n + m:
            raise VoxFormatError("truncated chunk")
        r = _Reader(data, body, body + n)
        if cid == b"SIZE":
            models.append([(r.i32(), r.i32(), r.i32()), np.zeros((0, 4), np.uint8)])
            pending = True
        elif cid == b"XYZI":
            if not pending:
                raise VoxFormatError("XYZI without SIZE")
            k = r.u32()
            if k * 4 > r.hi - r.i:
                raise VoxFormatError("truncated XYZI")
            models[-1][1] = np.frombuffer(data, np.uint8, k * 4, r.i).reshape(k, 4)
            pending = False
        elif cid == b"RGBA":
            if n < 1024:
                raise VoxFormatError("truncated RGBA")
            q = np.frombuffer(data, np.uint8, 1024, body).reshape(256, 4).astype(np.uint32)
            palette = [int(v) for v in (q[:, 0] << 24) | (q[:, 1] << 16) | (q[:, 2] << 8) | q[:, 3]]
        elif cid == b"nTRN":
            r.i32()
            r.dictionary()
            child = r.u32()
            r.i32()
            r.i32()
            nodes.append(("T", child, [r.dictionary() for _ in range(r.u32())]))
        elif cid == b"nGRP":
            r.i32()
            r.dictionary()
            nodes.append(("G", [r.u32() for _ in range(r.u32())]))
        elif cid == b"nSHP":
            r.i32()
            r.dictionary()
            shapes = []
            for _ in range(r.u32()):
                mid = r.u32()
                shapes.append((mid, r.dictionary()))
            nodes.append(("S", shapes))
        at = body + n + m
    return {"models": models, "nodes": nodes, "palette": palette}


# ---- magicavoxel.rs ------------------------------------------------------------------------------
def rotation(b):
    """parse_rotation_matrix (magicavoxel.rs:61-90) as a row-major 3x3 list."""
    c0, c1 = b & 3, (b >> 2) & 3
    c2 = ~(c0 ^ c1) & 3
    if max(c0, c1, c2) > 2:
        raise VoxPanic("index out of bounds: the len is 3 but the index is 3")
    m = [[0] * 3 for _ in range(3)]
    m[0][c0] = -1 if b & 0x10 else 1
    m[1][c1] = -1 if b & 0x20 else 1
    m[2][c2] = -1 if b & 0x40 else 1
    return m


def _matmul(a, b):
    return [[sum(a[i][k] * b[k][j] for k in range(3)) for j in range(3)] for i in range(3)]


def _transformed(v, m):  # magicavoxel.rs:96-102
    return [wrap32(v[0] * m[i][0] + v[1] * m[i][1] + v[2] * m[i][2]) for i in range(3)]


_SWAP = {("Lyup", "Ryup"): lambda c: (c[0], c[1], -c[2]), ("Lzup", "Rzup"): lambda c: (c[0], -c[1], c[2]),
         ("Lyup", "Lzup"): lambda c: (c[0], -c[2], c[1]), ("Lzup", "Lyup"): lambda c: (c[0], c[2], -c[1]),
         ("Lyup", "Rzup"): lambda c: (c[0], c[2], c[1]), ("Ryup", "Lzup"): lambda c: (c[0], c[2], c[1])}


def convert_coordinate(c, src, dst):
    """convert_coordinate (src/spatial/math/mod.rs:174-201)."""
    if src == dst:
        return tuple(c)
    for (a, b), f in _SWAP.items():
        if (src, dst) in ((a, b), (b, a)):
            return f(c)
    # (Ryup, Rzup) and (Rzup, Ryup) follow (Lyup, Lzup) and (Lzup, Lyup)
    pair = {("Ryup", "Rzup"): ("Lyup", "Lzup"), ("Rzup", "Ryup"): ("Lzup", "Lyup")}[(src, dst)]
    return _SWAP[pair](c)


def _rust_int(s, signed, lo, hi):
    body = s[1:] if s[:1] == "+" or (signed and s[:1] == "-") else s
    if not body or not all("0" <= ch <= "9" for ch in body):
        raise VoxPanic("invalid digit in %r" % s)
    v = -int(body) if s[:1] == "-" else int(body)
    if not lo <= v <= hi:
        raise VoxPanic("number out of range: %r" % s)
    return v


def _iterate(vox, fun):
    """iterate_vox_tree (magicavoxel.rs:104-202) for frame 0."""
    nodes, models = vox["nodes"], vox["models"]
    if not nodes or nodes[0][0] != "T":
        raise VoxPanic("The root node for a magicka voxel DAG should be a translation")
    ident = [[1, 0, 0], [0, 1, 0], [0, 0, 1]]
    stack = [[nodes[0][1], (0, 0, 0), ident, 0]]
    steps = 0
    while stack:
        steps += 1
        if len(stack) > len(nodes) + 1 or steps > (1 << 28):
            raise VoxPanic("the scene graph does not terminate")
        node, t, rot, index = stack[-1]
        if node >= len(nodes):
            raise VoxPanic("scene node index out of bounds")
        n = nodes[node]
        if n[0] == "T":
            if not n[2]:
                raise VoxPanic("index out of bounds: frames")
            fr = n[2][0]
            if "_t" in fr:
                parts = [_rust_int(p, True, I32_MIN, I32_MAX) for p in fr["_t"].split(" ")]
                if len(parts) < 3:
                    raise VoxPanic("index out of bounds: translation")
                t2 = tuple(wrap32(t[k] + parts[k]) for k in range(3))
            else:
                t2 = t
            r2 = _matmul(rot, rotation(_rust_int(fr["_r"], False, 0, 255))) if "_r" in fr else ident
            if index == 0:
                stack[-1][3] += 1
                stack.append([n[1], t2, r2, 0])
            else:
                stack.pop()
        elif n[0] == "G":
            if index < len(n[1]):
                stack[-1][3] += 1
                stack.append([n[1][index], t, rot, 0])
            else:
                stack.pop()
        else:
            for mid, attrs in n[1]:
                if _rust_int(attrs.get("_f", "0"), False, 0, (1 << 64) - 1) == 0:
                    if mid >= len(models):
                        raise VoxPanic("model index out of bounds")
                    fun(models[mid], t, rot)
            stack.pop()
            if stack:
                stack[-1][3] += 1


def _half(size, rot):
    # V3c<i32> / 2 truncates towards zero
    return [v // 2 if v >= 0 else -((-v) // 2) for v in _transformed(size, rot)]


def _bounds_rzup(vox):
    lo, hi = [I32_MAX] * 3, [I32_MIN] * 3

    def fun(model, pos, rot):
        h = _half(model[0], rot)
        for k in range(3):
            a, b = wrap32(pos[k] - h[k]), wrap32(pos[k] + h[k])
            lo[k] = min(lo[k], a, b)
            hi[k] = max(hi[k], b, a)
    _iterate(vox, fun)
    return lo, hi


def tree_size(vox):
    """Octree::load_vox_file's size (magicavoxel.rs:265-270)."""
    lo, hi = _bounds_rzup(vox)
    lo, hi = convert_coordinate(lo, "Rzup", "Lyup"), convert_coordinate(hi, "Rzup", "Lyup")
    e = max(wrap32(hi[k] - lo[k]) for k in range(3))
    ef = np.float32(e)
    with np.errstate(divide="ignore", invalid="ignore"):
        lg = float(np.ceil(np.log2(ef)))
    x = 0 if (math.isnan(lg) or lg <= 0) else (0xFFFFFFFF if lg >= 4294967295.0 else int(lg))
    return 0 if x >= 32 else (1 << x)


def plan(data):
    """(octree size, [(x, y, z, rgba) in insertion order]) of load_vox_file on these bytes."""
    vox = read(data)
    size = tree_size(vox)
    lo, _ = _bounds_rzup(vox)
    if vox["palette"] is None:
        raise VoxFormatError("no RGBA chunk")
    pal = vox["palette"]
    out = []

    def fun(model, pos, rot):
        h = _half(model[0], rot)
        bl = [wrap32(pos[k] - h[k] - lo[k] + (-1 if h[k] < 0 else 0)) for k in range(3)]
        for x, y, z, i in model[1].tolist():
            d = _transformed((x, y, z), rot)
            p = convert_coordinate([wrap32(bl[k] + d[k]) for k in range(3)], "Rzup", "Lyup")
            out.append((p[0] & 0xFFFFFFFF, p[1] & 0xFFFFFFFF, p[2] & 0xFFFFFFFF, pal[max(i - 1, 0)]))
    _iterate(vox, fun)
    return size, out


def build(oracle_mod, data, brick_dim, configure=None):
    """An oracle Tree holding the file's voxels, like Octree::load_vox_file (with `configure` run on
    the empty tree first, like MIPMapStrategy::load_vox_file)."""
    size, voxels = plan(data)
    try:
        t = oracle_mod.Tree(size, brick_dim)
    except oracle_mod.OracleError as e:  # Octree::new's error panics (magicavoxel.rs:271-279)
        raise VoxPanic("Octree::new(%d, %d) yielded error %d" % (size, brick_dim, e.code)) from e
    if configure is not None:
        configure(t)
    # an insert error panics in the reference (magicavoxel.rs:363-381)
    if voxels and max(max(v[:3]) for v in voxels) < 65536:
        ops = np.zeros(len(voxels), oracle_mod.OP_DTYPE)
        arr = np.array(voxels, dtype=np.uint64)
        ops["x"], ops["y"], ops["z"] = arr[:, 0], arr[:, 1], arr[:, 2]
        ops["op"], ops["kind"], ops["size"], ops["rgba"] = 0, 1, 1, arr[:, 3]
        try:
            t.apply_ops(ops)
        except oracle_mod.OracleError as e:
            raise VoxPanic("inserting into octree yielded error %d" % e.code) from e
    else:
        for x, y, z, c in voxels:
            rc = t.insert((x, y, z), albedo=c)
            if rc != 0:
                raise VoxPanic("inserting into octree at (%d, %d, %d) yielded error %d" % (x, y, z, rc))
    return t
