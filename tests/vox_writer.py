"""Writes MagicaVoxel .vox files (the published chunk format, version 200) for the import tests:
models, an RGBA palette, a scene graph of transforms, groups and shapes with translation, rotation
and frame attributes, and chunks the importer skips (LAYR, MATL, NOTE)."""
import struct

import numpy as np


def _string(s):
    b = s.encode()
    return struct.pack("<I", len(b)) + b


def _dict(d):
    out = struct.pack("<I", len(d))
    for k, v in d.items():
        out += _string(k) + _string(v)
    return out


def chunk(cid, content, children=b""):
    return cid + struct.pack("<II", len(content), len(children)) + content + children


def model_chunks(size, voxels):
    """size: (x, y, z); voxels: (n, 4) uint8 array of x, y, z, colour index (1..255)."""
    v = np.ascontiguousarray(voxels, dtype=np.uint8)
    return chunk(b"SIZE", struct.pack("<iii", *size)) + chunk(b"XYZI", struct.pack("<I", len(v)) + v.tobytes())


def transform(node_id, child, frames, attrs=None):
    body = struct.pack("<i", node_id) + _dict(attrs or {}) + struct.pack("<iiii", child, -1, 0, len(frames))
    for f in frames:
        body += _dict(f)
    return chunk(b"nTRN", body)


def group(node_id, children):
    return chunk(b"nGRP", struct.pack("<i", node_id) + _dict({}) + struct.pack("<I", len(children)) +
                 b"".join(struct.pack("<i", c) for c in children))


def shape(node_id, models):
    """models: [(model id, attribute dict)]"""
    body = struct.pack("<i", node_id) + _dict({}) + struct.pack("<I", len(models))
    for mid, attrs in models:
        body += struct.pack("<i", mid) + _dict(attrs)
    return chunk(b"nSHP", body)


def palette_chunk(colors):
    """colors: 256 RGBA u32 (0xRRGGBBAA)."""
    return chunk(b"RGBA", b"".join(struct.pack(">I", c) for c in colors))


def vox_file(models, nodes, colors, extra=True):
    """models: [(size, voxels)]; nodes: chunk bytes in node order; colors: 256 RGBA or None."""
    body = b"".join(model_chunks(s, v) for s, v in models) + b"".join(nodes)
    if extra:
        body += chunk(b"LAYR", struct.pack("<i", 0) + _dict({"_name": "layer"}) + struct.pack("<i", -1))
    if colors is not None:
        body += palette_chunk(colors)
    if extra:
        body += chunk(b"MATL", struct.pack("<i", 1) + _dict({"_type": "_diffuse"}))
        body += chunk(b"NOTE", struct.pack("<I", 0))
    return b"VOX " + struct.pack("<i", 200) + chunk(b"MAIN", b"", body)


VALID_ROTATIONS = [b for b in range(128)
                   if (b & 3) < 3 and ((b >> 2) & 3) < 3 and (b & 3) != ((b >> 2) & 3)]


def random_scene(rng, n_models=4, max_size=24, rotate=True, frames=True, density=0.3):
    """A random scene graph: root transform -> group -> per model a transform (translation, an
    optional rotation, sometimes several frames) -> a shape (sometimes with a second model of
    another frame), some transforms nested one group deeper."""
    models = []
    for _ in range(n_models):
        size = tuple(int(v) for v in rng.integers(1, max_size + 1, 3))
        n = int(np.prod(size))
        keep = rng.random(n) < density
        idx = np.nonzero(keep)[0]
        x, y, z = idx % size[0], (idx // size[0]) % size[1], idx // (size[0] * size[1])
        c = rng.integers(1, 256, len(idx))
        models.append((size, np.stack([x, y, z, c], 1).astype(np.uint8)))
    nodes = []
    # node ids in order of appearance: root transform 0, group 1, then per model transform + shape
    nodes.append(None)
    nodes.append(None)
    children = []
    inner = None
    for m in range(n_models):
        t = " ".join(str(int(v)) for v in rng.integers(-40, 41, 3))
        frame = {"_t": t}
        if rotate and rng.random() < 0.7:
            frame["_r"] = str(int(rng.choice(VALID_ROTATIONS)))
        fr = [frame]
        if frames and rng.random() < 0.3:
            fr.append({"_t": "100 100 100", "_f": "1"})
        tid = len(nodes)
        nodes.append(None)
        sid = len(nodes)
        shapes = [(m, {})]
        if frames and rng.random() < 0.3:
            shapes.append(((m + 1) % n_models, {"_f": "1"}))  # another frame's model: skipped
        nodes.append(shape(sid, shapes))
        nodes[tid] = transform(tid, sid, fr)
        if m >= 2 and rng.random() < 0.5:
            if inner is None:
                inner = [len(nodes), len(nodes) + 1, []]  # transform, group, its children
                nodes.append(None)
                nodes.append(None)
                children.append(inner[0])
            inner[2].append(tid)
        else:
            children.append(tid)
    if inner is not None:
        r = {"_t": "3 -2 5"}
        if rotate:
            r["_r"] = str(int(rng.choice(VALID_ROTATIONS)))
        nodes[inner[0]] = transform(inner[0], inner[1], [r])
        nodes[inner[1]] = group(inner[1], inner[2])
    nodes[0] = transform(0, 1, [{}])
    nodes[1] = group(1, children)
    colors = [0] + [int(v) | 0xFF for v in rng.integers(1, 1 << 32, 255, dtype=np.uint64)]
    colors = [int(c) for c in colors]
    return vox_file(models, nodes, colors)
