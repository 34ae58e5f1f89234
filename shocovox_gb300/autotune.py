"""Autotuner of the persistent batched cast (svo_cast_batched).

Sweeps threads per block, rays per warp grab, persistent CTAs per SM, for
batches with camera images (items with a row length) the shape of the ray
blocks a warp casts together, and for batches with rays in no particular order
(items without a row length) the ray-sort key, on the caller's own batch; then,
for the fastest of those, the staging depth (top tree levels every block copies
into shared memory) and, when it sorts, the lane-refill threshold of the sorted
cast.  Keeps the fastest and caches the choice per (GPU name,
workload signature) in a JSON file next to the built library, so later runs skip
the sweep.
"""
import json
import os
import time

from . import _lib

CACHE = os.path.join(os.path.dirname(_lib.lib_path()), "autotune_cache.json")
BLOCKS = (64, 96, 128)
CHUNKS = (32, 64, 128)
PER_SM = (0,)  # 0 = as many as occupancy allows
SHAPES = (3, 4)  # ray blocks of 8 x 4 or 16 x 2 for items with a row length
SORT_KEYS = (0, 1)  # index order, or sorted by direction octant and entry point
STAGING = (1, 2, 3, 4)  # staging depths tried on the best configuration found at depth 0
REFILL = (16, 24, 32)  # lane-refill thresholds tried on the best sorted configuration


def _load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(cache):
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    tmp = CACHE + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def signature(items):
    """Workload class: item count and total rays (log2-bucketed), octree sizes and brick dims present."""
    total = sum(it[2] for it in items)
    sizes = sorted({it[0].size for it in items})
    dims = sorted({it[0].brick_dim for it in items})
    return "items%d_rays2^%d_sizes%s_dims%s" % (len(items), max(total, 1).bit_length(), sizes, dims)


def tune(ws, items, gpu_name, time_fn, use_cache=True):
    """Returns (LaunchConfig, table).  time_fn(cfg) -> milliseconds of one batched cast."""
    key = "%s|%s|refill" % (gpu_name, signature(items))
    cache = _load() if use_cache else {}
    if key in cache:
        b, c, p, sh, so, st, rf = (list(cache[key]["config"]) + [0, 0, 0, 0])[:7]
        return _lib.LaunchConfig(b, c, p, sh, so, st, rf), {"cached": True, **cache[key]}
    shapes = SHAPES if any(len(it) > 4 and it[4] for it in items) else (0,)
    sorts = SORT_KEYS if any(not (len(it) > 4 and it[4]) and it[2] for it in items) else (0,)
    table = {}
    for b in BLOCKS:
        for c in CHUNKS:
            for p in PER_SM:
                for sh in shapes:
                    for so in sorts:
                        table["%dx%dx%dx%dx%dx0x0" % (b, c, p, sh, so)] = time_fn(
                            _lib.LaunchConfig(b, c, p, sh, so, 0, 0))
    b, c, p, sh, so, _, _ = (int(v) for v in min(table, key=table.get).split("x"))
    for st in STAGING:
        table["%dx%dx%dx%dx%dx%dx0" % (b, c, p, sh, so, st)] = time_fn(_lib.LaunchConfig(b, c, p, sh, so, st, 0))
    if so == 1:
        # the sorted cast: its lane-refill threshold at the best staging depth, for every block size (each
        # with its best rays per claim): the refilling kernel's occupancy is not the plain kernel's, so the
        # best block without refill need not be the best with it
        st = int(min((k for k in table if k.startswith("%dx%dx%dx%dx%dx" % (b, c, p, sh, so))), key=table.get).split("x")[5])
        for bb in BLOCKS:
            cc = int(min((k for k in table if k.startswith("%dx" % bb) and k.endswith("x%dx%dx%dx0x0" % (p, sh, so))),
                         key=table.get).split("x")[1])
            for rf in REFILL:
                table["%dx%dx%dx%dx%dx%dx%d" % (bb, cc, p, sh, so, st, rf)] = time_fn(
                    _lib.LaunchConfig(bb, cc, p, sh, so, st, rf))
    best = min(table, key=table.get)
    b, c, p, sh, so, st, rf = (int(v) for v in best.split("x"))
    entry = {"config": [b, c, p, sh, so, st, rf], "ms": table[best], "sweep_ms": table,
             "when": time.strftime("%Y-%m-%dT%H:%M:%S")}
    if use_cache:
        cache[key] = entry
        _store(cache)
    return _lib.LaunchConfig(b, c, p, sh, so, st, rf), {"cached": False, **entry}
