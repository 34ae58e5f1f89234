"""The batched cast's autotuner (shocovox_gb300/autotune.py): which knobs it sweeps for which batch,
that it keeps the fastest configuration, and its per-workload cache. Host logic only: the timing
function is a stand-in, so no GPU is needed."""
import json

import pytest

from shocovox_gb300 import autotune
from shocovox_gb300._lib import LaunchConfig

import bench


class FakeScene:
    def __init__(self, size, brick_dim):
        self.size, self.brick_dim = size, brick_dim


def items_of(*specs):
    """specs: (size, brick dim, rays, row length) -> batch items as the autotuner sees them."""
    return [(FakeScene(s, d), {}, n, {}, row) for s, d, n, row in specs]


def fake_time(best, best_stage=0, best_refill=0):
    seen = []

    def time_fn(cfg):
        key = (cfg.block, cfg.rays_per_chunk, cfg.blocks_per_sm, cfg.block_shape, cfg.sort_key)
        seen.append(key + (cfg.staging_depth, cfg.refill_below))
        if key != best:
            return 2.0 + 0.001 * len(seen)
        # the best knobs: fastest at depth best_stage, and with refill best_refill (when not 0)
        return 1.0 - 0.1 * (cfg.staging_depth == best_stage) - 0.05 * (best_refill and cfg.refill_below == best_refill)

    return time_fn, seen


@pytest.mark.parametrize("rows,want_shapes,want_sorts", [
    ((0,), {0}, {0, 1}),             # rays in no particular order: the sort key is swept
    ((640,), {3, 4}, {0}),           # a camera image: the ray-block shape is swept
    ((640, 0), {3, 4}, {0, 1}),      # both kinds in one batch
])
def test_sweep_covers_the_knobs_of_the_batch(rows, want_shapes, want_sorts):
    items = items_of(*[(128, 4, 5000, r) for r in rows])
    best = (96, 64, 0, max(want_shapes), max(want_sorts))
    time_fn, seen = fake_time(best)
    cfg, info = autotune.tune(None, items, "gpu", time_fn, use_cache=False)
    assert {k[3] for k in seen} == want_shapes
    assert {k[4] for k in seen} == want_sorts
    assert {k[0] for k in seen} == set(autotune.BLOCKS) and {k[1] for k in seen} == set(autotune.CHUNKS)
    first = len(autotune.BLOCKS) * len(autotune.CHUNKS) * len(want_shapes) * len(want_sorts)
    # the refill stage only for a sorted best, at every block size
    refills = len(autotune.BLOCKS) * len(autotune.REFILL) if best[4] == 1 else 0
    assert len(seen) == len(set(seen)) == first + len(autotune.STAGING) + refills
    assert all(k[5] == 0 and k[6] == 0 for k in seen[:first])  # the first stage: nothing staged, no refill
    stage = seen[first:first + len(autotune.STAGING)]
    assert [k[:5] for k in stage] == [best] * len(autotune.STAGING)  # then the depths on the best
    assert {k[5] for k in stage} == set(autotune.STAGING) and all(k[6] == 0 for k in stage)
    assert {k[6] for k in seen[first + len(autotune.STAGING):]} == (set(autotune.REFILL) if refills else set())
    assert {k[0] for k in seen[first + len(autotune.STAGING):]} == (set(autotune.BLOCKS) if refills else set())
    assert (cfg.block, cfg.rays_per_chunk, cfg.blocks_per_sm, cfg.block_shape, cfg.sort_key) == best
    assert cfg.staging_depth == 0 and cfg.refill_below == 0
    assert info["cached"] is False and info["config"] == list(best) + [0, 0]


@pytest.mark.parametrize("depth", [0, 2, 4])
def test_staging_depth_is_kept_only_when_faster(depth):
    items = items_of((512, 8, 100000, 0))
    best = (64, 32, 0, 0, 1)
    time_fn, seen = fake_time(best, best_stage=depth)
    cfg, info = autotune.tune(None, items, "gpu", time_fn, use_cache=False)
    assert cfg.staging_depth == depth and info["config"][5] == depth


@pytest.mark.parametrize("refill", [0, 24])
def test_refill_is_swept_for_the_sorted_cast(refill):
    items = items_of((1024, 8, 4_000_000, 0))
    best = (128, 32, 0, 0, 1)
    time_fn, seen = fake_time(best, best_stage=0, best_refill=refill)
    cfg, info = autotune.tune(None, items, "gpu", time_fn, use_cache=False)
    assert cfg.sort_key == 1 and cfg.refill_below == refill and info["config"][6] == refill
    # refill is tried only with the sort
    time_fn, seen = fake_time((128, 32, 0, 0, 0))
    autotune.tune(None, items, "gpu", time_fn, use_cache=False)
    assert {k[6] for k in seen} == {0}


def test_empty_items_do_not_ask_for_the_sort():
    items = items_of((64, 2, 0, 0), (128, 4, 3000, 320))
    time_fn, seen = fake_time(None)
    autotune.tune(None, items, "gpu", time_fn, use_cache=False)
    assert {k[4] for k in seen} == {0}


def test_cache_round_trip_and_older_entries(tmp_path, monkeypatch):
    monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "cache.json"))
    items = items_of((256, 8, 100000, 0), (64, 2, 2000, 0))
    best = (128, 32, 0, 0, 1)
    time_fn, seen = fake_time(best)
    cfg, info = autotune.tune(None, items, "GB300", time_fn)
    assert not info["cached"] and cfg.sort_key == 1
    n = len(seen)
    cfg2, info2 = autotune.tune(None, items, "GB300", time_fn)
    assert info2["cached"] and len(seen) == n  # no second sweep
    assert (cfg2.block, cfg2.rays_per_chunk, cfg2.blocks_per_sm, cfg2.block_shape, cfg2.sort_key) == best
    assert cfg2.staging_depth == cfg.staging_depth
    # another GPU name or workload class is tuned on its own
    autotune.tune(None, items, "other", time_fn)
    assert len(seen) > n
    # an entry with four knobs (no sort key, no staging depth) reads as index order, nothing staged
    with open(autotune.CACHE) as f:
        cache = json.load(f)
    key = "GB300|%s|refill" % autotune.signature(items)
    cache[key]["config"] = [64, 128, 0, 4]
    with open(autotune.CACHE, "w") as f:
        json.dump(cache, f)
    cfg3, _ = autotune.tune(None, items, "GB300", time_fn)
    assert (cfg3.block, cfg3.rays_per_chunk, cfg3.block_shape, cfg3.sort_key, cfg3.staging_depth) == (64, 128, 4, 0, 0)


def test_signature_buckets_the_workload():
    a = items_of((128, 4, 5000, 0), (256, 8, 3000, 0))
    b = items_of((256, 8, 4000, 0), (128, 4, 4000, 0))
    assert autotune.signature(a) == autotune.signature(b)  # same sizes, dims, count, log2 of rays
    assert autotune.signature(a) != autotune.signature(items_of((128, 4, 5000, 0)))
    assert autotune.signature(a) != autotune.signature(items_of((128, 4, 50000, 0), (256, 8, 30000, 0)))


def test_launch_count_of_a_batched_call():
    # the claim-order kernel once if any item is cast in claim order, the sort's six launches once
    # if any item is sorted
    cam, rnd, empty = (None, {}, 100, {}, 64), (None, {}, 100, {}, 0), (None, {}, 0, {}, 0)
    assert bench.batched_launches([cam, rnd], 0) == 1
    assert bench.batched_launches([cam, rnd], 1) == 7
    assert bench.batched_launches([rnd, rnd], 1) == 6
    assert bench.batched_launches([cam, empty], 1) == 1
    assert LaunchConfig(1, 2, 3, 4, 1).sort_key == 1 and LaunchConfig().sort_key == 0
    assert LaunchConfig(1, 2, 3, 4, 1, 3).staging_depth == 3 and LaunchConfig().staging_depth == 0
    assert LaunchConfig(1, 2, 3, 4, 1, 3, 24).refill_below == 24 and LaunchConfig().refill_below == 0
