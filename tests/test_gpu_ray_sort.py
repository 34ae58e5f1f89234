"""The batched cast's ray sort (svo_launch_config.sort_key = 1): the items without a row length are
binned by direction octant and entry point, scanned, scattered into bucket order and cast from there.
Every hit field and counter stays the oracle's (Octree::get_by_ray, src/raytracing/raytracing_on_cpu.rs:
316-565), whatever the bucket order, the launch configuration, the mix of sorted and claim-order items,
the workspace's growth between calls and a CUDA-graph replay."""
import numpy as np
import pytest

import shocovox_gb300 as svo
from test_gpu_cast import assert_same_hits, both, random_rays

pytestmark = pytest.mark.gpu


def make_items(oracle_mod, torch, specs, seed):
    """specs: (kind, size, brick dim, rays, row length); returns items, expected hits, tensors kept alive."""
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(seed)
    items, expected, keep = [], [], []
    for j, (kind, size, dim, nrays, row) in enumerate(specs):
        ops = svo.gen_scene(kind, size, dim, seed=seed + j, occupancy=0.1, spheres=3, octaves=2, base_freq=1.0 / 16,
                            height_lo=2.0, height_hi=size * 0.4)
        o, p = both(oracle_mod, size, dim, ops)
        origins, dirs = random_rays(rng, size, nrays)
        cols = {k: torch.from_numpy(np.ascontiguousarray(a[:, i]) if nrays else np.zeros(0, np.float32)).to(dev)
                for a, names in ((origins, ("ox", "oy", "oz")), (dirs, ("dx", "dy", "dz")))
                for i, k in enumerate(names)}
        out = {k: torch.zeros(max(nrays, 1), dtype=getattr(torch, np.dtype(t).name), device=dev)
               for k, t in svo.HIT_FIELDS.items()}
        items.append((p, {k: v.data_ptr() for k, v in cols.items()}, nrays, {k: v.data_ptr() for k, v in out.items()},
                      row))
        expected.append(o.cast(origins, dirs, threads=8) if nrays else None)
        keep.append((p, cols, out))
    return items, expected, keep


def check(keep, expected, label):
    for j, ((_, _, out), exp) in enumerate(zip(keep, expected)):
        if exp is None:
            continue
        n = len(exp["status"])
        g = {k: v.cpu().numpy()[:n] for k, v in out.items()}
        assert_same_hits(g, exp, counters=True, label="%s item %d" % (label, j))


def clear(keep):
    for _, _, out in keep:
        for v in out.values():
            v.fill_(0x5A)  # every field must be written by the cast


SPECS = [(0, 128, 4, 6000, 0), (3, 64, 2, 1, 0), (3, 32, 8, 0, 0), (1, 64, 8, 33, 0), (2, 256, 8, 20000, 0),
         (3, 64, 1, 2500, 40), (0, 64, 4, 3000, 0)]


def test_sorted_items_match_the_oracle(oracle_mod):
    torch = pytest.importorskip("torch")
    items, expected, keep = make_items(oracle_mod, torch, SPECS, 700)
    ws = svo.BatchWorkspace()
    s = torch.cuda.current_stream().cuda_stream
    with pytest.raises(Exception):
        ws.cast(items, svo.LaunchConfig(0, 0, 0, 0, 2), s)  # no such sort key
    for cfg in (svo.LaunchConfig(0, 0, 0, 0, 1), svo.LaunchConfig(64, 32, 0, 0, 1), svo.LaunchConfig(128, 100, 0, 4, 1),
                svo.LaunchConfig(96, 256, 3, 0, 1), svo.LaunchConfig(32, 64, 1, 5, 1)):
        clear(keep)
        ws.cast(items, cfg, s)
        torch.cuda.synchronize()
        check(keep, expected, "cfg %d/%d/%d" % (cfg.block, cfg.rays_per_chunk, cfg.blocks_per_sm))


def test_sort_only_items_and_literal_form(oracle_mod):
    # every item sorted (no claim-order launch), and the literal form of the cast (its rays key on their origin)
    torch = pytest.importorskip("torch")
    specs = [(0, 128, 4, 5000, 0), (2, 64, 2, 3000, 0)]
    items, expected, keep = make_items(oracle_mod, torch, specs, 800)
    ws = svo.BatchWorkspace()
    s = torch.cuda.current_stream().cuda_stream
    for mode in (0, 1):
        assert svo.lib().svo_set_cast_mode(mode) == 0
        try:
            clear(keep)
            ws.cast(items, svo.LaunchConfig(0, 0, 0, 0, 1), s)
            torch.cuda.synchronize()
        finally:
            svo.lib().svo_set_cast_mode(0)
        check(keep, expected, "cast mode %d" % mode)


def test_sort_buffers_grow_and_graph_replay(oracle_mod):
    torch = pytest.importorskip("torch")
    small, exp_small, keep_small = make_items(oracle_mod, torch, [(0, 64, 4, 500, 0)], 900)
    large, exp_large, keep_large = make_items(oracle_mod, torch, SPECS[:5], 901)
    ws = svo.BatchWorkspace()
    s = torch.cuda.current_stream().cuda_stream
    cfg = svo.LaunchConfig(128, 64, 7, 0, 1)
    for items, expected, keep, label in ((small, exp_small, keep_small, "small"), (large, exp_large, keep_large, "grown"),
                                         (small, exp_small, keep_small, "small again")):
        clear(keep)
        ws.cast(items, cfg, s)
        torch.cuda.synchronize()
        check(keep, expected, label)
    # a stream capture cannot grow the buffers: the largest call was made before it
    gs = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(gs):
        ws.cast(large, cfg, gs.cuda_stream)
        torch.cuda.synchronize()
        with torch.cuda.graph(graph, stream=gs):
            ws.cast(large, cfg, gs.cuda_stream)
    torch.cuda.synchronize()
    for rep in range(2):
        clear(keep_large)
        torch.cuda.synchronize()
        graph.replay()
        torch.cuda.synchronize()
        check(keep_large, exp_large, "graph replay %d" % rep)


def test_noalloc_refuses_the_sort():
    import ctypes
    from shocovox_gb300._lib import BatchItem, LaunchConfig
    arr = (BatchItem * 1)()
    rc = svo.lib().svo_cast_batched_noalloc(arr, 1, ctypes.byref(LaunchConfig(0, 0, 0, 0, 1)), None)
    assert rc == 6  # SVO_ERR_ARGUMENT
    assert b"needs a batch workspace" in svo.lib().svo_last_error()
