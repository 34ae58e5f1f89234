"""svo_cast_batched_noalloc gives the same results as svo_cast_batched.

The allocation-free entry point serves callers that cannot allocate device
memory when they cast (a fixed budget handed over at start-up, or a frame loop
where a cudaMalloc would synchronise the device): its item table and work
counter live in a fixed scratch array inside the library.  This file is named
to be collected last, and builds everything it needs itself, so it passes
alone in a fresh process as well as after the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-4  # voxel units, impact point and normal (ints compare exactly)
FIELDS = ("status", "brick_octant", "entry_kind", "node_key", "voxel_index", "pix", "albedo", "user",
          "px", "py", "pz", "nx", "ny", "nz")
COUNTERS = ("node_visits", "child_reads", "voxel_reads", "run_visits")


def _scene(svo, kind, size, dim, seed):
    ops = svo.gen_scene(kind, size, dim, seed=seed, occupancy=0.1, spheres=3, octaves=2, base_freq=1.0 / 16,
                        height_lo=2.0, height_hi=size * 0.35)
    t = svo.Octree(size, dim)
    t.apply_ops(ops)
    t.upload()
    return t


def _rays(rng, size, n):
    o = rng.uniform(-0.3 * size, 1.3 * size, (n, 3)).astype(np.float32)
    t = rng.uniform(0, size, (n, 3)).astype(np.float32)
    d = t - o
    d /= np.sqrt((d.astype(np.float64) ** 2).sum(1))[:, None].astype(np.float32)
    return o, d.astype(np.float32)


def _camera(svo, size, width, height):
    """A camera image in raster order (rows of `width` rays), cast with the item's row length."""
    return svo.gen_camera_rays([1.4 * size, 0.9 * size, 1.2 * size], [size / 2, size / 3, size / 2], 60.0,
                               width, height)


def _dev_rays(torch, o, d, dev):
    return {k: torch.from_numpy(np.ascontiguousarray(a[:, i]) if len(a) else np.zeros(0, np.float32)).to(dev)
            for a, names in ((o, ("ox", "oy", "oz")), (d, ("dx", "dy", "dz"))) for i, k in enumerate(names)}


def _outputs(torch, svo, n, dev, fields):
    tmap = {np.uint8: torch.uint8, np.uint32: torch.int32, np.float32: torch.float32}
    return {k: torch.zeros(max(n, 1), dtype=tmap[svo.HIT_FIELDS[k]], device=dev) for k in fields}


def _items(svo, batches):
    from shocovox_gb300._lib import BatchItem, Hits, Rays
    arr = (BatchItem * len(batches))()
    for i, (scene, rays, n, out, row) in enumerate(batches):
        arr[i].scene = scene.handle
        arr[i].rays = Rays(*[ctypes.c_void_p(rays[k].data_ptr()) for k in ("ox", "oy", "oz", "dx", "dy", "dz")])
        arr[i].n = n
        arr[i].hits = Hits(**{k: ctypes.c_void_p(out[k].data_ptr()) if k in out else None for k in svo.HIT_FIELDS})
        arr[i].row_length = row
    return arr


def _assert_same(got, ref, n, where):
    for k in ref:
        a, b = got[k][:n].cpu().numpy(), ref[k][:n].cpu().numpy()
        if a.dtype == np.float32:
            same = (a == b) | (np.isnan(a) & np.isnan(b))
            with np.errstate(invalid="ignore"):
                assert np.all(same | (np.abs(a.astype(np.float64) - b) <= TOL)), (where, k)
        else:
            assert np.array_equal(a, b), (where, k)


def _workspace_cast(svo, lib, batches, cfg, stream):
    ws = ctypes.c_void_p()
    assert lib.svo_batch_workspace_create(ctypes.byref(ws)) == 0
    try:
        arr = _items(svo, batches)
        rc = lib.svo_cast_batched(ws, arr, len(batches), ctypes.byref(cfg) if cfg is not None else None,
                                  ctypes.c_void_p(stream))
        assert rc == 0, lib.svo_last_error()
    finally:
        import torch
        torch.cuda.synchronize()
        lib.svo_batch_workspace_destroy(ws)


@pytest.fixture(scope="module")
def mixed_batch():
    """Four scenes, each with random rays (no row length) and most with a camera image (a row length)."""
    torch = pytest.importorskip("torch")
    import shocovox_gb300 as svo
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(12345)
    specs = [(3, 64, 4, 3000, (45, 23)), (0, 128, 8, 5000, (96, 40)), (1, 64, 2, 0, (17, 9)), (3, 32, 1, 2000, None)]
    items = []
    for j, (kind, size, dim, n, cam) in enumerate(specs):
        scene = _scene(svo, kind, size, dim, 900 + j)
        o, d = _rays(rng, size, n)
        items.append((scene, _dev_rays(torch, o, d, dev), n, 0))
        if cam:
            o, d = _camera(svo, size, *cam)
            items.append((scene, _dev_rays(torch, o, d, dev), len(o), cam[0]))
    return svo, torch, dev, items


@pytest.mark.parametrize("cfg_args", [None, (128, 32, 0, 0), (128, 64, 0, 3), (96, 32, 0, 4), (64, 256, 0, 5)])
def test_noalloc_batched_cast_matches_workspace_batched_cast(mixed_batch, cfg_args):
    svo, torch, dev, items = mixed_batch
    from shocovox_gb300._lib import LaunchConfig
    lib = svo.lib()
    stream = torch.cuda.current_stream().cuda_stream
    cfg = LaunchConfig(*cfg_args) if cfg_args else None
    ns = [it[2] for it in items]

    # reference results through the existing workspace entry point
    ref = [_outputs(torch, svo, n, dev, FIELDS) for n in ns]
    _workspace_cast(svo, lib, [(s, r, n, o, row) for (s, r, n, row), o in zip(items, ref)], cfg, stream)

    # two allocation-free calls in a row into fresh outputs each time
    for call in range(2):
        got = [_outputs(torch, svo, n, dev, FIELDS) for n in ns]
        arr = _items(svo, [(s, r, n, o, row) for (s, r, n, row), o in zip(items, got)])
        rc = lib.svo_cast_batched_noalloc(arr, len(ns), ctypes.byref(cfg) if cfg is not None else None,
                                          ctypes.c_void_p(stream))
        assert rc == 0, lib.svo_last_error()
        torch.cuda.synchronize()
        for j, n in enumerate(ns):
            _assert_same(got[j], ref[j], n, (cfg_args, call, j))
        assert int((got[1]["status"][:ns[1]] == 1).sum()) > 0


def test_noalloc_counters_match_workspace_counters(mixed_batch):
    """Counter outputs select the instrumented kernel; its counters equal the workspace cast's."""
    svo, torch, dev, items = mixed_batch
    from shocovox_gb300._lib import LaunchConfig
    lib = svo.lib()
    stream = torch.cuda.current_stream().cuda_stream
    cfg = LaunchConfig(128, 32, 0, 3)
    fields = FIELDS + COUNTERS
    ns = [it[2] for it in items]
    ref = [_outputs(torch, svo, n, dev, fields) for n in ns]
    _workspace_cast(svo, lib, [(s, r, n, o, row) for (s, r, n, row), o in zip(items, ref)], cfg, stream)
    for call in range(2):
        got = [_outputs(torch, svo, n, dev, fields) for n in ns]
        arr = _items(svo, [(s, r, n, o, row) for (s, r, n, row), o in zip(items, got)])
        assert lib.svo_cast_batched_noalloc(arr, len(ns), ctypes.byref(cfg), ctypes.c_void_p(stream)) == 0, \
            lib.svo_last_error()
        torch.cuda.synchronize()
        for j, n in enumerate(ns):
            _assert_same(got[j], ref[j], n, ("counters", call, j))
    assert sum(int(g["node_visits"][:n].to(torch.int64).sum()) for g, n in zip(got, ns)) > 0


def test_noalloc_full_item_table(mixed_batch):
    """128 items, the most one call accepts: every item a slice of one scene's rays."""
    svo, torch, dev, items = mixed_batch
    from shocovox_gb300._lib import LaunchConfig
    lib = svo.lib()
    stream = torch.cuda.current_stream().cuda_stream
    scene, rays, n, _ = items[1]
    per = n // 128
    assert per > 0
    ref = _outputs(torch, svo, n, dev, FIELDS)
    got = _outputs(torch, svo, n, dev, FIELDS)

    def sliced(out):
        return [(scene, {k: v[i * per:(i + 1) * per] for k, v in rays.items()}, per,
                 {k: v[i * per:(i + 1) * per] for k, v in out.items()}, 0) for i in range(128)]
    cfg = LaunchConfig(128, 32, 0, 0)
    _workspace_cast(svo, lib, sliced(ref), cfg, stream)
    for call in range(2):
        got = _outputs(torch, svo, n, dev, FIELDS)
        arr = _items(svo, sliced(got))
        assert lib.svo_cast_batched_noalloc(arr, 128, ctypes.byref(cfg), ctypes.c_void_p(stream)) == 0, \
            lib.svo_last_error()
        torch.cuda.synchronize()
        _assert_same(got, ref, 128 * per, ("128 items", call))


def test_noalloc_refuses_a_capturing_stream(mixed_batch):
    """The item table is copied from the call's stack frame, which a graph replay could not read again."""
    svo, torch, dev, items = mixed_batch
    lib = svo.lib()
    scene, rays, n, _ = items[0]
    out = _outputs(torch, svo, n, dev, FIELDS)
    arr = _items(svo, [(scene, rays, n, out, 0)])
    side = torch.cuda.Stream(dev)
    graph = torch.cuda.CUDAGraph()
    x = torch.zeros(4, device=dev)
    torch.cuda.synchronize()
    with torch.cuda.graph(graph, stream=side):
        x.add_(1.0)  # the graph is not empty
        rc = lib.svo_cast_batched_noalloc(arr, 1, None, ctypes.c_void_p(side.cuda_stream))
    assert rc == 6, rc  # SVO_ERR_ARGUMENT
    assert b"capturing" in lib.svo_last_error()
    graph.replay()
    torch.cuda.synchronize()
    assert float(x[0]) == 1.0
    assert int(out["status"].sum()) == 0  # nothing was enqueued


def test_noalloc_rejects_more_items_than_its_scratch_holds():
    import shocovox_gb300 as svo
    from shocovox_gb300._lib import BatchItem, LaunchConfig
    arr = (BatchItem * 129)()
    rc = svo.lib().svo_cast_batched_noalloc(arr, 129, ctypes.byref(LaunchConfig()), None)
    assert rc == 6  # SVO_ERR_ARGUMENT
    assert b"exceed the maximum of 128" in svo.lib().svo_last_error()
