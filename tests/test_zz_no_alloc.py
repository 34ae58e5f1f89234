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


def _outputs(torch, svo, n, dev):
    tmap = {np.uint8: torch.uint8, np.uint32: torch.int32, np.float32: torch.float32}
    return {k: torch.zeros(max(n, 1), dtype=tmap[svo.HIT_FIELDS[k]], device=dev) for k in FIELDS}


def _items(svo, batches):
    from shocovox_gb300._lib import BatchItem, Hits, Rays
    arr = (BatchItem * len(batches))()
    for i, (scene, rays, n, out) in enumerate(batches):
        arr[i].scene = scene.handle
        arr[i].rays = Rays(*[ctypes.c_void_p(rays[k].data_ptr()) for k in ("ox", "oy", "oz", "dx", "dy", "dz")])
        arr[i].n = n
        arr[i].hits = Hits(**{k: ctypes.c_void_p(out[k].data_ptr()) if k in out else None for k in svo.HIT_FIELDS})
    return arr


def test_noalloc_batched_cast_matches_workspace_batched_cast():
    torch = pytest.importorskip("torch")
    import shocovox_gb300 as svo
    from shocovox_gb300._lib import LaunchConfig
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(12345)
    specs = [(3, 64, 4, 3000), (0, 128, 8, 5000), (1, 64, 2, 0), (3, 32, 1, 2000)]
    scenes, rays, ns = [], [], []
    for j, (kind, size, dim, n) in enumerate(specs):
        scenes.append(_scene(svo, kind, size, dim, 900 + j))
        o, d = _rays(rng, size, n)
        rays.append({k: torch.from_numpy(np.ascontiguousarray(a[:, i]) if n else np.zeros(0, np.float32)).to(dev)
                     for a, names in ((o, ("ox", "oy", "oz")), (d, ("dx", "dy", "dz"))) for i, k in enumerate(names)})
        ns.append(n)
    lib = svo.lib()
    stream = torch.cuda.current_stream().cuda_stream
    cfg = LaunchConfig(128, 32, 0, 0)

    # reference results through the existing workspace entry point
    ref = [_outputs(torch, svo, n, dev) for n in ns]
    ws = ctypes.c_void_p()
    assert lib.svo_batch_workspace_create(ctypes.byref(ws)) == 0
    try:
        arr = _items(svo, list(zip(scenes, rays, ns, ref)))
        assert lib.svo_cast_batched(ws, arr, len(ns), ctypes.byref(cfg), ctypes.c_void_p(stream)) == 0
        torch.cuda.synchronize()
    finally:
        lib.svo_batch_workspace_destroy(ws)

    # two allocation-free calls in a row into fresh outputs each time
    for call in range(2):
        got = [_outputs(torch, svo, n, dev) for n in ns]
        arr = _items(svo, list(zip(scenes, rays, ns, got)))
        rc = lib.svo_cast_batched_noalloc(arr, len(ns), ctypes.byref(cfg), ctypes.c_void_p(stream))
        assert rc == 0, lib.svo_last_error()
        torch.cuda.synchronize()
        for j, n in enumerate(ns):
            for k in FIELDS:
                a, b = got[j][k][:n].cpu().numpy(), ref[j][k][:n].cpu().numpy()
                if a.dtype == np.float32:
                    same = (a == b) | (np.isnan(a) & np.isnan(b))
                    with np.errstate(invalid="ignore"):
                        assert np.all(same | (np.abs(a.astype(np.float64) - b) <= TOL)), (call, j, k)
                else:
                    assert np.array_equal(a, b), (call, j, k)
        assert int((got[1]["status"][:ns[1]] == 1).sum()) > 0


def test_noalloc_rejects_more_items_than_its_scratch_holds():
    import shocovox_gb300 as svo
    from shocovox_gb300._lib import BatchItem, LaunchConfig
    arr = (BatchItem * 129)()
    rc = svo.lib().svo_cast_batched_noalloc(arr, 129, ctypes.byref(LaunchConfig()), None)
    assert rc == 6  # SVO_ERR_ARGUMENT
    assert b"exceed the maximum of 128" in svo.lib().svo_last_error()
