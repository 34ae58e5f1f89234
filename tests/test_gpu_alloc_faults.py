"""Allocation failures during upload and server admission, injected on the host.

svo_set_device_allocator routes the scene images' device memory through the caller's allocator (here
PyTorch's caching allocator).  An allocator that returns NULL on a chosen call stands in for a device
that is out of memory: the upload must report SVO_ERR_OUT_OF_MEMORY, give back everything it took and
leave the scene without a device image; a server request that needs that upload fails with the same
status while the server keeps serving; with memory back, both succeed and cast like the oracle."""
import ctypes

import numpy as np
import pytest

import shocovox_gb300 as svo
from test_gpu_cast import assert_same_hits, both, random_rays

pytestmark = pytest.mark.gpu
OUT_OF_MEMORY, NOT_UPLOADED = 9, 8
ALLOC = ctypes.CFUNCTYPE(ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p)
FREE = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_void_p)


class Allocator:
    """Device memory from torch's caching allocator; `fail_at` = the call that returns NULL (1-based)."""

    def __init__(self, torch):
        self.torch = torch
        self.live, self.calls, self.fail_at = set(), 0, None
        self._alloc, self._free = ALLOC(self.alloc), FREE(self.free)  # kept alive while installed

    def alloc(self, nbytes, stream, user):
        self.calls += 1
        if self.fail_at is not None and self.calls >= self.fail_at:
            return None
        p = self.torch.cuda.caching_allocator_alloc(max(int(nbytes), 256))
        self.live.add(p)
        return p

    def free(self, ptr, user):
        self.live.discard(ptr)
        self.torch.cuda.caching_allocator_delete(ptr)

    def install(self):
        svo.check(svo.lib().svo_set_device_allocator(ctypes.cast(self._alloc, ctypes.c_void_p),
                                                     ctypes.cast(self._free, ctypes.c_void_p), None))


@pytest.fixture
def allocator():
    torch = pytest.importorskip("torch")
    torch.cuda.init()
    a = Allocator(torch)
    a.install()
    yield a
    svo.check(svo.lib().svo_set_device_allocator(None, None, None))


def test_upload_through_the_callers_allocator(oracle_mod, allocator):
    ops = svo.gen_scene(0, 64, 4, seed=5, spheres=3, octaves=2, base_freq=1 / 16, height_lo=2.0, height_hi=24.0)
    o, p = both(oracle_mod, 64, 4, ops)
    assert allocator.calls == 6 and len(allocator.live) == 6  # 5 pools + the top table
    origins, dirs = random_rays(np.random.default_rng(1), 64, 4000)
    assert_same_hits(p.cast_host(origins, dirs), o.cast(origins, dirs), counters=True, label="callers allocator")
    p.release_device()
    assert not allocator.live


@pytest.mark.parametrize("fail_at", [1, 2, 3, 4, 5, 6])
def test_upload_fails_cleanly_at_every_allocation(oracle_mod, allocator, fail_at):
    ops = svo.gen_scene(3, 64, 2, seed=7, occupancy=0.1, spheres=2)
    o = oracle_mod.Tree(64, 2)
    o.apply_ops(ops)
    p = svo.Octree(64, 2)
    p.apply_ops(ops)
    allocator.fail_at = fail_at
    assert svo.lib().svo_scene_upload(p.handle, None) == OUT_OF_MEMORY
    assert b"no memory" in svo.lib().svo_last_error()
    assert not allocator.live  # everything taken before the failure was given back
    assert p.stats()["device_bytes"] == 0
    origins, dirs = random_rays(np.random.default_rng(fail_at), 64, 1000)
    with pytest.raises(RuntimeError):
        p.cast_host(origins, dirs)  # no device image
    allocator.fail_at = None
    p.upload()
    assert_same_hits(p.cast_host(origins, dirs), o.cast(origins, dirs), counters=True, label="after recovery")


def test_server_admission_survives_an_allocation_failure(allocator):
    from shocovox_gb300 import OctreeError
    scenes = []
    for j in range(2):
        t = svo.Octree(64, 4)
        t.apply_ops(svo.gen_scene(0, 64, 4, seed=30 + j, spheres=2, octaves=2, base_freq=1 / 16, height_lo=2.0,
                                  height_hi=24.0))
        scenes.append(t)
    srv = svo.Server(budget_bytes=1 << 30, max_batch_requests=8, max_inflight=2)
    try:
        ids = [srv.add_scene(t) for t in scenes]
        w, h = 48, 32
        out = {k: np.zeros(w * h, dtype=svo.HIT_FIELDS[k]) for k in ("status", "albedo", "node_key")}
        allocator.fail_at = allocator.calls + 1  # the next upload's first allocation fails
        rid = srv.submit(ids[0], [100.0, 80.0, 90.0], [32.0, 12.0, 32.0], 60.0, w, h, out=out)
        with pytest.raises(OctreeError) as e:
            srv.wait(rid, 60.0)
        assert e.value.code == OUT_OF_MEMORY
        assert not allocator.live
        allocator.fail_at = None  # memory is back: the server goes on serving
        for j in ids:
            got = {k: np.zeros(w * h, dtype=svo.HIT_FIELDS[k]) for k in out}
            srv.wait(srv.submit(j, [100.0, 80.0, 90.0], [32.0, 12.0, 32.0], 60.0, w, h, out=got), 60.0)
            origins, dirs = svo.gen_camera_rays([100.0, 80.0, 90.0], [32.0, 12.0, 32.0], 60.0, w, h)
            scenes[j].upload()
            ref = scenes[j].cast_host(origins, dirs, fields=list(out), row_length=w)
            for k in out:
                assert np.array_equal(got[k], ref[k]), (j, k)
            assert int((got["status"] == 1).sum()) > 0
    finally:
        srv.close()
        for t in scenes:
            t.release_device()
    assert not allocator.live
