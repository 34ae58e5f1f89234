"""The serving loop: results equal single casts alone and in a mix; budget eviction; timeouts and bad ids."""
import numpy as np
import pytest

import shocovox_gb300 as svo

pytestmark = pytest.mark.gpu

FIELDS = ("status", "entry_kind", "node_key", "voxel_index", "albedo", "user", "px", "py", "pz", "nx", "ny", "nz")


SCENES = [(0, 64, 4), (3, 128, 8), (1, 64, 2)]


def scene_ops(j):
    kind, size, dim = SCENES[j]
    return svo.gen_scene(kind, size, dim, seed=500 + j, occupancy=0.1, spheres=3, octaves=2, base_freq=1.0 / 16,
                         height_lo=2.0, height_hi=size * 0.35)


def scenes():
    out = []
    for j, (_, size, dim) in enumerate(SCENES):
        t = svo.Octree(size, dim)
        t.apply_ops(scene_ops(j))
        out.append(t)
    return out


def requests(sc, rng, n):
    reqs = []
    for i in range(n):
        j = int(rng.integers(0, len(sc)))
        S = float(sc[j].size)
        a = rng.uniform(0, 2 * np.pi)
        eye = [S / 2 + 1.5 * S * np.cos(a), 1.1 * S, S / 2 + 1.5 * S * np.sin(a)]
        w, h = [(32, 24), (64, 48), (160, 120), (7, 5)][i % 4]
        reqs.append((j, eye, [S / 2, S / 3, S / 2], 60.0, w, h))
    return reqs


def out_arrays(w, h):
    return {k: np.zeros(w * h, dtype=svo.HIT_FIELDS[k]) for k in FIELDS}


def expected(sc, req):
    j, eye, target, fov, w, h = req
    o, d = svo.gen_camera_rays(eye, target, fov, w, h)
    sc[j].upload()
    return sc[j].cast_host(o, d, fields=FIELDS)


def same(a, b):
    for k in FIELDS:
        assert np.array_equal(a[k], b[k]), k


def test_server_results_are_the_same_alone_and_in_the_mix():
    sc = scenes()
    reqs = requests(sc, np.random.default_rng(1), 24)
    ref = [expected(sc, r) for r in reqs]
    srv = svo.Server(budget_bytes=1 << 34, max_batch_requests=8, max_inflight=2)
    ids = [srv.add_scene(t) for t in sc]
    assert ids == [0, 1, 2]
    # alone: one request in the server at a time
    for r, e in zip(reqs, ref):
        out = out_arrays(r[4], r[5])
        res = srv.wait(srv.submit(*r, out=out))
        assert res["batch_requests"] == 1
        same(out, e)
    # in the mix: all submitted at once, batched and overlapped by the server
    outs = [out_arrays(r[4], r[5]) for r in reqs]
    rids = [srv.submit(*r, out=o) for r, o in zip(reqs, outs)]
    results = [srv.wait(i) for i in rids]
    assert max(x["batch_requests"] for x in results) > 1
    for o, e in zip(outs, ref):
        same(o, e)
    st = srv.stats()
    assert st["requests_done"] == 48 and st["launches"] < 48
    srv.close()


def test_server_evicts_under_a_small_budget_and_stays_correct():
    sc = scenes()
    for t in sc:
        t.release_device()
    reqs = requests(sc, np.random.default_rng(2), 12)
    ref = [expected(sc, r) for r in reqs]
    for t in sc:
        t.release_device()
    srv = svo.Server(budget_bytes=1, max_batch_requests=1, max_inflight=1)
    for t in sc:
        srv.add_scene(t)
    outs = [out_arrays(r[4], r[5]) for r in reqs]
    rids = [srv.submit(*r, out=o) for r, o in zip(reqs, outs)]
    for i in rids:
        srv.wait(i)
    for o, e in zip(outs, ref):
        same(o, e)
    st = srv.stats()
    assert st["evictions"] > 0 and st["uploads"] > len(sc)
    srv.close()


def test_server_rejects_unknown_scene_and_reports_timeouts():
    sc = scenes()[:1]
    srv = svo.Server(max_inflight=1)
    srv.add_scene(sc[0])
    with pytest.raises(RuntimeError):
        srv.submit(5, [0, 0, 0], [1, 1, 1], 60.0, 4, 4, out={})
    big = out_arrays(1920, 1080)
    rid = srv.submit(0, [200.0, 90.0, 200.0], [32.0, 20.0, 32.0], 60.0, 1920, 1080, out=big)
    res = srv.wait(rid, timeout_s=0.0)  # a deadline that has already passed: not ready yet (or just done)
    if res is None:
        res = srv.wait(rid, timeout_s=60.0)
    assert res["done_s"] >= res["start_s"] >= res["submit_s"]
    with pytest.raises(RuntimeError):
        srv.wait(rid)  # a request is waited for once
    srv.close()


def test_budget_pressure_evicts_and_trims_with_the_same_results():
    """A budget of half the scene images: requests for six scenes keep evicting and uploading (in stream
    order, on the launches' streams) while launches overlap; every result equals the plain cast, and once
    the server is idle the resident images are back within the budget."""
    sc = scenes() + scenes()[:3]
    for j, t in enumerate(sc[3:]):  # three more scenes of their own
        t.insert((j + 1, j + 2, j + 3), albedo=0x10203040 + j, user=77 + j)
    images = []
    for t in sc:
        t.upload()
        images.append(t.stats()["device_bytes"])
        t.release_device()
    budget = sum(images) // 2
    reqs = requests(sc, np.random.default_rng(7), 120)
    ref = [expected(sc, r) for r in reqs]
    for t in sc:
        t.release_device()
    srv = svo.Server(budget_bytes=budget, max_batch_requests=4, max_inflight=3)
    try:
        ids = [srv.add_scene(t) for t in sc]
        outs = [out_arrays(r[4], r[5]) for r in reqs]
        rids = [srv.submit(*r, out=o) for r, o in zip(reqs, outs)]
        for rid in rids:
            srv.wait(rid, 120.0)
        for o, e in zip(outs, ref):
            same(o, e)
        st = srv.stats()
        assert st["evictions"] > 0 and st["uploads"] > len(ids)
        deadline = srv.now() + 10.0
        while srv.stats()["resident_bytes"] > budget and srv.now() < deadline:
            pass  # the trim runs as the last launches retire
        assert srv.stats()["resident_bytes"] <= budget
    finally:
        srv.close()


def test_evicted_scenes_upload_again_from_the_pinned_image_and_see_edits():
    """A budget that holds one of two scenes: each request on the other scene evicts the resident one.  An
    unchanged scene comes back from its pinned host image; a scene edited (unsynced) and then evicted, or
    edited and synced in place while resident and then evicted, comes back with the edit.  Every result
    equals the plain cast of a twin scene."""
    sc, twin = scenes(), scenes()
    image = []
    for t in sc[:2]:
        t.upload()
        image.append(t.stats()["device_bytes"])
    for t in sc + twin:
        t.release_device()
    # one scene always fits, two never do, and nothing is trimmed after a launch (the test edits and
    # syncs a resident scene while the server is idle)
    srv = svo.Server(budget_bytes=sum(image) - 1, max_batch_requests=1, max_inflight=1)
    try:
        for t in sc:
            srv.add_scene(t)
        rng = np.random.default_rng(11)
        base = requests(sc, rng, 6)
        a = next(r for r in base if r[0] == 0)
        b = next(r for r in base if r[0] == 1)

        def serve(r):
            out = out_arrays(r[4], r[5])
            srv.wait(srv.submit(*r, out=out), 60.0)
            return out

        def edit(j, k):
            S = sc[j].size
            pos, size = (S // 2, S // 4, S // 2 - 16 * k), 16
            for t in (sc[j], twin[j]):
                t.insert_at_lod(pos, size, albedo=0x11223344 + k, user=900 + k)

        first = serve(a)
        same(first, expected(twin, a))
        for _ in range(3):  # unchanged: evicted and uploaded again
            same(serve(b), expected(twin, b))
            same(serve(a), first)
        edit(0, 0)  # edited while resident, not synced; the next request evicts it
        same(serve(b), expected(twin, b))
        after = serve(a)
        same(after, expected(twin, a))
        assert not np.array_equal(after["albedo"], first["albedo"])
        edit(0, 1)  # edited and synced in place while resident
        sc[0].sync()
        synced = serve(a)
        same(synced, expected(twin, a))
        same(serve(b), expected(twin, b))
        same(serve(a), synced)  # uploaded again after the in-place sync: the pinned image was made again
        st = srv.stats()
        assert st["evictions"] >= 8 and st["uploads"] >= 10
    finally:
        srv.close()


def test_served_results_equal_the_oracle(oracle_mod):
    """Each request's rays are made on the device by the server; its results equal the oracle's cast of
    the rays that the oracle's own camera generator makes for the same request."""
    sc = scenes()
    trees = []
    for j, (_, size, dim) in enumerate(SCENES):
        o = oracle_mod.Tree(size, dim)
        o.apply_ops(scene_ops(j))
        trees.append(o)
    reqs = requests(sc, np.random.default_rng(5), 12)
    srv = svo.Server(max_batch_requests=4, max_inflight=2)
    try:
        for t in sc:
            srv.add_scene(t)
        outs = [out_arrays(r[4], r[5]) for r in reqs]
        rids = [srv.submit(*r, out=o) for r, o in zip(reqs, outs)]
        for rid in rids:
            srv.wait(rid, 60.0)
    finally:
        srv.close()
    for r, got in zip(reqs, outs):
        j, eye, target, fov, w, h = r
        o, d = oracle_mod.gen_camera_rays(eye, target, fov, w, h)
        ref = trees[j].cast(o, d)
        for k in FIELDS:
            a, b = got[k], np.asarray(ref[k])
            if a.dtype.kind == "f":
                same = (a == b) | (np.isnan(a) & np.isnan(b))
                with np.errstate(invalid="ignore"):
                    assert np.all(same | (np.abs(a.astype(np.float64) - b) <= 1e-4)), k
            else:
                assert np.array_equal(a.astype(np.uint32), b.astype(np.uint32)), k
