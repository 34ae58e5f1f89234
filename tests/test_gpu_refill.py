"""GPU parity of the refilling cast (svo_set_refill): a warp parks its rays at a node visit once fewer
than T of them are in flight, gives its idle lanes new rays and resumes.  Parking changes when a
ray's steps run, not which: hits and counters must be the oracle's for every threshold, with and
without staged top levels, for rays in no particular order, camera rows, deep sparse trees and rays
that reach the work cap."""
import numpy as np
import pytest

import shocovox_gb300 as svo
from test_gpu_cast import assert_same_hits, both, random_rays

pytestmark = pytest.mark.gpu
THRESHOLDS = (1, 8, 16, 32)
UNCOUNTED = [f for f in svo.HIT_FIELDS if f not in ("node_visits", "child_reads", "voxel_reads", "run_visits")]


@pytest.fixture
def knobs():
    lib = svo.lib()
    yield lambda refill, depth=0: (svo.check(lib.svo_set_refill(refill)), svo.check(lib.svo_set_staging_depth(depth)))
    lib.svo_set_refill(0)
    lib.svo_set_staging_depth(0)


@pytest.mark.parametrize("kind,size,dim", [(2, 512, 8), (0, 128, 4), (3, 64, 1)])
def test_refill_matches_oracle(oracle_mod, knobs, kind, size, dim):
    ops = svo.gen_scene(kind, size, dim, seed=70 + kind, occupancy=0.06, spheres=4, octaves=2, base_freq=1.0 / 16,
                        height_lo=2.0, height_hi=size * 0.35)
    o, p = both(oracle_mod, size, dim, ops)
    rng = np.random.default_rng(kind)
    origins, dirs = svo.gen_sphere_rays([size / 2] * 3, size * np.sqrt(3.0) / 2, 60_000, 5 + kind)
    ro, rd = random_rays(rng, size, 20_000)
    origins, dirs = np.concatenate([origins, ro]), np.concatenate([dirs, rd])
    ref = o.cast(origins, dirs)
    for t in THRESHOLDS:
        for depth in (0, 3):
            knobs(t, depth)
            assert_same_hits(p.cast_host(origins, dirs), ref, counters=True, label="refill %d depth %d" % (t, depth))
            assert_same_hits(p.cast_host(origins, dirs, fields=UNCOUNTED), ref, label="refill %d uncounted" % t)


def test_refill_camera_rows(oracle_mod, knobs):
    ops = svo.gen_scene(1, 256, 8, seed=77, octaves=3, base_freq=1.0 / 64, height_lo=5.0, height_hi=80.0)
    o, p = both(oracle_mod, 256, 8, ops)
    cam_o, cam_d = svo.gen_camera_rays([40.0, 120.0, 30.0], [200.0, 20.0, 180.0], 70.0, 320, 200)
    ref = o.cast(cam_o, cam_d)
    for t in THRESHOLDS:
        knobs(t)
        assert_same_hits(p.cast_host(cam_o, cam_d, fields=UNCOUNTED, row_length=320), ref, label="rows refill %d" % t)
        assert_same_hits(p.cast_host(cam_o, cam_d, row_length=320), ref, counters=True, label="rows counted %d" % t)


def test_refill_deep_sparse_tree(oracle_mod, knobs):
    from helpers import COMPLEX, INSERT, ops_from
    rng = np.random.default_rng(8)
    recs = [(INSERT, int(x), int(y), int(z), COMPLEX, 0x11223344 + i, 9 + i)
            for i, (x, y, z) in enumerate(rng.integers(0, 4096, (200, 3)))]
    o, p = both(oracle_mod, 4096, 2, ops_from(recs))
    origins, dirs = random_rays(rng, 4096, 40_000, inside_frac=0.7)
    ref = o.cast(origins, dirs)
    for t in THRESHOLDS:
        knobs(t, 4)
        assert_same_hits(p.cast_host(origins, dirs), ref, counters=True, label="deep refill %d" % t)


def test_refill_is_checked():
    assert svo.lib().svo_set_refill(33) == 6
    assert svo.lib().svo_set_refill(-1) == 6
    assert svo.lib().svo_set_refill(0) == 0


@pytest.mark.parametrize("n_items", [1, 4])
@pytest.mark.parametrize("refill", [8, 24, 32])
def test_sorted_batched_cast_with_refill(oracle_mod, n_items, refill):
    """svo_launch_config.refill_below on the ray sort's cast: one sorted item (its views in the kernel
    parameters) and several, staged top levels or not, counters included."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    tmap = {np.uint8: torch.uint8, np.uint32: torch.int32, np.float32: torch.float32}
    rng = np.random.default_rng(40 + n_items)
    items, refs, outs = [], [], []
    for j, (kind, size, dim) in enumerate([(2, 512, 8), (3, 128, 2), (0, 128, 4), (1, 64, 8)][:n_items]):
        ops = svo.gen_scene(kind, size, dim, seed=90 + j, occupancy=0.06, spheres=3, octaves=2, base_freq=1.0 / 16,
                            height_lo=2.0, height_hi=size * 0.35)
        o, p = both(oracle_mod, size, dim, ops)
        so, sd = svo.gen_sphere_rays([size / 2] * 3, size * np.sqrt(3.0) / 2, 40_000, 3 + j)
        ro, rd = random_rays(rng, size, 4_000)
        a, b = np.concatenate([so, ro]), np.concatenate([sd, rd])
        refs.append(o.cast(a, b))
        r = {k: torch.from_numpy(np.ascontiguousarray(arr[:, i])).to(dev)
             for arr, ks in ((a, ("ox", "oy", "oz")), (b, ("dx", "dy", "dz"))) for i, k in enumerate(ks)}
        out = {k: torch.zeros(len(a), dtype=tmap[t], device=dev) for k, t in svo.HIT_FIELDS.items()}
        outs.append((out, r, len(a)))
        items.append((p, {k: v.data_ptr() for k, v in r.items()}, len(a), {k: v.data_ptr() for k, v in out.items()}, 0))
    ws = svo.BatchWorkspace()
    for depth in (0, 2):
        ws.cast(items, svo.LaunchConfig(128, 32, 0, 0, 1, depth, refill), 0)
        torch.cuda.synchronize()
        for j, ((out, _, n), ref) in enumerate(zip(outs, refs)):
            got = {k: v[:n].cpu().numpy().view(svo.HIT_FIELDS[k]) for k, v in out.items()}
            assert_same_hits(got, ref, counters=True, label="item %d refill %d depth %d" % (j, refill, depth))


def test_batched_refill_is_checked():
    p = svo.Octree(64, 4)
    p.insert((1, 1, 1), albedo=0xFF)
    p.upload()
    with pytest.raises(RuntimeError):
        svo.BatchWorkspace().cast([(p, {k: 0 for k in ("ox", "oy", "oz", "dx", "dy", "dz")}, 0, {}, 0)],
                                  svo.LaunchConfig(128, 32, 0, 0, 1, 0, 33), 0)
