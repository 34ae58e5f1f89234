"""The oracle's workload generators equal the product's bit for bit.

The benchmark's reference arm builds its scene and rays with the oracle's
generators (oracle/workloads.cpp) so that it loads no product code; its
numbers are comparable with the product's only if both make the same op lists
and the same rays.  These tests compare the two generators on every recipe kind
and on the benchmark's own workloads, and run the reference arm to check that
it loads no product code.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import shocovox_gb300 as svo

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

RECIPES = [
    (0, 128, 4, 0x5EED0001, dict(spheres=32, octaves=2, base_freq=1 / 32, height_lo=0.0, height_hi=96.0)),
    (0, 64, 2, 5, dict(spheres=0, octaves=1, base_freq=1 / 8, height_lo=1.0, height_hi=30.0)),
    (1, 128, 8, 7, dict(octaves=3, base_freq=1 / 32, height_lo=3.0, height_hi=40.0, cave_threshold=0.55)),
    (1, 64, 4, 8, dict(octaves=2, base_freq=1 / 16, height_lo=0.0, height_hi=60.0, cave_threshold=0.45)),
    (2, 256, 8, 9, dict(occupancy=0.05)),
    (2, 128, 4, 10, dict(occupancy=0.2)),
    (3, 64, 2, 11, dict(occupancy=0.12, spheres=8)),
    (3, 128, 8, 12, dict(occupancy=0.02, spheres=3, octaves=3)),
    (4, 512, 8, 13, dict(occupancy=0.03)),
    (4, 256, 4, 14, dict(occupancy=0.05)),
]


@pytest.fixture(scope="module")
def orc(oracle_mod):
    return oracle_mod


@pytest.mark.parametrize("kind,size,dim,seed,kw", RECIPES)
def test_scene_ops_equal(orc, kind, size, dim, seed, kw):
    a = svo.gen_scene(kind, size, dim, seed, **kw)
    b = orc.gen_scene(kind, size, dim, seed, **kw)
    assert len(a) > 0
    assert a.tobytes() == b.tobytes()


def test_multiscene_recipes_equal(orc):
    """The first scenes of multiscene64 at their own sizes (kind 3, noise + spheres)."""
    specs = [sp for sp in bench.multiscene_specs(bench.WORKLOADS["multiscene64"]) if sp["size"] <= 128][:6]
    assert specs
    for sp in specs:
        kw = dict(occupancy=sp["occupancy"], spheres=sp["spheres"], octaves=sp["octaves"], base_freq=sp["base_freq"])
        a = svo.gen_scene(sp["kind"], sp["size"], sp["brick_dim"], sp["seed"], **kw)
        b = orc.gen_scene(sp["kind"], sp["size"], sp["brick_dim"], sp["seed"], **kw)
        assert a.tobytes() == b.tobytes()


@pytest.mark.parametrize("workload", ["terrain512", "heightfield128", "incoherent1024"])
def test_benchmark_rays_equal(orc, workload):
    w = bench.WORKLOADS[workload]
    o1, d1 = bench.make_rays(svo, w)
    o2, d2 = bench.make_rays(orc, w)
    assert o1.tobytes() == o2.tobytes() and d1.tobytes() == d2.tobytes()


def test_terrain512_ops_equal(orc):
    """The reference arm's default scene at full size (12.56 M inserts)."""
    w = bench.WORKLOADS["terrain512"]
    a = bench.scene_ops(svo, w)
    b = bench.scene_ops(orc, w)
    assert len(a) == len(b) > 12_000_000
    assert a.tobytes() == b.tobytes()


def test_strided_camera_rays(orc):
    o, d = svo.gen_camera_rays([10.0, 200.0, -30.0], [64.0, 10.0, 64.0], 60.0, 321, 97)
    for first, stride in ((0, 1), (3, 1024), (1023, 1024), (7, 13)):
        so, sd = orc.gen_camera_rays_strided([10.0, 200.0, -30.0], [64.0, 10.0, 64.0], 60.0, 321, 97, first, stride)
        assert so.tobytes() == o[first::stride].tobytes() and sd.tobytes() == d[first::stride].tobytes()


def test_sphere_rays_equal(orc):
    for seed in (1, 0x5EED0003):
        o1, d1 = svo.gen_sphere_rays([512.0] * 3, 886.8, 50_000, seed)
        o2, d2 = orc.gen_sphere_rays([512.0] * 3, 886.8, 50_000, seed)
        assert o1.tobytes() == o2.tobytes() and d1.tobytes() == d2.tobytes()


def test_reference_arm_loads_no_product_code():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          "heightfield128", "--steps", "1", "--warmup", "0"], capture_output=True, text=True,
                         timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr
    rec = json.loads(out.stdout.strip().splitlines()[-1])
    assert rec["impl"] == "reference"
    assert rec["config"]["product_code_loaded"] is False
    assert rec["config"]["rays_per_step"] == 640 * 480  # the whole batch, the same configuration as ours
    assert rec["value"] > 0 and rec["e2e"]["value"] == rec["value"]


def test_parity_helpers():
    ref = {"status": np.array([1, 0, 1], np.uint8), "node_key": np.array([5, 0, 7], np.uint32),
           "px": np.array([1.0, np.nan, 2.0], np.float32), "albedo": np.array([9, 0, 3], np.uint32)}
    same = {k: v.copy() for k, v in ref.items()}
    r = bench.compare_hits(same, ref, "same")
    assert r["mismatches"] == 0 and r["rays_checked"] == 3
    off = {k: v.copy() for k, v in ref.items()}
    off["px"][2] += np.float32(1e-3)
    off["node_key"][0] = 6
    r = bench.compare_hits(off, ref, "off")
    assert r["mismatches"] == 2 and set(r["first_mismatch"]) == {"px", "node_key"}
    m = bench.merge_parity([bench.compare_hits(same, ref, "a"), r])
    assert m["mismatches"] == 2 and m["rays_checked"] == 6
    assert bench.parity_failed({"comparisons": {"x": {"parity": m}}})
    assert not bench.parity_failed({"parity": bench.merge_parity([bench.compare_hits(same, ref)])})
    assert bench.parity_failed({"comparisons": {"served16": {"error": "RuntimeError: x"}}})


def test_reported_figures_helpers():
    """The arithmetic behind the reported figures: repeats to median and spread, the comparison with the
    plain cast (a win counts as outside the spread only if the slowest repeat beats plain's fastest), and
    the algorithmic bytes of a cast."""
    n = 4_000_000
    plain = bench.spread(n, [1.00, 1.02, 0.98])
    assert plain["value"] == round(n / 1.00e-3 / 1e6, 3) and plain["ms_per_step"] == 1.0 and plain["repeats"] == 3
    assert plain["min"] == round(n / 1.02e-3 / 1e6, 3) and plain["max"] == round(n / 0.98e-3 / 1e6, 3)
    close = bench.spread(n, [0.97, 0.99, 0.96])  # faster median, but its slowest repeat is inside plain's spread
    v = bench.versus(close, plain)
    assert v["beats_plain"] and not v["beats_plain_outside_spread"] and v["median_ratio"] > 1
    clear = bench.spread(n, [0.90, 0.91, 0.89])
    assert bench.versus(clear, plain)["beats_plain_outside_spread"]
    assert not bench.versus(bench.spread(n, [1.1, 1.1, 1.1]), plain)["beats_plain"]
    # 12 B per performed visit, 4 B per child read and per voxel tested, 8 B per hit
    assert bench.alg_bytes_of(10, 3, 2, 1) == 120 + 12 + 8 + 8
