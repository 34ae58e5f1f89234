"""NVTX ranges: libsvo marks its phases (construction, upload, cast, batched cast, server) with NVTX
ranges, so a profiler's timeline shows them beside the kernels.  A probe tool (tests/nvtx_probe.c,
an NVTX injection library built here) records every range a child process pushes; the child builds a
scene, uploads it and casts where a GPU is present.  Runs with or without a GPU."""
import os
import shutil
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

CHILD = r"""
import numpy as np, shocovox_gb300 as svo
ops = svo.gen_scene(0, 64, 4, seed=3, spheres=2, octaves=2, base_freq=1 / 16, height_lo=2.0, height_hi=20.0)
t = svo.Octree(64, 4)
t.apply_ops(ops)
try:
    t.upload()
    o, d = svo.gen_camera_rays([90.0, 70.0, 80.0], [32.0, 10.0, 32.0], 60.0, 64, 48)
    t.cast_host(o, d, row_length=64)
    print("GPU")
except Exception as e:  # no GPU here: the upload fails after its range was pushed
    print("NOGPU", e)
"""


def _probe(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    if not cc or not os.path.isdir(os.path.join(inc, "nvtx3")):
        pytest.skip("no C compiler or NVTX headers")
    so = str(tmp_path / "libnvtx_probe.so")
    subprocess.check_call([cc, "-O1", "-shared", "-fPIC", "-I", inc, os.path.join(HERE, "nvtx_probe.c"), "-o", so])
    return so


def test_ranges_reach_an_nvtx_tool(tmp_path):
    so = _probe(tmp_path)
    log = tmp_path / "ranges.txt"
    env = dict(os.environ, NVTX_INJECTION64_PATH=so, NVTX_PROBE_OUT=str(log), PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, "-c", CHILD], env=env, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = log.read_text().splitlines()
    pushed = [ln[5:] for ln in lines if ln.startswith("push ")]
    assert "svo_apply_ops" in pushed and "svo_scene_upload" in pushed
    if r.stdout.startswith("GPU"):
        assert "svo_cast_host" in pushed
    # every range is closed, in order
    depth = 0
    for ln in lines:
        depth += 1 if ln.startswith("push ") else -1
        assert depth >= 0
    assert depth == 0


def test_no_tool_attached():
    env = {k: v for k, v in os.environ.items() if not k.startswith("NVTX_INJECTION")}
    env["PYTHONPATH"] = ROOT
    r = subprocess.run([sys.executable, "-c", CHILD], env=env, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
