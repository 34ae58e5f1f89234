"""Closed-form restart runs (shocovox_gb300/csrc/svo_restart.h) against one addition at a time.

get_by_ray restarts from the root with the point moved by direction * 0.1
(src/raytracing/raytracing_on_cpu.rs:548-562); the device cast takes runs of
restarts whose root test fails in closed form.  The check program compiles the
same header for the host and compares run lengths and end points bit for bit over
random points, steps (ties, binade edges, tiny and zero steps) and run limits.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_restart_runs_match_additions(tmp_path):
    exe = str(tmp_path / "restart_run_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                    os.path.join(HERE, "restart_run_check.cpp")], check=True)
    r = subprocess.run([exe, "60000"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("OK")
