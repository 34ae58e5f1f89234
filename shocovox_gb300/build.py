"""Builds libsvo.so in-tree (shocovox_gb300/_lib/) for sm_103a.

Host sources are compiled with g++ and -ffp-contract=off (no FMA contraction,
so construction-side f32 arithmetic rounds like the Rust reference on both
x86_64 and aarch64); the CUDA source with nvcc for sm_103a only, with
-fmad=false -prec-div=true -prec-sqrt=true -ftz=false for the same reason on
the device.  Translation units compile in parallel.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libsvo.so")

HOST_SOURCES = ["svo_octree.cpp", "svo_capi.cpp", "svo_scenes.cpp", "svo_persist.cpp", "svo_vox.cpp"]
CUDA_SOURCES = ["svo_device.cu", "svo_batch.cu", "svo_server.cu", "svo_render.cu"]
HEADERS = ["svo_octree.h", "svo_internal.h", "svo_cast.cuh", "svo_restart.h", "svo_queue.h", "svo_lod.h", "svo_trace.h",
           "svo_refill.cuh"]

CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wextra",
            "-Wno-unused-parameter"]
NVCCFLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo", "-O3", "-std=c++17",
             "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
             "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: libsvo needs the CUDA toolkit to build")


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in HOST_SOURCES + CUDA_SOURCES + HEADERS]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "svo.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_nvcc=()):
    """Compiles libsvo.so if a source is newer than it; returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    cxx = os.environ.get("CXX", "g++")
    # the host sources include the toolkit's header-only NVTX (svo_trace.h)
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    objs, procs = [], []
    for src in HOST_SOURCES:
        obj = os.path.join(OUT_DIR, src.replace(".cpp", ".o"))
        cmd = [cxx] + CXXFLAGS + ["-I", cuda_inc, "-c", os.path.join(CSRC, src), "-o", obj]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    for src in CUDA_SOURCES:
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        cmd = [nvcc] + NVCCFLAGS + list(extra_nvcc) + ["-c", os.path.join(CSRC, src), "-o", obj]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + out.decode(errors="replace"))
        if p.returncode:
            failed.append(cmd[-3])
    if failed:
        raise RuntimeError("libsvo build failed: %s" % ", ".join(failed))
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp] + objs + ["-lpthread", "-ldl"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
