"""The C-ABI library builds, loads without a GPU and exports every entry point of include/svo.h."""
import ctypes
import os
import re
import subprocess

import shocovox_gb300 as svo
from shocovox_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared_functions():
    src = open(os.path.join(ROOT, "include", "svo.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(svo_\w+)\s*\(", src)))


def test_every_declared_symbol_is_exported_and_bound():
    L = ctypes.CDLL(_lib.lib_path() if os.path.exists(_lib.lib_path()) else svo.build.build())
    names = declared_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(L, n), "libsvo does not export %s" % n
        assert n in _lib.SIGNATURES, "the Python binding does not declare %s" % n


def test_exports_via_nm():
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.lib_path()], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (svo_\w+)", out))
    assert set(declared_functions()) <= exported


def test_header_compiles_as_c():
    # the boundary is plain C: the header must compile with a C compiler and no CUDA headers
    src = '#include "svo.h"\nint main(void){ svo_scene* s = 0; (void)s; return (int)sizeof(svo_op) - 20; }\n'
    p = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-x", "c", "-",
                        "-o", "/dev/null"], input=src, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr


def test_host_entry_points_work_without_gpu():
    t = svo.Octree(16, 2)
    assert t.insert((3, 4, 5), albedo=0x11223344, user=9) == 0
    assert t.get((3, 4, 5)) == (3, 0x11223344, 9)
    st = t.stats()
    assert st["size"] == 16 and st["brick_dim"] == 2 and st["reserved_nodes"] >= 2
    assert svo.lib().svo_version() >= 100


def test_errors_cross_the_boundary_as_status_codes():
    h = ctypes.c_void_p()
    assert svo.lib().svo_scene_create(12, 4, ctypes.byref(h)) == 1
    assert b"InvalidSize" in svo.lib().svo_last_error()
    assert svo.lib().svo_scene_create(16, 2, None) == 6
    assert svo.lib().svo_insert(None, 0, 0, 0, 1, 1, 0) == 6


def test_generators_are_deterministic():
    a = svo.gen_scene(0, 32, 2, seed=3, spheres=2, octaves=2, base_freq=1 / 16, height_lo=1, height_hi=10)
    b = svo.gen_scene(0, 32, 2, seed=3, spheres=2, octaves=2, base_freq=1 / 16, height_lo=1, height_hi=10)
    assert len(a) > 100 and a.tobytes() == b.tobytes()
    o1, d1 = svo.gen_camera_rays([10, 20, 30], [0, 0, 0], 60.0, 16, 8)
    n = (d1.astype("f8") ** 2).sum(1)
    assert abs(n - 1).max() < 1e-6
    o2, d2 = svo.gen_sphere_rays([8, 8, 8], 13.0, 1000, 7)
    assert abs(((o2 - 8) ** 2).sum(1) ** 0.5 - 13).max() < 1e-3


def test_struct_layouts_match_bindings(tmp_path):
    """Every struct of svo.h has the size and field offsets of its ctypes mirror."""
    from shocovox_gb300 import _lib as L
    pairs = {"svo_rays": L.Rays, "svo_hits": L.Hits, "svo_viewport": L.Viewport, "svo_scene_stats": L.SceneStats,
             "svo_scene_recipe": L.SceneRecipe, "svo_launch_config": L.LaunchConfig,
             "svo_server_config": L.ServerConfig, "svo_request": L.Request, "svo_request_result": L.RequestResult,
             "svo_server_stats": L.ServerStats, "svo_batch_item": L.BatchItem}
    c_fields = {
        "svo_hits": [f for f, _ in L.Hits._fields_], "svo_rays": [f for f, _ in L.Rays._fields_],
        "svo_viewport": [f for f, _ in L.Viewport._fields_],
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "svo.h"', 'int main(void) {']
    for name in pairs:
        lines.append('  printf("%s %%zu\\n", sizeof(%s));' % (name, name))
    for name, fields in c_fields.items():
        for f in fields:
            lines.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (name, f, name, f))
    lines.append('  return 0;\n}')
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", INCLUDE, str(src), "-o", str(exe)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())
    for name, cls in pairs.items():
        assert int(got[name]) == ctypes.sizeof(cls), name
    for name, fields in c_fields.items():
        cls = pairs[name]
        for f in fields:
            assert int(got["%s.%s" % (name, f)]) == getattr(cls, f).offset, (name, f)


def test_process_wide_knobs_check_their_ranges():
    """The setters of the cast knobs accept their documented ranges and refuse the rest (no GPU needed:
    they only set process-wide values)."""
    lib = svo.lib()
    try:
        for mode in range(4):  # host transfer: auto, staged, in place, in place one block per warp
            assert lib.svo_set_host_transfer(mode) == 0
        assert lib.svo_set_host_transfer(4) == 6 and lib.svo_set_host_transfer(-1) == 6
        for t in (0, 1, 24, 32):
            assert lib.svo_set_refill(t) == 0
        assert lib.svo_set_refill(33) == 6 and lib.svo_set_refill(-1) == 6
        for k in range(5):
            assert lib.svo_set_staging_depth(k) == 0
        assert lib.svo_set_staging_depth(5) == 6
    finally:
        lib.svo_set_host_transfer(0)
        lib.svo_set_refill(0)
        lib.svo_set_staging_depth(0)
