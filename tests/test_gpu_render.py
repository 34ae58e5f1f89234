"""GPU parity of the fused viewport render (svo_render_viewport) with the oracle's restatement of
examples/cpu_render.rs:77-138: every byte of the image and the count of unshaded pixels."""
import numpy as np
import pytest

import shocovox_gb300 as svo
from shocovox_gb300._lib import SvoError
from helpers import DATA, INSERT, ops_from
from test_gpu_cast import both
from test_oracle_render import normalized, vp_dict

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
F = np.float32


def aimed(angle, radius, centre, **kw):
    """The example's orbit camera, moved so that it circles `centre` instead of the world origin."""
    v = svo.orbit_viewport(angle, radius, **kw)
    o = np.array(list(v.origin), F) + F(centre)
    d = normalized(np.full(3, F(centre)) - o)
    return svo.viewport(o, d, up=list(v.up), width=v.width, height=v.height, fov=v.fov, light=list(v.light),
                        background=v.background)


def render_gpu(tree, vp, W, H):
    dev = torch.device("cuda", 0)
    img = torch.zeros((H, W, 4), dtype=torch.uint8, device=dev)
    bad = torch.zeros(1, dtype=torch.int64, device=dev)
    tree.render_viewport(vp, W, H, img.data_ptr(), bad.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return img.cpu().numpy(), int(bad.item())


def check(oracle_mod, size, dim, ops, vps, sizes, label):
    o, p = both(oracle_mod, size, dim, ops)
    shaded = 0
    for vp in vps:
        for W, H in sizes:
            want, want_bad = o.render_viewport(vp_dict(vp), W, H, threads=8)
            got, bad = render_gpu(p, vp, W, H)
            diff = np.nonzero(np.any(got != want, axis=-1))
            assert len(diff[0]) == 0, "%s %dx%d: %d pixels differ, first (row %d, col %d): gpu %s cpu %s" % (
                label, W, H, len(diff[0]), diff[0][0], diff[1][0], got[diff[0][0], diff[1][0]],
                want[diff[0][0], diff[1][0]])
            assert bad == want_bad, label
            shaded += int((want[..., 3] == 255).sum() - (np.all(want == [128, 128, 128, 255], axis=-1)).sum())
    assert shaded > 0, label


def test_render_heightfield_with_spheres(oracle_mod):
    ops = svo.gen_scene(0, 128, 4, seed=0x5EED0001, spheres=32, octaves=2, base_freq=1.0 / 32, height_lo=0.0,
                        height_hi=96.0)
    vps = [aimed(a, 200.0, 64.0) for a in (0.0, 1.3, 3.9)] + [svo.orbit_viewport(0.7, 150.0)]
    check(oracle_mod, 128, 4, ops, vps, [(160, 120), (97, 61)], "heightfield128")


def test_render_terrain_with_caves_and_unshaded_pixels(oracle_mod):
    ops = svo.gen_scene(1, 256, 8, seed=23, octaves=3, base_freq=1.0 / 64, height_lo=5.0, height_hi=85.0,
                        cave_threshold=0.55)
    # voxels with user data only: the example's albedo().unwrap() panics on them
    extra = ops_from([(INSERT, 100 + i, 120, 100 + j, DATA, 0, 1 + i + 8 * j) for i in range(8) for j in range(8)])
    vps = [aimed(a, 300.0, 128.0) for a in (0.4, 2.6)] + [aimed(5.0, 220.0, 128.0, fov=6.0, width=2.0, height=1.5)]
    check(oracle_mod, 256, 8, np.concatenate([ops, extra]), vps, [(128, 96)], "terrain256")


def test_render_empty_tree_is_background(oracle_mod):
    o, p = both(oracle_mod, 64, 4, ops_from([]))
    vp = aimed(1.0, 90.0, 32.0, background=0x11223344)
    got, bad = render_gpu(p, vp, 40, 24)
    assert bad == 0
    assert np.all(got == np.array([0x11, 0x22, 0x33, 0x44], np.uint8))


def test_render_rejects_bad_arguments():
    p = svo.Octree(16, 2)
    with pytest.raises(SvoError):
        p.render_viewport(svo.orbit_viewport(0.0, 30.0), 8, 8, 0)  # NULL output
    with pytest.raises(SvoError):  # not uploaded
        p.render_viewport(svo.orbit_viewport(0.0, 30.0), 8, 8, 64)


def test_several_viewports_in_one_launch_equal_single_renders(oracle_mod):
    # svo_render_viewports: frame k of one launch is svo_render_viewport's image of view k, also past 16
    # views (two launches) and with sky pixels (rays missing the root box) mixed in
    ops = svo.gen_scene(0, 128, 4, seed=0x5EED0001, spheres=8, octaves=2, base_freq=1.0 / 32, height_lo=0.0,
                        height_hi=96.0)
    o, p = both(oracle_mod, 128, 4, ops)
    vps = [aimed(0.37 * k, 160.0 + 7 * k, 64.0) for k in range(19)]
    W, H = 72, 40
    dev = torch.device("cuda", 0)
    img = torch.zeros((len(vps), H, W, 4), dtype=torch.uint8, device=dev)
    bad = torch.zeros(1, dtype=torch.int64, device=dev)
    p.render_viewports(vps, W, H, img.data_ptr(), bad.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = img.cpu().numpy()
    for k, vp in enumerate(vps):
        single, _ = render_gpu(p, vp, W, H)
        assert np.array_equal(got[k], single), k
    want, _ = o.render_viewport(vp_dict(vps[3]), W, H, threads=8)
    assert np.array_equal(got[3], want)
    # a large frame (work queue), 3 views
    W, H = 300, 200
    img = torch.zeros((3, H, W, 4), dtype=torch.uint8, device=dev)
    p.render_viewports(vps[:3], W, H, img.data_ptr(), bad.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = img.cpu().numpy()
    for k in range(3):
        want, _ = o.render_viewport(vp_dict(vps[k]), W, H, threads=8)
        assert np.array_equal(got[k], want), k
