"""The oracle's viewport render (examples/cpu_render.rs:77-138) against a numpy restatement.

The numpy side forms the example's rays in f32 with its operation order, casts them with the
oracle's get_by_ray and shades them; the oracle's own render loop must produce the same bytes.
"""
import numpy as np
import pytest

import shocovox_gb300 as svo
from helpers import ALBEDO, DATA, INSERT, ops_from

F = np.float32


def normalized(v):
    n = np.sqrt((v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1]) + v[..., 2] * v[..., 2])
    return v / n[..., None]


def reference_frame(vp, W, H):
    """cpu_render.rs:82-98 and the per-pixel ray of :106-115, in f32."""
    o = np.array(vp["origin"], F)
    d = np.array(vp["direction"], F)
    up = np.array(vp["up"], F)
    right = normalized(np.array([up[1] * d[2] - up[2] * d[1], up[2] * d[0] - up[0] * d[2],
                                 up[0] * d[1] - up[1] * d[0]], F))
    pw = F(vp["width"]) / F(W)
    ph = F(vp["height"]) / F(H)
    bl = ((o + d * F(vp["fov"])) - up * (F(vp["height"]) / F(2))) - right * (F(vp["width"]) / F(2))
    x = np.arange(W, dtype=F)[None, :, None]
    y = np.arange(H, dtype=F)[:, None, None]
    glass = (bl + (right * x) * pw) + (up * y) * ph  # (H, W, 3), indexed by the example's y
    dirs = normalized(glass - o)
    return o, dirs


def shade(hits, vp, H, W):
    light = np.array(vp["light"], F)
    img = np.zeros((H, W, 4), np.uint8)
    st = hits["status"].reshape(H, W)
    kind = hits["entry_kind"].reshape(H, W)
    alb = hits["albedo"].reshape(H, W).astype(np.uint32)
    n = np.stack([hits["nx"], hits["ny"], hits["nz"]], -1).reshape(H, W, 3)
    strength = F(1) - (((n[..., 0] * light[0] + n[..., 1] * light[1]) + n[..., 2] * light[2]) / F(2) + F(0.5))
    bg = vp["background"]
    for c, sh in enumerate((24, 16, 8)):
        v = ((alb >> sh) & 0xFF).astype(F) * strength
        with np.errstate(invalid="ignore"):
            u8 = np.where(v > 0, np.minimum(np.where(np.isnan(v), 0, v), 255), 0).astype(np.uint8)
        img[..., c] = np.where(st == 0, (bg >> sh) & 0xFF, np.where((st == 1) & (kind & 1 == 1), u8, 0))
    img[..., 3] = np.where(st == 0, bg & 0xFF, np.where((st == 1) & (kind & 1 == 1), 255, 0))
    unshaded = int(((st != 0) & ~((st == 1) & (kind & 1 == 1))).sum())
    return img[::-1], unshaded  # row 0 of the image is the example's y = H - 1


def vp_dict(v):
    return {"origin": list(v.origin), "direction": list(v.direction), "up": list(v.up), "width": v.width,
            "height": v.height, "fov": v.fov, "light": list(v.light), "background": v.background}


@pytest.mark.parametrize("angle,radius,W,H", [(0.3, 80.0, 64, 48), (2.1, 60.0, 37, 29), (4.0, 100.0, 50, 50)])
def test_oracle_render_matches_numpy_restatement(oracle_mod, angle, radius, W, H):
    ops = svo.gen_scene(0, 64, 4, seed=17, spheres=4, octaves=2, base_freq=1.0 / 16, height_lo=4.0, height_hi=40.0)
    extra = ops_from([(INSERT, 30 + i, 45, 30, DATA, 0, 7 + i) for i in range(4)])  # user data only: unshaded
    t = oracle_mod.Tree(64, 4)
    t.apply_ops(np.concatenate([ops, extra]))
    vp = vp_dict(svo.orbit_viewport(angle, radius))
    # the example looks at the world origin; aim the orbit at the scene's centre instead
    o = np.array(vp["origin"], F) + F(32)
    vp["origin"] = list(o)
    vp["direction"] = list(normalized(np.full(3, F(32)) - o))
    img, bad = t.render_viewport(vp, W, H, threads=4)
    origin, dirs = reference_frame(vp, W, H)
    hits = t.cast(np.broadcast_to(origin, (H * W, 3)), dirs.reshape(-1, 3), threads=4)
    want, want_bad = shade(hits, vp, H, W)
    assert (hits["status"] == 1).sum() > W * H // 8
    assert np.array_equal(img, want)
    assert bad == want_bad


def test_example_constants():
    v = svo.orbit_viewport(0.0, 10.0)
    assert (v.width, v.height, v.fov, v.background) == (4.0, 4.0, 3.0, 0x808080FF)
    assert list(v.up) == [0.0, 1.0, 0.0]
    assert np.allclose(list(v.light), [0.0, -0.70710677, 0.70710677])
    assert np.allclose(list(v.origin), [0.0, 10.0, 10.0])
