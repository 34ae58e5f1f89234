"""Headless counterpart of the reference's examples/cpu_render.rs: orbit a camera around a scene
and write each frame rendered by svo_render_viewport (ray generation, cast and diffuse shading in
one kernel) to a binary PPM file.

    python -m shocovox_gb300.render --size 256 --frames 4 --out frame

The scene is one of the library's seeded recipes (no .vox file is read).  The example's viewport
constants (4 x 4 units at distance 3, light normalize(0, -1, 1), grey background) are the
defaults; the orbit is centred on the scene instead of the world origin.
"""
import argparse
import time

import numpy as np

from . import Octree, gen_scene, orbit_viewport, viewport


def write_ppm(path, rgba):
    h, w, _ = rgba.shape
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(np.ascontiguousarray(rgba[..., :3]).tobytes())


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--kind", type=int, default=1, help="scene recipe (0 heightfield, 1 terrain with caves, 2 sparse "
                                                        "blocks, 3 3D noise, 4 boxes)")
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--brick-dim", type=int, default=8)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--width", type=int, default=640)
    ap.add_argument("--height", type=int, default=480)
    ap.add_argument("--frames", type=int, default=1)
    ap.add_argument("--radius", type=float, default=None, help="orbit radius (default 1.2 x size)")
    ap.add_argument("--out", default="frame", help="output prefix: <out>_<frame>.ppm")
    args = ap.parse_args(argv)

    import torch
    S = args.size
    ops = gen_scene(args.kind, S, args.brick_dim, args.seed, occupancy=0.1, spheres=8, octaves=3,
                    base_freq=1.0 / max(8, S // 4), height_lo=0.05 * S, height_hi=0.4 * S)
    tree = Octree(S, args.brick_dim)
    tree.apply_ops(ops)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    tree.upload(stream.cuda_stream)
    img = torch.empty((args.height, args.width, 4), dtype=torch.uint8, device=dev)
    bad = torch.zeros(1, dtype=torch.int64, device=dev)
    radius = args.radius if args.radius is not None else 1.2 * S
    centre = np.float32(S / 2)
    for k in range(args.frames):
        v = orbit_viewport(0.3 + k * 2 * np.pi / max(args.frames, 1), radius)
        o = np.array(list(v.origin), np.float32) + centre
        d = np.full(3, centre, np.float32) - o
        d = d / np.sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2], dtype=np.float32)
        vp = viewport(o, d)
        t0 = time.perf_counter()
        tree.render_viewport(vp, args.width, args.height, img.data_ptr(), bad.data_ptr(), stream.cuda_stream)
        frame = img.cpu().numpy()
        dt = time.perf_counter() - t0
        path = "%s_%d.ppm" % (args.out, k)
        write_ppm(path, frame)
        print("%s: %dx%d in %.2f ms (incl. copy to host), %d unshaded pixels" % (
            path, args.width, args.height, dt * 1e3, int(bad.item())))


if __name__ == "__main__":
    main()
