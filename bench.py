#!/usr/bin/env python
"""Benchmark: Mrays/s of the sparse-voxel-octree first-hit cast on one GB300.

Default workload ("terrain512", coherent primary rays at scale): a 512^3
octree with brick dimension 8 filled with a seeded 3-octave value-noise
terrain with caves (3D noise threshold 0.55, ~9.4% occupancy), 4 pinhole
cameras at 1920x1080 and 70 deg FOV at seeded positions above the terrain:
8,294,400 f32 rays per step.  A step is one cast of the whole batch.

  value  rays/s with rays and hits resident in HBM (device pointers, svo_cast)
  e2e    the same batch through the host-buffer C-ABI call svo_cast_host:
         host->device copy of the rays and device->host copy of the results
         inside the timed region

`--impl reference` times the oracle's CPU cast (a restatement of the
reference's get_by_ray; the Rust crate cannot be built here) on the host
cores over a bounded sample of the same rays.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

S_TERRAIN = 512
WORKLOADS = {
    "terrain512": dict(kind=1, size=512, brick_dim=8, seed=0x5EED0002, spheres=0, octaves=3, base_freq=1.0 / 128,
                       height_lo=0.02 * S_TERRAIN, height_hi=0.33 * S_TERRAIN, cave_threshold=0.55,
                       rays=("cameras", 4, 1920, 1080, 70.0)),
    "heightfield128": dict(kind=0, size=128, brick_dim=4, seed=0x5EED0001, spheres=32, octaves=2, base_freq=1.0 / 32,
                           height_lo=0.0, height_hi=96.0, cave_threshold=0.55, rays=("orbit", 1, 640, 480, 60.0)),
    "incoherent1024": dict(kind=2, size=1024, brick_dim=8, seed=0x5EED0003, occupancy=0.05,
                           rays=("sphere", 1 << 22)),
}
OUT_FIELDS = ("status", "entry_kind", "albedo", "user", "px", "py", "pz", "nx", "ny", "nz")
OUT_BYTES = {"status": 1, "entry_kind": 1, "albedo": 4, "user": 4, "px": 4, "py": 4, "pz": 4, "nx": 4, "ny": 4,
             "nz": 4}


def scene_ops(svo, w):
    return svo.gen_scene(w["kind"], w["size"], w["brick_dim"], w["seed"], occupancy=w.get("occupancy", 0.1),
                         spheres=w.get("spheres", 0), octaves=w.get("octaves", 2), base_freq=w.get("base_freq", 1 / 32),
                         height_lo=w.get("height_lo", 0.0), height_hi=w.get("height_hi", 0.0),
                         cave_threshold=w.get("cave_threshold", 0.55))


def make_rays(svo, w):
    spec = w["rays"]
    S = float(w["size"])
    rng = np.random.default_rng(w["seed"])
    if spec[0] == "cameras":
        _, ncam, width, height, fov = spec
        os_, ds = [], []
        for _ in range(ncam):
            eye = [rng.uniform(0.15, 0.85) * S, 0.45 * S, rng.uniform(0.15, 0.85) * S]
            target = [rng.uniform(0.1, 0.9) * S, 0.1 * S, rng.uniform(0.1, 0.9) * S]
            o, d = svo.gen_camera_rays(eye, target, fov, width, height)
            os_.append(o)
            ds.append(d)
        return np.concatenate(os_), np.concatenate(ds)
    if spec[0] == "orbit":
        _, _, width, height, fov = spec
        az, el = rng.uniform(0, 2 * np.pi), 0.5
        c = S / 2
        eye = [c + 200 * np.cos(el) * np.sin(az), c + 200 * np.sin(el), c + 200 * np.cos(el) * np.cos(az)]
        return svo.gen_camera_rays(eye, [c, c, c], fov, width, height)
    if spec[0] == "sphere":
        return svo.gen_sphere_rays([S / 2] * 3, S * np.sqrt(3.0) / 2, spec[1], w["seed"])
    raise ValueError(spec)


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(workload):
    """DRAM bytes per cast launch from the committed ncu summary of this workload, if any."""
    p = os.path.join(ROOT, "profiles", "cast_%s_traffic.json" % workload)
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f).get("dram_bytes_per_launch")
    return None


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples taken while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = str(gpu_index)
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.gpu, "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def oracle_tree_async(ops, w):
    """Builds the oracle tree in a thread (the C call releases the GIL)."""
    from oracle import oracle
    box = {}

    def run():
        t = oracle.Tree(w["size"], w["brick_dim"])
        t.apply_ops(ops)
        box["tree"] = t

    th = threading.Thread(target=run)
    th.start()
    return th, box


def cpu_cast_rate(tree, origins, dirs, target_s, threads):
    """Rays/s of the oracle cast over a strided sample sized for about target_s seconds."""
    n = len(origins)
    probe = max(1, n // 20000)
    t0 = time.perf_counter()
    tree.cast(origins[::probe], dirs[::probe], threads=threads)
    rate = len(origins[::probe]) / max(time.perf_counter() - t0, 1e-6)
    m = int(min(n, max(20000, rate * target_s)))
    step = max(1, n // m)
    so, sd = origins[::step], dirs[::step]
    t0 = time.perf_counter()
    tree.cast(so, sd, threads=threads)
    dt = time.perf_counter() - t0
    return len(so) / dt, len(so), step, dt


def batched_variants(svo, torch, scene, rp, hp, n, stream, args):
    """The persistent work-queue kernel on the same batch: a short autotune sweep, then K timed steps."""
    ws = svo.BatchWorkspace()
    items = [(scene, rp, n, hp)]
    s = stream.cuda_stream
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(cfg, reps):
        ws.cast(items, cfg, s)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            ws.cast(items, cfg, s)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    sweep = []
    for block in (64, 128, 256):
        for chunk in (32, 64, 256):
            cfg = svo.LaunchConfig(block, chunk, 0, 0)
            sweep.append(((block, chunk), timed(cfg, 2)))
    (block, chunk), _ = min(sweep, key=lambda t: t[1])
    ms = timed(svo.LaunchConfig(block, chunk, 0, 0), args.steps)
    return {"persistent_autotuned": {"value": round(n / (ms / 1e3) / 1e6, 3), "unit": "Mrays/s",
                                     "ms_per_step": round(ms, 4), "block": block, "rays_per_chunk": chunk},
            "sweep_ms": {"%dx%d" % k: round(v, 3) for k, v in sweep}}


def run_reference(args, w):
    rank, _, world = dist_env()
    if rank != 0:
        return
    import shocovox_gb300 as svo
    from oracle import oracle
    t0 = time.perf_counter()
    ops = scene_ops(svo, w)
    tree = oracle.Tree(w["size"], w["brick_dim"])
    tree.apply_ops(ops)
    origins, dirs = make_rays(svo, w)
    setup_s = time.perf_counter() - t0
    threads = os.cpu_count() or 1
    n = len(origins)
    # calibrate a per-step sample of about 2 s of CPU work
    rate, _, _, _ = cpu_cast_rate(tree, origins, dirs, 1.0, threads)
    m = int(min(n, max(10000, rate * 2.0)))
    stride = max(1, n // m)
    so, sd = np.ascontiguousarray(origins[::stride]), np.ascontiguousarray(dirs[::stride])
    for _ in range(args.warmup):
        tree.cast(so, sd, threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        tree.cast(so, sd, threads=threads)
    dt = time.perf_counter() - t0
    value = len(so) * args.steps / dt / 1e6
    sample = "every %dth ray of the %d-ray batch (%d rays per step), oracle tree built in %.1fs" % (
        stride, n, len(so), setup_s)
    print(json.dumps({
        "impl": "reference", "metric": "Mrays/s", "value": round(value, 4), "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "rays_per_step": len(so), "note": "CPU oracle cast, all host threads"},
        "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="terrain512", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-variants", action="store_true", help="skip the persistent-kernel autotune sweep")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, w)
        return

    rank, local_rank, world = dist_env()
    import torch
    import shocovox_gb300 as svo
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")  # timing reduction only; the cast itself has no collective
        pg = dist
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)

    t0 = time.perf_counter()
    ops = scene_ops(svo, w)
    want_cpu = rank == 0 and not args.no_cpu_baseline
    if want_cpu:
        oth, obox = oracle_tree_async(ops, w)
    scene = svo.Octree(w["size"], w["brick_dim"])
    scene.apply_ops(ops)
    build_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream(dev)
    scene.upload(stream.cuda_stream)
    origins, dirs = make_rays(svo, w)
    n = len(origins)
    cols_host = [np.ascontiguousarray(origins[:, i]) for i in range(3)] + [np.ascontiguousarray(dirs[:, i])
                                                                          for i in range(3)]
    rays_dev = {k: torch.from_numpy(c).to(dev) for k, c in zip(("ox", "oy", "oz", "dx", "dy", "dz"), cols_host)}
    tmap = {np.uint8: torch.uint8, np.uint32: torch.int32, np.float32: torch.float32}
    outs = {k: torch.empty(n, dtype=tmap[svo.HIT_FIELDS[k]], device=dev) for k in OUT_FIELDS}
    rp = {k: v.data_ptr() for k, v in rays_dev.items()}
    hp = {k: v.data_ptr() for k, v in outs.items()}
    s = stream.cuda_stream

    clocks = ClockSampler(local_rank)
    clocks.start()  # samples from the warm-up on, so that short timed regions still get samples
    for _ in range(args.warmup):
        scene.cast(rp, hp, n, s)
    torch.cuda.synchronize()

    # algorithmic bytes of one launch from the instrumented cast (counters equal the oracle's, see tests)
    cnt = {k: torch.empty(n, dtype=torch.int32, device=dev) for k in ("node_visits", "child_reads", "voxel_reads")}
    st = torch.empty(n, dtype=torch.uint8, device=dev)
    scene.cast(rp, dict(status=st.data_ptr(), **{k: v.data_ptr() for k, v in cnt.items()}), n, s)
    torch.cuda.synchronize()
    visits, creads, vreads = (int(cnt[k].to(torch.int64).sum()) for k in ("node_visits", "child_reads", "voxel_reads"))
    hits = int((st == 1).sum())
    alg_bytes = 12 * visits + 4 * creads + 4 * vreads + 8 * hits
    del cnt

    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        scene.cast(rp, hp, n, s)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    if pg:
        pg.barrier()
    if pg:
        t = torch.tensor([ms], dtype=torch.float64)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        ms = float(t[0])
    ms_step = ms / args.steps
    value = n * world / (ms_step / 1e3) / 1e6

    variants = None
    if not args.no_variants:
        variants = batched_variants(svo, torch, scene, rp, hp, n, stream, args)
    clk = clocks.stop()

    # end to end through the host-buffer C-ABI call (pinned host memory)
    pin_cols = [torch.from_numpy(c).pin_memory() for c in cols_host]
    pin_out = {k: torch.empty(n, dtype=tmap[svo.HIT_FIELDS[k]]).pin_memory() for k in OUT_FIELDS}
    cols_np = [c.numpy() for c in pin_cols]
    out_np = {k: v.numpy() for k, v in pin_out.items()}
    for _ in range(max(1, args.warmup)):
        scene.cast_host_soa(cols_np, out_np, s)
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        scene.cast_host_soa(cols_np, out_np, s)
    e2e_s = time.perf_counter() - t0
    if pg:
        t = torch.tensor([e2e_s], dtype=torch.float64)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        e2e_s = float(t[0])
    e2e_value = n * world * args.steps / e2e_s / 1e6

    cpu = None
    if want_cpu:
        oth.join()
        tree = obox["tree"]
        threads = os.cpu_count() or 1
        rate, m, stride, dt = cpu_cast_rate(tree, origins, dirs, args.cpu_seconds, threads)
        cpu = {"value": round(rate / 1e6, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
               "sample": "every %dth ray of the batch (%d rays, %.1fs on %d threads)" % (stride, m, dt, threads)}

    peak, peak_src = measured_peak()
    achieved = alg_bytes / (ms_step / 1e3) / 1e9
    traffic = profile_traffic(args.workload)
    if rank == 0:
        st = scene.stats()
        print(json.dumps({
            "metric": "Mrays/s", "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "octree": "%d^3" % w["size"], "brick_dim": w["brick_dim"],
                       "rays_per_step": n, "hit_rate": round(hits / n, 4), "nodes": st["nodes"],
                       "per_ray": {"node_visits": round(visits / n, 2), "child_reads": round(creads / n, 2),
                                   "voxel_reads": round(vreads / n, 2)},
                       "parted_bricks": st["parted_bricks"], "voxels_inserted": int(len(ops)),
                       "l2": "inputs larger than L2 (rays %.0f MB + hits %.0f MB per step); the %.0f MB scene image "
                             "stays resident" % (n * 24 / 1e6, n * sum(OUT_BYTES.values()) / 1e6,
                                                 st["device_bytes"] / 1e6),
                       "build_s": round(build_s, 1), "parallelism": "replicas" if world > 1 else "single"},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_src,
                         "alg_bytes_per_launch": alg_bytes,
                         "alg_bytes_per_ray": round(alg_bytes / n, 2)},
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e_value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": n * 24,
                    "d2h_bytes_per_step": n * sum(OUT_BYTES.values())},
            "gpu_launches": args.steps,
            "clocks": clk,
            "variants": variants,
        }))
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
