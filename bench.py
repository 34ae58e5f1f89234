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
    "multiscene64": dict(multi=64, seed=0x5EED0004),
    "served16": dict(served=16, seed=0x5EED0005, rate=2000.0, requests=600, budget_gb=60.0),
    # terrain512 with MIP maps, cast through get_by_ray_at_lod at a viewing distance of 256
    "lod512": dict(lod=256.0, kind=1, size=512, brick_dim=8, seed=0x5EED0002, spheres=0, octaves=3,
                   base_freq=1.0 / 128, height_lo=0.02 * S_TERRAIN, height_hi=0.33 * S_TERRAIN, cave_threshold=0.55,
                   rays=("cameras", 4, 1920, 1080, 70.0)),
    # the terrain512 scene seen through examples/cpu_render.rs's viewport: fused ray generation + cast + shading
    "viewport512": dict(viewport=4, kind=1, size=512, brick_dim=8, seed=0x5EED0002, spheres=0, octaves=3,
                        base_freq=1.0 / 128, height_lo=0.02 * S_TERRAIN, height_hi=0.33 * S_TERRAIN,
                        cave_threshold=0.55, width=1920, height=1080),
}
RESOLUTIONS = [(320, 240), (640, 480), (1280, 720), (1920, 1080), (3840, 2160)]
OUT_FIELDS = ("status", "entry_kind", "albedo", "user", "px", "py", "pz", "nx", "ny", "nz")
COUNTERS = ("node_visits", "child_reads", "voxel_reads", "run_visits")
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


def ray_rows(w):
    """Row length of the workload's rays when they are camera images in raster order, else 0."""
    spec = w.get("rays", ())
    return spec[2] if spec and spec[0] in ("cameras", "orbit") else 0


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(workload):
    """The committed ncu summary of this workload's cast launch (DRAM and L2 bytes per launch), if any."""
    p = os.path.join(ROOT, "profiles", "cast_%s_traffic.json" % workload)
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples taken while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index, interval_ms=200):
        self.gpu = str(gpu_index)
        self.interval_ms = str(interval_ms)
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.gpu, "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", self.interval_ms],
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


def alg_bytes_of(performed_visits, child_reads, voxel_reads, hits):
    """Algorithmic bytes of a cast: 12 B (occupancy bits + node kind) per node visit the cast performs,
    4 B per child key read, 4 B per voxel tested, 8 B (albedo + user) per hit.  Restart visits that the
    cast counts in closed form read nothing and are left out (performed = node_visits - run_visits)."""
    return 12 * performed_visits + 4 * child_reads + 4 * voxel_reads + 8 * hits


def max_over_ranks(seconds, pg):
    """The slowest rank's time: the job is done when the last replica is (gloo all-reduce on the host)."""
    if pg is None:
        return seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t[0])


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


def cpu_cast_rate(tree, origins, dirs, target_s, threads, **cast_args):
    """Rays/s of the oracle cast over a strided sample sized for about target_s seconds."""
    n = len(origins)
    probe = max(1, n // 20000)
    t0 = time.perf_counter()
    tree.cast(origins[::probe], dirs[::probe], threads=threads, **cast_args)
    rate = len(origins[::probe]) / max(time.perf_counter() - t0, 1e-6)
    m = int(min(n, max(20000, rate * target_s)))
    step = max(1, n // m)
    so, sd = origins[::step], dirs[::step]
    t0 = time.perf_counter()
    tree.cast(so, sd, threads=threads, **cast_args)
    dt = time.perf_counter() - t0
    reps = 1
    # a whole batch that takes the CPU less than the target is cast again until the target is reached
    if step == 1 and dt < target_s:
        more = int(min(1000, target_s / max(dt, 1e-6)))
        t0 = time.perf_counter()
        for _ in range(more):
            tree.cast(so, sd, threads=threads, **cast_args)
        dt, reps = time.perf_counter() - t0, more
    return reps * len(so) / dt, reps * len(so), step, dt


def batched_variants(svo, torch, scene, rp, hp, n, stream, args, row=0):
    """The persistent work-queue kernel on the same batch: a short autotune sweep, then K timed steps."""
    ws = svo.BatchWorkspace()
    items = [(scene, rp, n, hp, row)]
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
    for block in (64, 96, 128):
        for chunk in (32, 64, 256):
            for shape in ((3, 4) if row else (0,)):
                for sort in ((0,) if row else (0, 1)):
                    cfg = svo.LaunchConfig(block, chunk, 0, shape, sort)
                    sweep.append(((block, chunk, shape, sort), timed(cfg, 2)))
    (block, chunk, shape, sort), _ = min(sweep, key=lambda t: t[1])
    ms = timed(svo.LaunchConfig(block, chunk, 0, shape, sort), args.steps)
    out = {"persistent_autotuned": {"value": round(n / (ms / 1e3) / 1e6, 3), "unit": "Mrays/s",
                                    "ms_per_step": round(ms, 4), "block": block, "rays_per_chunk": chunk,
                                    "block_shape": shape, "sort_key": sort,
                                    "launches_per_step": batched_launches(items, sort)},
           "sweep_ms": {"%dx%dx%dx%d" % k: round(v, 3) for k, v in sweep}}
    if not row:
        # the best of each ray order, timed over K steps
        for so in (0, 1):
            (b, c, sh, _), _ = min((t for t in sweep if t[0][3] == so), key=lambda t: t[1])
            ms = timed(svo.LaunchConfig(b, c, 0, sh, so), args.steps)
            out["persistent_sort%d" % so] = {"value": round(n / (ms / 1e3) / 1e6, 3), "unit": "Mrays/s",
                                             "ms_per_step": round(ms, 4), "block": b, "rays_per_chunk": c}
    return out


def batched_launches(items, sort_key):
    """Kernel launches of one svo_cast_batched call: the claim-order cast if any item is cast in claim
    order, plus the ray sort's bin, three scan, scatter and cast launches if any item is sorted."""
    sorted_items = [it for it in items if sort_key and not (len(it) > 4 and it[4]) and it[2]]
    claimed = [it for it in items if it[2] and it not in sorted_items]
    return (1 if claimed else 0) + (6 if sorted_items else 0)


def multiscene_specs(w):
    """64 scenes: size from {64..512}^3, brick dim from {2,4,8}, occupancy 2-20%, noise + spheres,
    a log-uniform 1K-1M ray batch each (half camera rays, half random directions)."""
    rng = np.random.default_rng(w["seed"])
    specs = []
    for i in range(w["multi"]):
        size = int(rng.choice([64, 128, 256, 512]))
        dim = int(rng.choice([2, 4, 8]))
        occ = float(rng.uniform(0.02, 0.20))
        nrays = int(np.exp(rng.uniform(np.log(1e3), np.log(1e6))))
        specs.append(dict(kind=3, size=size, brick_dim=dim, seed=w["seed"] + 17 * i, occupancy=occ, spheres=8,
                          octaves=2, base_freq=1.0 / 32, nrays=nrays, eye_angle=float(rng.uniform(0, 2 * np.pi))))
    return specs


def multiscene_rays(svo, sp):
    S = float(sp["size"])
    n = sp["nrays"]
    ncam = n // 2
    w_ = max(1, int(np.ceil(np.sqrt(ncam * 16 / 9))))
    h_ = max(1, int(np.ceil(ncam / w_)))
    a = sp["eye_angle"]
    eye = [S / 2 + 1.6 * S * np.cos(a), 1.2 * S, S / 2 + 1.6 * S * np.sin(a)]
    o1, d1 = svo.gen_camera_rays(eye, [S / 2, S / 3, S / 2], 60.0, w_, h_)
    o2, d2 = svo.gen_sphere_rays([S / 2] * 3, S * np.sqrt(3.0) / 2, n - ncam, sp["seed"])
    # the camera rays are rows of w_ rays in raster order (the last row cut short)
    return np.concatenate([o1[:ncam], o2]), np.concatenate([d1[:ncam], d2]), ncam, w_


def run_multiscene(args, w):
    """Batched multi-scene cast: serial plain dispatch vs one persistent launch vs that launch in a CUDA graph."""
    import concurrent.futures as cf
    import torch
    import shocovox_gb300 as svo
    from shocovox_gb300 import autotune
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    specs = multiscene_specs(w)
    t0 = time.perf_counter()

    def build(sp):
        ops = svo.gen_scene(sp["kind"], sp["size"], sp["brick_dim"], sp["seed"], occupancy=sp["occupancy"],
                            spheres=sp["spheres"], octaves=sp["octaves"], base_freq=sp["base_freq"])
        t = svo.Octree(sp["size"], sp["brick_dim"])
        t.apply_ops(ops)
        return t, len(ops)

    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        built = list(ex.map(build, specs))
    build_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream(dev)
    s = stream.cuda_stream
    tmap = {np.uint8: torch.uint8, np.uint32: torch.int32, np.float32: torch.float32}
    # one batch: every ray column and hit field is one buffer over all scenes, each scene a slice
    ray_keys = ("ox", "oy", "oz", "dx", "dy", "dz")
    host_rays = [multiscene_rays(svo, sp) for sp in specs]
    counts = [len(r[0]) for r in host_rays]
    begins = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    total = int(begins[-1])
    all_o = np.concatenate([r[0] for r in host_rays])
    all_d = np.concatenate([r[1] for r in host_rays])
    host_cols = [np.ascontiguousarray(all_o[:, i]) for i in range(3)] + [np.ascontiguousarray(all_d[:, i]) for i in range(3)]
    dev_cols = {k: torch.from_numpy(c).to(dev) for k, c in zip(ray_keys, host_cols)}
    dev_out = {k: torch.empty(total, dtype=tmap[svo.HIT_FIELDS[k]], device=dev) for k in OUT_FIELDS}
    # per scene two items: its camera rays (rows of the image: cast in 8 x 4 ray blocks) and its
    # random rays
    scenes, items, outs = [], [], []
    for i, (t, _) in enumerate(built):
        t.upload(s)
        a, b = int(begins[i]), int(begins[i + 1])
        scenes.append(t)
        outs.append({k: v[a:b] for k, v in dev_out.items()})
        ncam, row = host_rays[i][2], host_rays[i][3]
        for lo, hi, r in ((a, a + ncam, row), (a + ncam, b, 0)):
            if hi > lo:
                rays = {k: v[lo:hi] for k, v in dev_cols.items()}
                out = {k: v[lo:hi] for k, v in dev_out.items()}
                items.append((t, {k: v.data_ptr() for k, v in rays.items()}, hi - lo,
                              {k: v.data_ptr() for k, v in out.items()}, r))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    def serial():
        for (t, rp, n, hp, row) in items:
            t.cast(rp, hp, n, s, row_length=row)

    ws = svo.BatchWorkspace()
    bitems = items
    cfg, tune_info = autotune.tune(ws, bitems, torch.cuda.get_device_name(0),
                                   lambda c: timed(lambda: ws.cast(bitems, c, s), 2))

    def batched():
        ws.cast(bitems, cfg, s)

    clocks = ClockSampler(0)
    clocks.start()
    for _ in range(args.warmup):
        serial()
        batched()
    torch.cuda.synchronize()
    serial_ms = timed(serial, args.steps)
    ref_out = [{k: v.clone() for k, v in out.items()} for out in outs]
    batched_ms = timed(batched, args.steps)
    same = all(torch.equal(a[k], b[k]) for a, b in zip(ref_out, outs) for k in OUT_FIELDS)
    # one persistent launch captured in a CUDA graph (workspace already sized, blocks per SM fixed)
    if cfg.blocks_per_sm == 0:
        per_sm = {64: 14, 96: 9, 128: 7}.get(cfg.block, 2)  # resident blocks at 72 registers per thread
        gcfg = svo.LaunchConfig(cfg.block, cfg.rays_per_chunk, per_sm, cfg.block_shape, cfg.sort_key)
    else:
        gcfg = cfg
    gstream = torch.cuda.Stream(dev)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(gstream):
        ws.cast(bitems, gcfg, gstream.cuda_stream)
        torch.cuda.synchronize()
        with torch.cuda.graph(graph, stream=gstream):
            ws.cast(bitems, gcfg, gstream.cuda_stream)
    torch.cuda.synchronize()
    graph_ms = timed(graph.replay, args.steps)
    clk = clocks.stop()

    # algorithmic bytes of the batch, from the instrumented batched cast
    cnt = [dict(status=torch.zeros(n, dtype=torch.uint8, device=dev),
                **{k: torch.zeros(n, dtype=torch.int32, device=dev) for k in COUNTERS})
           for (_, _, n, _, _) in items]
    citems = [(t, rp, n, {k: v.data_ptr() for k, v in c.items()}, row) for (t, rp, n, _, row), c in zip(items, cnt)]
    ws.cast(citems, cfg, s)
    torch.cuda.synchronize()
    sums = {k: sum(int(c[k].to(torch.int64).sum()) for c in cnt) for k in COUNTERS}
    hits = sum(int((c["status"] == 1).sum()) for c in cnt)
    alg = alg_bytes_of(sums["node_visits"] - sums["run_visits"], sums["child_reads"], sums["voxel_reads"], hits)

    # end to end: host rays in, one batched launch, host hits out (pinned buffers, copies in the timed region;
    # one copy per ray column and per hit field of the whole batch)
    pin_in = {k: torch.from_numpy(c).pin_memory() for k, c in zip(ray_keys, host_cols)}
    pin_out = {k: torch.empty(total, dtype=tmap[svo.HIT_FIELDS[k]]).pin_memory() for k in OUT_FIELDS}

    def e2e():
        for k in ray_keys:
            dev_cols[k].copy_(pin_in[k], non_blocking=True)
        ws.cast(bitems, cfg, s)
        for k in OUT_FIELDS:
            pin_out[k].copy_(dev_out[k], non_blocking=True)

    e2e()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(args.steps):
        e2e()
    torch.cuda.synchronize()
    e2e_serial_s = (time.perf_counter() - t1) / args.steps
    serial_hits = {k: v.clone() for k, v in pin_out.items()}

    # the same with the batch cut into 4 groups of consecutive items, each on its own stream with its
    # own workspace: one group's copies overlap another group's launch
    base = dev_cols["ox"].data_ptr()
    offs = [(it[1]["ox"] - base) // 4 for it in bitems]
    n_groups, groups, cur_g, acc = 4, [], [], 0
    for it, off in zip(bitems, offs):
        cur_g.append((it, off))
        acc += it[2]
        if len(groups) < n_groups - 1 and acc >= total * (len(groups) + 1) / n_groups:
            groups.append(cur_g)
            cur_g = []
    if cur_g:
        groups.append(cur_g)
    g_ranges = [(g[0][1], g[-1][1] + g[-1][0][2]) for g in groups]
    g_streams = [torch.cuda.Stream(dev) for _ in groups]
    g_ws = [svo.BatchWorkspace() for _ in groups]
    g_start = torch.cuda.Event()

    def e2e_groups():
        g_start.record(stream)
        for g, (lo, hi), st, wsg in zip(groups, g_ranges, g_streams, g_ws):
            st.wait_event(g_start)
            with torch.cuda.stream(st):
                for k in ray_keys:
                    dev_cols[k][lo:hi].copy_(pin_in[k][lo:hi], non_blocking=True)
                wsg.cast([it for it, _ in g], cfg, st.cuda_stream)
                for k in OUT_FIELDS:
                    pin_out[k][lo:hi].copy_(dev_out[k][lo:hi], non_blocking=True)
        for st in g_streams:
            stream.wait_stream(st)

    e2e_groups()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(args.steps):
        e2e_groups()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t1) / args.steps
    groups_same = all(torch.equal(serial_hits[k], pin_out[k]) for k in OUT_FIELDS)

    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle
        # a bounded sample: the 8 cheapest scenes to rebuild on the CPU, 20k rays each at most
        order = sorted(range(len(specs)), key=lambda i: built[i][1])[:8]
        rays_done, secs = 0, 0.0
        threads = os.cpu_count() or 1
        for i in order:
            sp = specs[i]
            ops = svo.gen_scene(sp["kind"], sp["size"], sp["brick_dim"], sp["seed"], occupancy=sp["occupancy"],
                                spheres=sp["spheres"], octaves=sp["octaves"], base_freq=sp["base_freq"])
            ot = oracle.Tree(sp["size"], sp["brick_dim"])
            ot.apply_ops(ops)
            o, d = host_rays[i][:2]
            step = max(1, len(o) // 20000)
            tt = time.perf_counter()
            ot.cast(o[::step], d[::step], threads=threads)
            secs += time.perf_counter() - tt
            rays_done += len(o[::step])
        cpu = {"value": round(rays_done / secs / 1e6, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
               "sample": "%d rays over the 8 smallest of the 64 scenes" % rays_done}

    peak, peak_src = measured_peak()
    print(json.dumps({
        "metric": "Mrays/s", "value": round(total / (graph_ms / 1e3) / 1e6, 3), "unit": "Mrays/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(graph_ms, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "multiscene64", "scenes": len(specs), "rays_per_step": total,
                   "sizes": sorted({sp["size"] for sp in specs}), "brick_dims": sorted({sp["brick_dim"] for sp in specs}),
                   "voxels_inserted": int(sum(b[1] for b in built)), "build_s": round(build_s, 1),
                   "l2": "rays %.0f MB + hits %.0f MB per step (larger than L2)" % (total * 24 / 1e6, total * 34 / 1e6),
                   "timed": "the batched cast replayed from a CUDA graph (one persistent launch; with sort_key 1 the ray sort's six launches too)",
                   "ray_order": "per scene: camera rays as rows of the image (8 x 4 ray blocks per warp), "
                                "random rays in order or sorted by direction octant and entry point (autotune.sort_key)",
                   "serial_plain": {"value": round(total / (serial_ms / 1e3) / 1e6, 3), "ms_per_step": round(serial_ms, 4),
                                    "launches_per_step": len(items)},
                   "batched": {"value": round(total / (batched_ms / 1e3) / 1e6, 3), "ms_per_step": round(batched_ms, 4)},
                   "batched_equals_serial": bool(same),
                   "autotune": {"block": cfg.block, "rays_per_chunk": cfg.rays_per_chunk, "block_shape": cfg.block_shape,
                                "sort_key": cfg.sort_key, "cached": tune_info["cached"],
                                "sweep_ms": tune_info.get("sweep_ms")}},
        "roofline": {"bound": "hbm", "achieved": round(alg / (graph_ms / 1e3) / 1e9, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(alg / (graph_ms / 1e3) / 1e9 / peak, 4), "traffic": None, "peak_source": peak_src,
                     "alg_bytes_per_launch": alg, "alg_bytes_per_ray": round(alg / total, 2)},
        "cpu_baseline": cpu,
        "e2e": {"value": round(total / e2e_s / 1e6, 3), "unit": "Mrays/s", "h2d_bytes_per_step": total * 24,
                "d2h_bytes_per_step": total * sum(OUT_BYTES.values()),
                "how": "4 groups of items, each copy-in, batched launch, copy-out on its own stream",
                "one_stream": round(total / e2e_serial_s / 1e6, 3), "same_hits_as_one_stream": bool(groups_same)},
        "gpu_launches": args.steps * batched_launches(bitems, gcfg.sort_key),
        "clocks": clk,
    }))


def run_served(args, w):
    """Served load: Poisson camera requests over 16 resident scenes, continuous batching vs serial dispatch."""
    import torch
    import shocovox_gb300 as svo
    torch.cuda.set_device(0)
    rng = np.random.default_rng(w["seed"])
    sizes = [int(v) for v in rng.permutation(np.repeat([256, 512, 1024, 2048], w["served"] // 4))]
    t0 = time.perf_counter()
    scenes = []
    for i, S in enumerate(sizes):
        ops = svo.gen_scene(4, S, 8, w["seed"] + 31 * i, occupancy=float(rng.uniform(0.01, 0.05)))
        t = svo.Octree(S, 8)
        t.apply_ops(ops)
        scenes.append(t)
    build_s = time.perf_counter() - t0
    n_req = w["requests"]
    arrivals = np.cumsum(rng.exponential(1.0 / w["rate"], n_req))
    reqs = []
    for k in range(n_req):
        j = int(rng.integers(0, len(scenes)))
        S = float(sizes[j])
        a, el = rng.uniform(0, 2 * np.pi), rng.uniform(0.35, 0.7)
        eye = [S / 2 + 1.4 * S * np.cos(el) * np.cos(a), S / 2 + 1.4 * S * np.sin(el), S / 2 + 1.4 * S * np.cos(el) * np.sin(a)]
        target = [S / 2 + rng.uniform(-0.1, 0.1) * S, S / 2, S / 2 + rng.uniform(-0.1, 0.1) * S]
        wd, ht = RESOLUTIONS[int(rng.integers(0, len(RESOLUTIONS)))]
        reqs.append((j, eye, target, 60.0, wd, ht))
    total_rays = sum(r[4] * r[5] for r in reqs)
    # pinned result buffers (status + albedo per ray), reused round-robin by later requests
    ring = 48
    maxn = max(r[4] * r[5] for r in reqs)
    bufs = [{"status": torch.empty(maxn, dtype=torch.uint8).pin_memory().numpy(),
             "albedo": torch.empty(maxn, dtype=torch.int32).pin_memory().numpy()} for _ in range(ring)]

    def serve(srv, paced):
        ids = [srv.add_scene(t) for t in scenes]
        assert ids == list(range(len(scenes)))
        # warm-up: every scene resident and the launch path exercised once
        for j in range(len(scenes)):
            srv.wait(srv.submit(j, [0.0, float(sizes[j]), 0.0], [sizes[j] / 2] * 3, 60.0, 64, 64,
                                out={k: v[:4096] for k, v in bufs[0].items()}))
        start = srv.now()
        rids, res = [], [None] * len(reqs)
        for k, r in enumerate(reqs):
            if k >= ring:  # the result buffers of request k - ring are reused: it must be done
                res[k - ring] = srv.wait(rids[k - ring], 600.0)
            if paced:
                delay = start + arrivals[k] - srv.now()
                if delay > 0:
                    time.sleep(delay)
            out = {kk: v[:r[4] * r[5]] for kk, v in bufs[k % ring].items()}
            rids.append(srv.submit(*r, out=out))
        for k in range(max(0, len(reqs) - ring), len(reqs)):
            res[k] = srv.wait(rids[k], 600.0)
        lat = np.array([x["done_s"] - x["submit_s"] for x in res])
        span = max(x["done_s"] for x in res) - min(x["submit_s"] for x in res)
        st = srv.stats()
        srv.close()
        return {"value": round(total_rays / span / 1e6, 3), "p50_ms": round(float(np.percentile(lat, 50)) * 1e3, 2),
                "p99_ms": round(float(np.percentile(lat, 99)) * 1e3, 2), "span_s": round(span, 3),
                "launches": st["launches"], "uploads": st["uploads"], "evictions": st["evictions"],
                "mean_batch": round(float(np.mean([x["batch_requests"] for x in res])), 2)}

    # latency-bound: clock samples once a second (each nvidia-smi query is a driver call on the host)
    clocks = ClockSampler(0, interval_ms=1000)
    clocks.start()
    budget = int(w["budget_gb"] * (1 << 30))
    # paced load: launches of at most 4 M rays keep a large request from delaying the next ones
    batched = serve(svo.Server(budget_bytes=budget, max_batch_requests=64, max_batch_rays=1 << 22, max_inflight=3),
                    paced=True)
    serial = serve(svo.Server(budget_bytes=budget, max_batch_requests=1, max_inflight=1), paced=True)
    # capacity: the same requests submitted as fast as result buffers free up (48 in flight)
    batched_cap = serve(svo.Server(budget_bytes=budget, max_batch_requests=64, max_batch_rays=1 << 25,
                                   max_inflight=3), paced=False)
    serial_cap = serve(svo.Server(budget_bytes=budget, max_batch_requests=1, max_inflight=1), paced=False)
    clk = clocks.stop()
    print(json.dumps({
        "metric": "Mrays/s", "value": batched["value"], "unit": "Mrays/s", "n_gpus": 1, "steps": n_req, "warmup": len(scenes),
        "ms_per_step": round(batched["span_s"] / n_req * 1e3, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "served16", "scenes": len(scenes), "sizes": sizes, "requests": n_req,
                   "arrival_rate_per_s": w["rate"], "rays": total_rays, "budget_gb": w["budget_gb"],
                   "build_s": round(build_s, 1), "outputs": "status + albedo per ray, to pinned host memory",
                   "server_config": {"paced": "max_batch_requests 64, max_batch_rays 2^22, max_inflight 3",
                                     "capacity": "max_batch_requests 64, max_batch_rays 2^25, max_inflight 3",
                                     "serial_dispatch": "max_batch_requests 1, max_inflight 1"},
                   "served": batched, "serial_dispatch": serial,
                   "capacity": {"note": "all requests queued, 48 outstanding", "served": batched_cap,
                                "serial_dispatch": serial_cap},
                   "p50_ms": batched["p50_ms"], "p99_ms": batched["p99_ms"]},
        "roofline": None, "cpu_baseline": None,
        "e2e": {"value": batched["value"], "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(total_rays * 5 / n_req)},
        "gpu_launches": batched["launches"], "clocks": clk,
    }))


def viewport_rays(vp, W, H):
    """The rays of svo_render_viewport's pixels in image order (row 0 = top), formed on the host with
    examples/cpu_render.rs's f32 operations (the device forms the same bits)."""
    F = np.float32

    def norm(v):
        n = np.sqrt((v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1]) + v[..., 2] * v[..., 2])
        return v / n[..., None]
    o, d, up = (np.array(list(getattr(vp, k)), F) for k in ("origin", "direction", "up"))
    right = norm(np.array([up[1] * d[2] - up[2] * d[1], up[2] * d[0] - up[0] * d[2], up[0] * d[1] - up[1] * d[0]], F))
    pw, ph = F(vp.width) / F(W), F(vp.height) / F(H)
    bl = ((o + d * F(vp.fov)) - up * (F(vp.height) / F(2))) - right * (F(vp.width) / F(2))
    x = np.arange(W, dtype=F)[None, :, None]
    y = np.arange(H, dtype=F)[:, None, None]
    dirs = norm(((bl + (right * x) * pw) + (up * y) * ph) - o)[::-1].reshape(-1, 3)
    return np.ascontiguousarray(np.broadcast_to(o, dirs.shape)), np.ascontiguousarray(dirs)


def run_viewport(args, w):
    """Fused render (svo_render_viewport) of 4 orbit viewports vs the plain cast of the same rays."""
    import torch
    import shocovox_gb300 as svo
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    t0 = time.perf_counter()
    ops = scene_ops(svo, w)
    scene = svo.Octree(w["size"], w["brick_dim"])
    scene.apply_ops(ops)
    build_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream(dev)
    s = stream.cuda_stream
    scene.upload(s)
    S, W, H = float(w["size"]), w["width"], w["height"]
    rng = np.random.default_rng(w["seed"])
    vps = []
    for _ in range(w["viewport"]):
        v = svo.orbit_viewport(rng.uniform(0, 2 * np.pi), 1.1 * S)
        o = np.array(list(v.origin), np.float32) + np.float32(S / 2)
        d = np.array([S / 2, 0.2 * S, S / 2], np.float32) - o
        d = d / np.sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2], dtype=np.float32)
        vps.append(svo.viewport(o, d, fov=2.0))
    n = W * H * len(vps)
    img = torch.empty((len(vps), H, W, 4), dtype=torch.uint8, device=dev)
    bad = torch.zeros(1, dtype=torch.int64, device=dev)
    pin = torch.empty((len(vps), H, W, 4), dtype=torch.uint8).pin_memory()

    def render():  # the 4 frames in one launch (svo_render_viewports)
        scene.render_viewports(vps, W, H, img.data_ptr(), bad.data_ptr(), s)

    def render_one_per_call():
        for k, vp in enumerate(vps):
            scene.render_viewport(vp, W, H, img[k].data_ptr(), bad.data_ptr(), s)

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(0)
    clocks.start()
    for _ in range(args.warmup):
        render()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        render()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    # end to end: the frames land in pinned host memory every step
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(args.steps):
        render()
        pin.copy_(img, non_blocking=True)
    torch.cuda.synchronize()
    e2e_one_s = (time.perf_counter() - t1) / args.steps
    # the same with two launches of two frames on two streams: one pair's copy overlaps the other's render
    pair_streams = [torch.cuda.Stream(dev) for _ in range(2)]
    pair_start = torch.cuda.Event()

    def render_pairs_to_host():
        pair_start.record(stream)
        for q, st in enumerate(pair_streams):
            st.wait_event(pair_start)
            with torch.cuda.stream(st):
                scene.render_viewports(vps[2 * q:2 * q + 2], W, H, img[2 * q].data_ptr(), bad.data_ptr(), st.cuda_stream)
                pin[2 * q:2 * q + 2].copy_(img[2 * q:2 * q + 2], non_blocking=True)
        for st in pair_streams:
            stream.wait_stream(st)
    render_pairs_to_host()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(args.steps):
        render_pairs_to_host()
    torch.cuda.synchronize()
    e2e_pairs_s = (time.perf_counter() - t1) / args.steps
    e2e_s = e2e_pairs_s
    # the same frames with one svo_render_viewport call (one launch) per frame
    render_one_per_call()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        render_one_per_call()
    e1.record(stream)
    torch.cuda.synchronize()
    per_view_ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()

    # the same rays through the plain cast (rays resident in HBM), and the algorithmic bytes
    host = [viewport_rays(vp, W, H) for vp in vps]
    o_all = np.concatenate([h[0] for h in host])
    d_all = np.concatenate([h[1] for h in host])
    cols = [np.ascontiguousarray(o_all[:, i]) for i in range(3)] + [np.ascontiguousarray(d_all[:, i]) for i in range(3)]
    rays = {k: torch.from_numpy(c).to(dev) for k, c in zip(("ox", "oy", "oz", "dx", "dy", "dz"), cols)}
    rp = {k: v.data_ptr() for k, v in rays.items()}
    tmap = {np.uint8: torch.uint8, np.uint32: torch.int32, np.float32: torch.float32}
    outs = {k: torch.empty(n, dtype=tmap[svo.HIT_FIELDS[k]], device=dev) for k in ("status", "albedo", "nx", "ny", "nz")}
    hp = {k: v.data_ptr() for k, v in outs.items()}
    for _ in range(args.warmup):
        scene.cast(rp, hp, n, s, row_length=W)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        scene.cast(rp, hp, n, s, row_length=W)
    e1.record(stream)
    torch.cuda.synchronize()
    cast_ms = e0.elapsed_time(e1) / args.steps
    # the same rays cast one frame per launch, as the render launches
    per = W * H

    def cast_frames():
        for k in range(len(vps)):
            scene.cast({kk: v + 4 * k * per for kk, v in rp.items()},
                       {kk: v + (1 if kk == "status" else 4) * k * per for kk, v in hp.items()}, per, s, row_length=W)
    cast_frames()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        cast_frames()
    e1.record(stream)
    torch.cuda.synchronize()
    cast_frames_ms = e0.elapsed_time(e1) / args.steps
    cnt = {k: torch.empty(n, dtype=torch.int32, device=dev) for k in COUNTERS}
    st = torch.empty(n, dtype=torch.uint8, device=dev)
    scene.cast(rp, dict(status=st.data_ptr(), **{k: v.data_ptr() for k, v in cnt.items()}), n, s, row_length=W)
    torch.cuda.synchronize()
    visits, creads, vreads, runs = (int(cnt[k].to(torch.int64).sum()) for k in COUNTERS)
    hits = int((st == 1).sum())
    # a fused pixel reads the scene like its cast and writes 4 bytes instead of 24 B in + hit fields out
    alg = alg_bytes_of(visits - runs, creads, vreads, hits) + 4 * n
    del cnt, rays, outs

    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle
        ot = oracle.Tree(w["size"], w["brick_dim"])
        ot.apply_ops(ops)
        threads = os.cpu_count() or 1
        rate, m, stride, dt = cpu_cast_rate(ot, o_all, d_all, args.cpu_seconds, threads)
        cpu = {"value": round(rate / 1e6, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
               "sample": "every %dth pixel ray of the 4 frames (%d rays, %.1fs on %d threads), cast only" % (
                   stride, m, dt, threads)}
    peak, peak_src = measured_peak()
    achieved = alg / (ms / 1e3) / 1e9
    print(json.dumps({
        "metric": "Mrays/s", "value": round(n / (ms / 1e3) / 1e6, 3), "unit": "Mrays/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "viewport512", "octree": "%d^3" % w["size"], "brick_dim": w["brick_dim"],
                   "frames_per_step": len(vps), "resolution": [W, H], "rays_per_step": n, "hit_rate": round(hits / n, 4),
                   "per_ray": {"node_visits": round(visits / n, 2), "child_reads": round(creads / n, 2),
                               "voxel_reads": round(vreads / n, 2), "restart_run_visits": round(runs / n, 2)},
                   "build_s": round(build_s, 1), "unshaded_pixels": int(bad.item()),
                   "l2": "frames %.0f MB per step (larger than L2); the scene image stays resident" % (n * 4 / 1e6),
                   "timed": "svo_render_viewports: the 4 frames in one launch",
                   "render_one_view_per_launch": {"value": round(n / (per_view_ms / 1e3) / 1e6, 3),
                                                  "ms_per_step": round(per_view_ms, 4)},
                   "cast_of_same_rays": {"value": round(n / (cast_ms / 1e3) / 1e6, 3), "ms_per_step": round(cast_ms, 4),
                                         "note": "svo_cast, rays resident in HBM, status+albedo+normal out, "
                                                 "all frames in one launch"},
                   "cast_of_same_rays_per_frame": {"value": round(n / (cast_frames_ms / 1e3) / 1e6, 3),
                                                   "ms_per_step": round(cast_frames_ms, 4),
                                                   "note": "the same, one launch per frame like the render"}},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": profile_traffic(args.workload).get("dram_bytes_per_launch"), "peak_source": peak_src,
                     "alg_bytes_per_launch": alg, "alg_bytes_per_ray": round(alg / n, 2)},
        "cpu_baseline": cpu,
        "e2e": {"value": round(n / e2e_s / 1e6, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": n * 4,
                "paths": {"one_launch_then_copy": round(n / e2e_one_s / 1e6, 3),
                          "two_streams_of_two_frames": round(n / e2e_pairs_s / 1e6, 3)}},
        "gpu_launches": args.steps, "clocks": clk,
    }))


def run_lod(args, w):
    """get_by_ray_at_lod with MIP maps (svo_cast_lod) on the terrain512 scene and cameras."""
    import torch
    import shocovox_gb300 as svo
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    t0 = time.perf_counter()
    ops = scene_ops(svo, w)
    scene = svo.Octree(w["size"], w["brick_dim"])
    scene.apply_ops(ops)
    build_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    scene.switch_albedo_mip_maps(True)  # recalculate_mips with the default strategy
    mip_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream(dev)
    s = stream.cuda_stream
    scene.upload(s)
    origins, dirs = make_rays(svo, w)
    n = len(origins)
    cols = [np.ascontiguousarray(origins[:, i]) for i in range(3)] + [np.ascontiguousarray(dirs[:, i]) for i in range(3)]
    rays = {k: torch.from_numpy(c).to(dev) for k, c in zip(("ox", "oy", "oz", "dx", "dy", "dz"), cols)}
    rp = {k: v.data_ptr() for k, v in rays.items()}
    tmap = {np.uint8: torch.uint8, np.uint32: torch.int32, np.float32: torch.float32}
    out = {k: torch.empty(n, dtype=tmap[svo.HIT_FIELDS[k]], device=dev) for k in OUT_FIELDS}
    hp = {k: v.data_ptr() for k, v in out.items()}
    vd = w["lod"]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    row = ray_rows(w)  # camera images in raster order: svo_cast_lod_rows
    clocks = ClockSampler(0)
    clocks.start()
    ms = timed(lambda: scene.cast_lod(rp, hp, n, vd, s, row_length=row))
    max_ms = timed(lambda: scene.cast_lod(rp, hp, n, float(np.finfo(np.float32).max), s, row_length=row))
    plain_ms = timed(lambda: scene.cast(rp, hp, n, s, row_length=row))
    lod_plain_order_ms = timed(lambda: scene.cast_lod(rp, hp, n, vd, s))
    # end to end: rays from pinned host memory, status + albedo back, copies in the timed region
    pin_in = {k: torch.from_numpy(c).pin_memory() for k, c in zip(("ox", "oy", "oz", "dx", "dy", "dz"), cols)}
    pin_out = {k: torch.empty(n, dtype=tmap[svo.HIT_FIELDS[k]]).pin_memory() for k in ("status", "albedo")}

    # one camera image per stream: its rays in, its LOD cast, its status and albedo out, so that one
    # image's copies overlap another's cast
    frames = w["rays"][1]
    per = n // frames
    f_streams = [torch.cuda.Stream(dev) for _ in range(frames)]
    f_start = torch.cuda.Event()

    def e2e():
        f_start.record(stream)
        for f, st in enumerate(f_streams):
            lo, hi = f * per, (f + 1) * per
            st.wait_event(f_start)
            with torch.cuda.stream(st):
                for k, v in pin_in.items():
                    rays[k][lo:hi].copy_(v[lo:hi], non_blocking=True)
                scene.cast_lod({k: v + 4 * lo for k, v in rp.items()},
                               {k: v + np.dtype(svo.HIT_FIELDS[k]).itemsize * lo for k, v in hp.items()},
                               per, vd, st.cuda_stream, row_length=row)
                for k, v in pin_out.items():
                    v[lo:hi].copy_(out[k][lo:hi], non_blocking=True)
        for st in f_streams:
            stream.wait_stream(st)
    e2e()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(args.steps):
        e2e()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t1) / args.steps
    clk = clocks.stop()
    cnt = {k: torch.empty(n, dtype=torch.int32, device=dev) for k in COUNTERS}
    st = torch.empty(n, dtype=torch.uint8, device=dev)
    oct_ = torch.empty(n, dtype=torch.uint8, device=dev)
    scene.cast_lod(rp, dict(status=st.data_ptr(), brick_octant=oct_.data_ptr(), **{k: v.data_ptr() for k, v in cnt.items()}),
                   n, vd, s)
    torch.cuda.synchronize()
    visits, creads, vreads, runs = (int(cnt[k].to(torch.int64).sum()) for k in COUNTERS)
    hits = int((st == 1).sum())
    mip_hits = int(((st == 1) & (oct_ == 8)).sum())
    alg = alg_bytes_of(visits - runs, creads, vreads, hits)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle
        ot = oracle.Tree(w["size"], w["brick_dim"])
        ot.apply_ops(ops)
        ot.mip_switch(True)
        threads = os.cpu_count() or 1
        rate, m, step, dt = cpu_cast_rate(ot, origins, dirs, args.cpu_seconds, threads, viewing_distance=vd)
        cpu = {"value": round(rate / 1e6, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
               "sample": "every %dth ray of the batch (%d rays, %.1fs on %d threads)" % (step, m, dt, threads)}
    peak, peak_src = measured_peak()
    achieved = alg / (ms / 1e3) / 1e9
    st_ = scene.stats()
    print(json.dumps({
        "metric": "Mrays/s", "value": round(n / (ms / 1e3) / 1e6, 3), "unit": "Mrays/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "lod512", "octree": "%d^3" % w["size"], "brick_dim": w["brick_dim"],
                   "rays_per_step": n, "viewing_distance": vd, "hit_rate": round(hits / n, 4),
                   "mip_hit_rate": round(mip_hits / n, 4), "build_s": round(build_s, 1),
                   "mip_recalculation_s": round(mip_s, 1), "nodes": st_["nodes"],
                   "per_ray": {"node_visits": round(visits / n, 2), "child_reads": round(creads / n, 2),
                               "voxel_reads": round(vreads / n, 2)},
                   "l2": "inputs larger than L2 (rays %.0f MB + hits %.0f MB per step)" % (
                       n * 24 / 1e6, n * sum(OUT_BYTES.values()) / 1e6),
                   "lod_at_f32_max": {"value": round(n / (max_ms / 1e3) / 1e6, 3), "ms_per_step": round(max_ms, 4)},
                   "svo_cast_same_rays": {"value": round(n / (plain_ms / 1e3) / 1e6, 3),
                                          "ms_per_step": round(plain_ms, 4)},
                   "ray_order": "rows of %d rays (svo_cast_lod_rows: 8 x 4 ray blocks per warp)" % row,
                   "svo_cast_lod_plain_order": {"value": round(n / (lod_plain_order_ms / 1e3) / 1e6, 3),
                                                "ms_per_step": round(lod_plain_order_ms, 4)}},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": profile_traffic(args.workload).get("dram_bytes_per_launch"), "peak_source": peak_src,
                     "alg_bytes_per_launch": alg, "alg_bytes_per_ray": round(alg / n, 2)},
        "cpu_baseline": cpu,
        "e2e": {"value": round(n / e2e_s / 1e6, 3), "unit": "Mrays/s", "h2d_bytes_per_step": n * 24,
                "d2h_bytes_per_step": n * 5,
                "how": "per camera image on its own stream: rays in, svo_cast_lod_rows, status + albedo out"},
        "gpu_launches": args.steps, "clocks": clk,
    }))


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
        if "multi" in w or "served" in w or "viewport" in w or "lod" in w:
            print(json.dumps({"impl": "reference", "unavailable": "the reference arm times the default single-scene workload"}))
            return
        run_reference(args, w)
        return
    if "multi" in w:
        run_multiscene(args, w)
        return
    if "served" in w:
        run_served(args, w)
        return
    if "viewport" in w:
        run_viewport(args, w)
        return
    if "lod" in w:
        run_lod(args, w)
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

    # camera rays in raster order: svo_cast_rows hands warps 8 x 4 blocks of neighbouring pixels
    row = ray_rows(w)
    clocks = ClockSampler(local_rank)
    clocks.start()  # samples from the warm-up on, so that short timed regions still get samples
    for _ in range(args.warmup):
        scene.cast(rp, hp, n, s, row_length=row)
    torch.cuda.synchronize()

    # algorithmic bytes of one launch from the instrumented cast (counters equal the oracle's, see tests)
    cnt = {k: torch.empty(n, dtype=torch.int32, device=dev) for k in COUNTERS}
    st = torch.empty(n, dtype=torch.uint8, device=dev)
    scene.cast(rp, dict(status=st.data_ptr(), **{k: v.data_ptr() for k, v in cnt.items()}), n, s, row_length=row)
    torch.cuda.synchronize()
    visits, creads, vreads, runs = (int(cnt[k].to(torch.int64).sum()) for k in COUNTERS)
    hits = int((st == 1).sum())
    alg_bytes = alg_bytes_of(visits - runs, creads, vreads, hits)
    del cnt

    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        scene.cast(rp, hp, n, s, row_length=row)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    if pg:
        pg.barrier()
    ms = max_over_ranks(ms, pg)
    ms_step = ms / args.steps
    value = n * world / (ms_step / 1e3) / 1e6
    # the same rays through plain svo_cast (warps take 32 consecutive rays of one row)
    plain = None
    if row:
        if pg:
            pg.barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            scene.cast(rp, hp, n, s)
        e1.record(stream)
        torch.cuda.synchronize()
        pms = max_over_ranks(e0.elapsed_time(e1), pg) / args.steps
        plain = {"value": round(n * world / (pms / 1e3) / 1e6, 3), "ms_per_step": round(pms, 4)}

    variants = None
    if not args.no_variants:
        variants = batched_variants(svo, torch, scene, rp, hp, n, stream, args, row)
    clk = clocks.stop()

    # end to end through the host-buffer C-ABI call (pinned host memory)
    pin_cols = [torch.from_numpy(c).pin_memory() for c in cols_host]
    pin_out = {k: torch.empty(n, dtype=tmap[svo.HIT_FIELDS[k]]).pin_memory() for k in OUT_FIELDS}
    cols_np = [c.numpy() for c in pin_cols]
    out_np = {k: v.numpy() for k, v in pin_out.items()}
    for _ in range(max(1, args.warmup)):
        scene.cast_host_soa(cols_np, out_np, s, row_length=row)
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        scene.cast_host_soa(cols_np, out_np, s, row_length=row)
    e2e_s = max_over_ranks(time.perf_counter() - t0, pg)
    e2e_value = n * world * args.steps / e2e_s / 1e6
    # the two ways svo_cast_host can move the data (svo_set_host_transfer), each timed the same way
    e2e_paths = {}
    for mode, name in ((1, "staged_copies"), (2, "direct_host_access")):
        if svo.lib().svo_set_host_transfer(mode) != 0:
            e2e_paths[name] = None
            continue
        scene.cast_host_soa(cols_np, out_np, s, row_length=row)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            scene.cast_host_soa(cols_np, out_np, s, row_length=row)
        e2e_paths[name] = round(n * world * args.steps / max_over_ranks(time.perf_counter() - t0, pg) / 1e6, 3)
    svo.lib().svo_set_host_transfer(0)

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
    prof = profile_traffic(args.workload)
    traffic = prof.get("dram_bytes_per_launch")
    l2 = None
    if prof.get("l2_bytes_per_launch"):
        l2 = {"bytes_per_launch": prof["l2_bytes_per_launch"],
              "gbs": round(prof["l2_bytes_per_launch"] / (ms_step / 1e3) / 1e9, 1),
              "hit_rate_pct": prof.get("l2_hit_rate_pct"), "l1_hit_rate_pct": prof.get("l1_hit_rate_pct"),
              "frac_of_l2_peak": round(prof["l2_throughput_pct_of_peak"] / 100.0, 4),
              "source": "ncu capture of one launch (profiles/); gbs with this run's kernel time"}
    if rank == 0:
        st = scene.stats()
        print(json.dumps({
            "metric": "Mrays/s", "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "octree": "%d^3" % w["size"], "brick_dim": w["brick_dim"],
                       "rays_per_step": n, "hit_rate": round(hits / n, 4), "nodes": st["nodes"],
                       "per_ray": {"node_visits": round(visits / n, 2), "child_reads": round(creads / n, 2),
                                   "voxel_reads": round(vreads / n, 2), "restart_run_visits": round(runs / n, 2)},
                       "parted_bricks": st["parted_bricks"], "voxels_inserted": int(len(ops)),
                       "l2": "inputs larger than L2 (rays %.0f MB + hits %.0f MB per step); the %.0f MB scene image "
                             "stays resident" % (n * 24 / 1e6, n * sum(OUT_BYTES.values()) / 1e6,
                                                 st["device_bytes"] / 1e6),
                       "build_s": round(build_s, 1), "parallelism": "replicas" if world > 1 else "single",
                       "ray_order": ("rows of %d rays (svo_cast_rows: 8 x 4 ray blocks per warp)" % row) if row
                       else "as generated (svo_cast)",
                       "svo_cast_plain_order": plain},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_src,
                         "alg_bytes_per_launch": alg_bytes,
                         "alg_bytes_per_ray": round(alg_bytes / n, 2), "l2": l2},
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e_value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": n * 24,
                    "d2h_bytes_per_step": n * sum(OUT_BYTES.values()), "paths": e2e_paths},
            "gpu_launches": args.steps,
            "clocks": clk,
            "variants": variants,
        }))
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
