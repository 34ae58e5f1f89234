#!/usr/bin/env python
"""Benchmark: Mrays/s of the sparse-voxel-octree first-hit cast on one GB300.

Default workload ("terrain512", coherent primary rays at scale): a 512^3
octree with brick dimension 8 filled with a seeded 3-octave value-noise
terrain with caves (3D noise threshold 0.55, ~9.4% occupancy), 4 pinhole
cameras at 1920x1080 and 70 deg FOV at seeded positions above the terrain:
8,294,400 f32 rays per step.  A step is one cast of the whole batch.

  value   rays/s with rays and hits resident in HBM (device pointers, svo_cast_rows)
  e2e     the same batch through the host-buffer C-ABI call svo_cast_host_rows:
          host->device copy of the rays and device->host copy of the results
          inside the timed region
  parity  every ray of the batch cast again by the CPU oracle (a restatement of
          the reference's get_by_ray) and compared field by field with the
          timed launch, the instrumented launch, the other ray orders and the
          host-buffer path: hit identity and counters exactly, impact point and
          normal within 1e-4 voxel units.  A mismatch makes the run exit 1.

The default run also measures, in sub-objects of its one JSON line
("comparisons"), the plain cast against the batched and served forms on the
incoherent-ray, multi-scene and served workloads, each over repeated timings
with its own parity check and clock record.

`--impl reference` times the oracle's CPU cast (the reference is a Rust crate
that cannot be built here) on all host cores over the whole batch of the same
workload, with the scene and rays made by the oracle's own generators: it
loads no product code.
"""
import argparse
import gc
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
    # 10,000 Poisson requests at 2,000/s (5 s); the device budget is half the 16 scene images, so
    # scenes are evicted and uploaded again while requests run
    "served16": dict(served=16, seed=0x5EED0005, rate=2000.0, requests=10000, budget_frac=0.5, repeats=3),
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
RAY_KEYS = ("ox", "oy", "oz", "dx", "dy", "dz")
REPEATS = 5  # timed repeats of each compared variant (median and spread are reported)

# ---- parity against the oracle --------------------------------------------------------------------
TOL = 1e-4  # voxel units: impact point and normal
ID_FIELDS = ("status", "brick_octant", "entry_kind", "node_key", "voxel_index", "pix", "albedo", "user")
FLOAT_FIELDS = ("px", "py", "pz", "nx", "ny", "nz")
CHECKED_COUNTERS = ("node_visits", "child_reads", "voxel_reads")
ALL_CHECKED = ID_FIELDS + FLOAT_FIELDS + CHECKED_COUNTERS


def compare_hits(got, ref, label=""):
    """Compares product results `got` (host arrays) with the oracle's cast `ref` of the same rays, over
    the fields `got` has: hit identity and counters exactly, point and normal within TOL (NaN on both
    sides agrees).  Returns a parity record."""
    fields = [k for k in ALL_CHECKED if k in got]
    n = len(got[fields[0]]) if fields else 0
    bad = np.zeros(n, dtype=bool)
    err = {"p": 0.0, "n": 0.0}
    first = {}
    for k in fields:
        a, b = np.asarray(got[k]), np.asarray(ref[k])
        if k in FLOAT_FIELDS:
            a64, b64 = a.astype(np.float64), b.astype(np.float64)
            same = (a64 == b64) | (np.isnan(a64) & np.isnan(b64))
            with np.errstate(invalid="ignore"):
                d = np.where(same, 0.0, np.abs(a64 - b64))
            d = np.where(np.isnan(d), np.inf, d)
            off = ~(d <= TOL)
            if n:
                err[k[0]] = max(err[k[0]], float(d.max()))
        else:
            off = a.astype(np.uint32) != b.astype(np.uint32)
        if off.any():
            first[k] = int(np.argmax(off))
        bad |= off
    rec = {"rays_checked": n, "mismatches": int(bad.sum()), "fields": fields,
           "max_point_err": _finite(err["p"]), "max_normal_err": _finite(err["n"]), "tolerance": TOL}
    if first:
        rec["first_mismatch"] = {k: int(v) for k, v in first.items()}
    if label:
        rec["what"] = label
    return rec


def _finite(v):
    return v if np.isfinite(v) else "inf"


def merge_parity(recs):
    """One record over several checks: rays and mismatches add up, the largest errors are kept."""
    recs = [r for r in recs if r]
    if not recs:
        return None

    def mx(k):
        vals = [r[k] for r in recs]
        return "inf" if "inf" in vals else max(vals)
    return {"rays_checked": sum(r["rays_checked"] for r in recs), "mismatches": sum(r["mismatches"] for r in recs),
            "checks": [r.get("what", "") for r in recs], "max_point_err": mx("max_point_err"),
            "max_normal_err": mx("max_normal_err"), "tolerance": TOL,
            "bad": [r for r in recs if r["mismatches"]][:4]}


def parity_failed(rec):
    """True when a record or any nested record reports a mismatch (or an unchecked error)."""
    if isinstance(rec, dict):
        if "parity" in rec and isinstance(rec["parity"], dict) and rec["parity"].get("mismatches", 0):
            return True
        if rec.get("error"):
            return True
        return any(parity_failed(v) for k, v in rec.items() if k != "parity")
    if isinstance(rec, list):
        return any(parity_failed(v) for v in rec)
    return False


# ---- workload generation (gen = the product module or the oracle module: same signatures) -------
def scene_ops(gen, w):
    return gen.gen_scene(w["kind"], w["size"], w["brick_dim"], w["seed"], occupancy=w.get("occupancy", 0.1),
                         spheres=w.get("spheres", 0), octaves=w.get("octaves", 2), base_freq=w.get("base_freq", 1 / 32),
                         height_lo=w.get("height_lo", 0.0), height_hi=w.get("height_hi", 0.0),
                         cave_threshold=w.get("cave_threshold", 0.55))


def make_rays(gen, w):
    spec = w["rays"]
    S = float(w["size"])
    rng = np.random.default_rng(w["seed"])
    if spec[0] == "cameras":
        _, ncam, width, height, fov = spec
        os_, ds = [], []
        for _ in range(ncam):
            eye = [rng.uniform(0.15, 0.85) * S, 0.45 * S, rng.uniform(0.15, 0.85) * S]
            target = [rng.uniform(0.1, 0.9) * S, 0.1 * S, rng.uniform(0.1, 0.9) * S]
            o, d = gen.gen_camera_rays(eye, target, fov, width, height)
            os_.append(o)
            ds.append(d)
        return np.concatenate(os_), np.concatenate(ds)
    if spec[0] == "orbit":
        _, _, width, height, fov = spec
        az, el = rng.uniform(0, 2 * np.pi), 0.5
        c = S / 2
        eye = [c + 200 * np.cos(el) * np.sin(az), c + 200 * np.sin(el), c + 200 * np.cos(el) * np.cos(az)]
        return gen.gen_camera_rays(eye, [c, c, c], fov, width, height)
    if spec[0] == "sphere":
        return gen.gen_sphere_rays([S / 2] * 3, S * np.sqrt(3.0) / 2, spec[1], w["seed"])
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
        return self

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


def host_fields(svo, d):
    """Device result tensors -> host numpy arrays of the product's field types."""
    return {k: v.cpu().numpy().view(svo.HIT_FIELDS[k]) for k, v in d.items()}


def device_outputs(torch, svo, n, dev, fields):
    tmap = {np.uint8: torch.uint8, np.uint32: torch.int32, np.float32: torch.float32}
    return {k: torch.empty(max(n, 1), dtype=tmap[svo.HIT_FIELDS[k]], device=dev) for k in fields}


def spread(n_rays, ms_list):
    """Median Mrays/s over repeats with the slowest and fastest repeat."""
    ms = np.asarray(ms_list, dtype=np.float64)
    rate = n_rays / (ms / 1e3) / 1e6
    return {"value": round(float(np.median(rate)), 3), "min": round(float(rate.min()), 3),
            "max": round(float(rate.max()), 3), "ms_per_step": round(float(np.median(ms)), 4),
            "repeats": len(ms_list)}


def versus(batched, plain):
    """How a batched form compares with the plain cast over repeats: median ratio, and whether its
    slowest repeat still beats plain's fastest (a win outside the run-to-run spread)."""
    return {"median_ratio": round(batched["value"] / plain["value"], 4),
            "beats_plain": batched["value"] > plain["value"],
            "beats_plain_outside_spread": batched["min"] > plain["max"]}


def interleaved_repeats(variants, steps, repeats, stream, torch):
    """Times every variant (name -> fn) over `steps` calls, `repeats` times, interleaving the variants so
    that drift of the clocks affects all alike.  Returns name -> [ms per step]."""
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {k: [] for k in variants}
    for _ in range(repeats):
        for k, fn in variants.items():
            fn()
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(steps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            out[k].append(e0.elapsed_time(e1) / steps)
    return out


def batched_launches(items, sort_key):
    """Kernel launches of one svo_cast_batched call: the claim-order cast if any item is cast in claim
    order, plus the ray sort's bin, three scan, scatter and cast launches if any item is sorted."""
    sorted_items = [it for it in items if sort_key and not (len(it) > 4 and it[4]) and it[2]]
    claimed = [it for it in items if it[2] and it not in sorted_items]
    return (1 if claimed else 0) + (6 if sorted_items else 0)


def autotune_batched(svo, torch, ws, items, stream, fixed_sort=None):
    """The project's autotuner (shocovox_gb300.autotune, no cache) on `items`: threads per block x rays
    per claim x ray-block shape (items with a row length) or ray-sort key (items without), then the
    staging depth of the best.  fixed_sort: only configurations with that sort key are kept.
    Returns (LaunchConfig, {config string: ms})."""
    from shocovox_gb300 import autotune
    s = stream.cuda_stream
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(cfg):
        if fixed_sort is not None and cfg.sort_key != fixed_sort:
            return float("inf")
        ws.cast(items, cfg, s)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(2):
            ws.cast(items, cfg, s)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 2

    cfg, info = autotune.tune(ws, items, torch.cuda.get_device_name(0), timed, use_cache=False)
    return cfg, {k: round(v, 4) for k, v in info["sweep_ms"].items() if v != float("inf")}


def cfg_record(c):
    return {"block": c.block, "rays_per_chunk": c.rays_per_chunk, "block_shape": c.block_shape, "sort_key": c.sort_key,
            "staging_depth": c.staging_depth, "refill_below": c.refill_below}


# ---- single scene: terrain512 (default), heightfield128, incoherent1024 ----------------------------
def run_single(args, w, workload):
    """The plain cast of one scene's batch (svo_cast_rows for camera images), with the ray orders, the
    persistent batched kernel and the host-buffer path beside it, every output checked against the
    oracle's cast of the whole batch."""
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
    want_check = rank == 0 and not args.no_parity
    if want_check:
        oth, obox = oracle_tree_async(ops, w)
    scene = svo.Octree(w["size"], w["brick_dim"])
    scene.apply_ops(ops)
    build_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream(dev)
    s = stream.cuda_stream
    scene.upload(s)
    origins, dirs = make_rays(svo, w)
    n = len(origins)
    cols_host = [np.ascontiguousarray(origins[:, i]) for i in range(3)] + [np.ascontiguousarray(dirs[:, i])
                                                                          for i in range(3)]
    rays_dev = {k: torch.from_numpy(c).to(dev) for k, c in zip(RAY_KEYS, cols_host)}
    outs = device_outputs(torch, svo, n, dev, OUT_FIELDS)
    rp = {k: v.data_ptr() for k, v in rays_dev.items()}
    hp = {k: v.data_ptr() for k, v in outs.items()}
    checks = []  # (label, host results) compared with the oracle at the end

    # camera rays in raster order: svo_cast_rows hands warps 8 x 4 blocks of neighbouring pixels
    row = ray_rows(w)
    lib = svo.lib()
    svo.check(lib.svo_set_refill(args.refill))  # the timed cast's knobs (0, 0: queue_kernel, nothing staged)
    svo.check(lib.svo_set_staging_depth(args.staging_depth))
    clocks = ClockSampler(local_rank).start()  # samples from the warm-up on, so short timed regions get samples
    for _ in range(args.warmup):
        scene.cast(rp, hp, n, s, row_length=row)
    torch.cuda.synchronize()

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
    if want_check:
        checks.append(("timed launch (%s)" % ("svo_cast_rows" if row else "svo_cast"), host_fields(svo, outs)))

    # the instrumented cast: every field and the counters (algorithmic bytes of one launch)
    full = device_outputs(torch, svo, n, dev, list(svo.HIT_FIELDS))
    scene.cast(rp, {k: v.data_ptr() for k, v in full.items()}, n, s, row_length=row)
    torch.cuda.synchronize()
    visits, creads, vreads, runs = (int(full[k].to(torch.int64).sum()) for k in COUNTERS)
    hits = int((full["status"] == 1).sum())
    alg_bytes = alg_bytes_of(visits - runs, creads, vreads, hits)
    if want_check:
        checks.append(("instrumented launch, every field and counter", host_fields(svo, full)))
    del full

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
        if want_check:
            checks.append(("svo_cast, plain ray order", host_fields(svo, outs)))

    variants = None
    if not args.no_variants:
        # the plain cast with the top tree levels staged in shared memory (svo_set_staging_depth)

        def staged(k):
            def run():
                lib.svo_set_staging_depth(k)
                scene.cast(rp, hp, n, s, row_length=row)
            return run
        st_reps = interleaved_repeats({k: staged(k) for k in range(5)}, args.steps, 3, stream, torch)
        lib.svo_set_staging_depth(0)
        stage_sweep = {"depth%d" % k: spread(n * world, v) for k, v in st_reps.items()}
        if want_check:
            lib.svo_set_staging_depth(4)
            scene.cast(rp, hp, n, s, row_length=row)
            torch.cuda.synchronize()
            lib.svo_set_staging_depth(0)
            checks.append(("%s, staging depth 4" % ("svo_cast_rows" if row else "svo_cast"), host_fields(svo, outs)))

        # the plain cast refilling idle lanes (svo_set_refill): park below T rays in flight
        def refilled(t):
            def run():
                lib.svo_set_refill(t)
                scene.cast(rp, hp, n, s, row_length=row)
            return run
        rf_reps = interleaved_repeats({t: refilled(t) for t in (0, 8, 16, 24, 32)}, args.steps, 3, stream, torch)
        lib.svo_set_refill(0)
        refill_sweep = {"park_below%d" % t: spread(n * world, v) for t, v in rf_reps.items()}
        if want_check:
            lib.svo_set_refill(16)
            scene.cast(rp, hp, n, s, row_length=row)
            torch.cuda.synchronize()
            lib.svo_set_refill(0)
            checks.append(("%s, refill below 16" % ("svo_cast_rows" if row else "svo_cast"), host_fields(svo, outs)))
        ws = svo.BatchWorkspace()
        items = [(scene, rp, n, hp, row)]
        cfg, sweep = autotune_batched(svo, torch, ws, items, stream)
        bms = interleaved_repeats({"b": lambda: ws.cast(items, cfg, s)}, args.steps, 1, stream, torch)["b"][0]
        variants = {"persistent_autotuned": dict({"value": round(n / (bms / 1e3) / 1e6, 3), "unit": "Mrays/s",
                                                  "ms_per_step": round(bms, 4),
                                                  "launches_per_step": batched_launches(items, cfg.sort_key)},
                                                 **cfg_record(cfg)),
                    "sweep_ms": sweep,
                    "plain_staging_depth_sweep": stage_sweep,
                    "plain_refill_sweep": refill_sweep}
        if want_check:
            checks.append(("persistent batched kernel, autotuned", host_fields(svo, outs)))
    clk = clocks.stop()

    # end to end through the host-buffer C-ABI call (pinned host memory), with the timed cast's knobs
    lib.svo_set_refill(args.refill)
    lib.svo_set_staging_depth(args.staging_depth)
    pin_cols = [torch.from_numpy(c).pin_memory() for c in cols_host]
    pin_out = {k: torch.empty(n, dtype=outs[k].dtype).pin_memory() for k in OUT_FIELDS}
    cols_np = [c.numpy() for c in pin_cols]
    out_np = {k: v.numpy().view(svo.HIT_FIELDS[k]) for k, v in pin_out.items()}
    for _ in range(max(1, args.warmup)):
        scene.cast_host_soa(cols_np, out_np, s, row_length=row)
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        scene.cast_host_soa(cols_np, out_np, s, row_length=row)
    e2e_s = max_over_ranks(time.perf_counter() - t0, pg)
    e2e_value = n * world * args.steps / e2e_s / 1e6
    if want_check:
        checks.append(("host buffers (svo_cast_host%s)" % ("_rows" if row else ""), {k: v.copy() for k, v in out_np.items()}))
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
        if want_check:
            checks.append(("host buffers, %s" % name, {k: v.copy() for k, v in out_np.items()}))
    svo.lib().svo_set_host_transfer(0)
    lib.svo_set_refill(0)
    lib.svo_set_staging_depth(0)

    # the oracle casts the whole batch once (all host threads): the CPU baseline and the parity reference
    cpu, parity = None, None
    if want_check:
        oth.join()
        tree = obox["tree"]
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        ref = tree.cast(origins, dirs, threads=threads)
        cpu_s = time.perf_counter() - t0
        # one core: every 64th ray (the same rays, so it stays a bounded sample of this batch)
        o1, d1 = np.ascontiguousarray(origins[::64]), np.ascontiguousarray(dirs[::64])
        t0 = time.perf_counter()
        tree.cast(o1, d1, threads=1)
        one_s = time.perf_counter() - t0
        cpu = {"value": round(n / cpu_s / 1e6, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
               "sample": "the whole %d-ray batch, once (%.1fs on %d threads)" % (n, cpu_s, threads),
               "single_core": {"value": round(len(o1) / one_s / 1e6, 4), "unit": "Mrays/s",
                               "sample": "every 64th ray of the batch (%d rays, %.1fs on 1 thread)" % (len(o1), one_s)}}
        parity = merge_parity([compare_hits(got, ref, label) for label, got in checks])
        del ref
    checks.clear()

    peak, peak_src = measured_peak()
    achieved = alg_bytes / (ms_step / 1e3) / 1e9
    prof = profile_traffic(workload)
    traffic = prof.get("dram_bytes_per_launch")
    l2 = None
    if prof.get("l2_bytes_per_launch"):
        l2 = {"bytes_per_launch": prof["l2_bytes_per_launch"],
              "gbs": round(prof["l2_bytes_per_launch"] / (ms_step / 1e3) / 1e9, 1),
              "hit_rate_pct": prof.get("l2_hit_rate_pct"), "l1_hit_rate_pct": prof.get("l1_hit_rate_pct"),
              "frac_of_l2_peak": (round(prof["l2_throughput_pct_of_peak"] / 100.0, 4)
                                  if prof.get("l2_throughput_pct_of_peak") is not None else None),
              "source": "ncu capture of one launch (profiles/); gbs with this run's kernel time"}
    io_bytes = n * 24 + n * sum(OUT_BYTES.values())
    st = scene.stats()
    rec = {
        "metric": "Mrays/s", "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload, "octree": "%d^3" % w["size"], "brick_dim": w["brick_dim"],
                   "rays_per_step": n, "hit_rate": round(hits / n, 4), "nodes": st["nodes"],
                   "per_ray": {"node_visits": round(visits / n, 2), "child_reads": round(creads / n, 2),
                               "voxel_reads": round(vreads / n, 2), "restart_run_visits": round(runs / n, 2)},
                   "parted_bricks": st["parted_bricks"], "voxels_inserted": int(len(ops)),
                   "l2": "inputs larger than L2 (rays %.0f MB + hits %.0f MB per step); the %.0f MB scene image "
                         "stays resident" % (n * 24 / 1e6, n * sum(OUT_BYTES.values()) / 1e6, st["device_bytes"] / 1e6),
                   "build_s": round(build_s, 1), "parallelism": "replicas" if world > 1 else "single",
                   "ray_order": ("rows of %d rays (svo_cast_rows: 8 x 4 ray blocks per warp)" % row) if row
                   else "as generated (svo_cast)",
                   "timed_cast_knobs": {"refill_park_below": args.refill, "staging_depth": args.staging_depth},
                   "svo_cast_plain_order": plain},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_src,
                     "alg_bytes_per_launch": alg_bytes, "alg_bytes_per_ray": round(alg_bytes / n, 2),
                     "io_bytes_per_launch": io_bytes,
                     "io_note": "rays in (24 B) and hit fields out (34 B) per ray: DRAM traffic that the "
                                "algorithmic bytes (scene reads) do not count", "l2": l2},
        "cpu_baseline": cpu,
        "e2e": {"value": round(e2e_value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": n * 24,
                "d2h_bytes_per_step": n * sum(OUT_BYTES.values()), "paths": e2e_paths},
        "gpu_launches": args.steps,
        "clocks": clk,
        "variants": variants,
        "parity": parity,
    }
    del outs, rays_dev
    torch.cuda.empty_cache()
    return rec, pg


# ---- comparison (a): incoherent rays, plain cast vs batched forms ---------------------------------
def compare_incoherent(args):
    """incoherent1024: plain svo_cast against the autotuned persistent batched cast in index order and
    with the ray sort, timed over interleaved repeats, every variant's hits checked against the oracle."""
    import torch
    import shocovox_gb300 as svo
    w = WORKLOADS["incoherent1024"]
    dev = torch.device("cuda", 0)
    t0 = time.perf_counter()
    ops = scene_ops(svo, w)
    oth, obox = oracle_tree_async(ops, w)
    scene = svo.Octree(w["size"], w["brick_dim"])
    scene.apply_ops(ops)
    build_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream(dev)
    s = stream.cuda_stream
    scene.upload(s)
    origins, dirs = make_rays(svo, w)
    n = len(origins)
    rays = {k: torch.from_numpy(np.ascontiguousarray(a[:, i])).to(dev)
            for a, names in ((origins, RAY_KEYS[:3]), (dirs, RAY_KEYS[3:])) for i, k in enumerate(names)}
    rp = {k: v.data_ptr() for k, v in rays.items()}
    outs = {v: device_outputs(torch, svo, n, dev, OUT_FIELDS) for v in ("plain", "index_order", "sorted", "refill")}
    hp = {v: {k: t.data_ptr() for k, t in o.items()} for v, o in outs.items()}
    ws = svo.BatchWorkspace()
    items = {v: [(scene, rp, n, hp[v], 0)] for v in ("index_order", "sorted")}
    best, sweeps = {}, {}
    for v, key in (("index_order", 0), ("sorted", 1)):
        best[v], sweeps[v] = autotune_batched(svo, torch, ws, items[v], stream, fixed_sort=key)
    lib = svo.lib()

    def plain_cast(t, out):  # svo_cast, refilling idle lanes below t rays in flight (0: never)
        def run():
            lib.svo_set_refill(t)
            scene.cast(rp, hp[out], n, s)
        return run
    # the refill threshold: a short sweep
    t_sweep = interleaved_repeats({t: plain_cast(t, "refill") for t in (8, 16, 24, 32)}, max(2, args.steps // 4), 1,
                                  stream, torch)
    t_best = min(t_sweep, key=lambda t: t_sweep[t][0])
    clocks = ClockSampler(0).start()
    for _ in range(args.warmup):
        plain_cast(0, "plain")()
    reps = interleaved_repeats({"plain": plain_cast(0, "plain"),
                                "refill": plain_cast(t_best, "refill"),
                                "index_order": lambda: ws.cast(items["index_order"], best["index_order"], s),
                                "sorted": lambda: ws.cast(items["sorted"], best["sorted"], s)},
                               args.steps, REPEATS, stream, torch)
    lib.svo_set_refill(0)
    clk = clocks.stop()
    got = {v: host_fields(svo, o) for v, o in outs.items()}
    oth.join()
    t0 = time.perf_counter()
    ref = obox["tree"].cast(origins, dirs, threads=os.cpu_count() or 1)
    cpu_s = time.perf_counter() - t0
    parity = merge_parity([compare_hits(got[v], ref, v) for v in got])
    plain = spread(n, reps["plain"])
    res = {"svo_cast": plain,
           "svo_cast_refill": dict(spread(n, reps["refill"]), park_below=t_best, vs_plain=versus(spread(n, reps["refill"]), plain),
                                   sweep_ms={"park_below%d" % t: round(v[0], 4) for t, v in t_sweep.items()})}
    for v in ("index_order", "sorted"):
        c = best[v]
        res["batched_" + v] = dict(spread(n, reps[v]), launches_per_step=batched_launches(items[v], c.sort_key),
                                   vs_plain=versus(spread(n, reps[v]), plain), autotune_sweep_ms=sweeps[v],
                                   **cfg_record(c))
    del outs, rays
    torch.cuda.empty_cache()
    return {"workload": "incoherent1024 (1024^3, brick 8, ~5% occupancy, 2^22 rays from the bounding sphere in "
                        "uniform directions)", "rays_per_step": n, "unit": "Mrays/s", "build_s": round(build_s, 1),
            "steps_per_repeat": args.steps, "variants": res,
            "l2": "rays 100 MB + hit fields 143 MB per step (larger than L2)",
            "cpu_oracle": {"value": round(n / cpu_s / 1e6, 3), "unit": "Mrays/s", "cores": os.cpu_count() or 1},
            "parity": parity, "clocks": clk}


# ---- comparison (b): many scenes in one persistent launch ------------------------------------------
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
    """Batched multi-scene cast: serial plain dispatch vs one persistent launch vs that launch in a CUDA
    graph, repeated; every item's hits checked against the oracle's cast of the same rays."""
    import concurrent.futures as cf
    import torch
    import shocovox_gb300 as svo
    from oracle import oracle
    from shocovox_gb300 import autotune
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    specs = multiscene_specs(w)
    workers = min(16, os.cpu_count() or 4)
    t0 = time.perf_counter()

    def ops_of(sp):
        return svo.gen_scene(sp["kind"], sp["size"], sp["brick_dim"], sp["seed"], occupancy=sp["occupancy"],
                             spheres=sp["spheres"], octaves=sp["octaves"], base_freq=sp["base_freq"])

    all_ops = [ops_of(sp) for sp in specs]
    gen_s = time.perf_counter() - t0

    def build(i):
        t = svo.Octree(specs[i]["size"], specs[i]["brick_dim"])
        t.apply_ops(all_ops[i])
        return t

    def build_oracle(i):
        t = oracle.Tree(specs[i]["size"], specs[i]["brick_dim"])
        t.apply_ops(all_ops[i])
        return t

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        built = list(ex.map(build, range(len(specs))))
    build_s = time.perf_counter() - t0
    n_voxels = int(sum(len(o) for o in all_ops))
    # the oracle trees build on the host threads while the GPU runs
    opool = None
    ofut = None
    if not args.no_parity:
        opool = cf.ThreadPoolExecutor(max_workers=workers)
        ofut = [opool.submit(build_oracle, i) for i in range(len(specs))]
    stream = torch.cuda.current_stream(dev)
    s = stream.cuda_stream
    # one batch: every ray column and hit field is one buffer over all scenes, each scene a slice
    host_rays = [multiscene_rays(svo, sp) for sp in specs]
    counts = [len(r[0]) for r in host_rays]
    begins = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    total = int(begins[-1])
    all_o = np.concatenate([r[0] for r in host_rays])
    all_d = np.concatenate([r[1] for r in host_rays])
    host_cols = [np.ascontiguousarray(all_o[:, i]) for i in range(3)] + [np.ascontiguousarray(all_d[:, i]) for i in range(3)]
    dev_cols = {k: torch.from_numpy(c).to(dev) for k, c in zip(RAY_KEYS, host_cols)}
    dev_out = device_outputs(torch, svo, total, dev, OUT_FIELDS)
    # per scene two items: its camera rays (rows of the image: cast in 8 x 4 ray blocks) and its
    # random rays
    items = []
    for i, t in enumerate(built):
        t.upload(s)
        a, b = int(begins[i]), int(begins[i + 1])
        ncam, row = host_rays[i][2], host_rays[i][3]
        for lo, hi, r in ((a, a + ncam, row), (a + ncam, b, 0)):
            if hi > lo:
                items.append((t, {k: v[lo:hi].data_ptr() for k, v in dev_cols.items()}, hi - lo,
                              {k: v[lo:hi].data_ptr() for k, v in dev_out.items()}, r))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def serial():
        for (t, rp, n, hp, row) in items:
            t.cast(rp, hp, n, s, row_length=row)

    ws = svo.BatchWorkspace()

    def time_cfg(c):
        ws.cast(items, c, s)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(2):
            ws.cast(items, c, s)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 2

    cfg, tune_info = autotune.tune(ws, items, torch.cuda.get_device_name(0), time_cfg)

    def batched():
        ws.cast(items, cfg, s)

    checks = []
    serial()
    torch.cuda.synchronize()
    checks.append(("serial plain launches", host_fields(svo, dev_out)))
    dev_out_clear(dev_out)
    batched()
    torch.cuda.synchronize()
    checks.append(("one batched launch", host_fields(svo, dev_out)))
    # one persistent launch captured in a CUDA graph (workspace already sized, blocks per SM fixed)
    gcfg = cfg  # blocks per SM from occupancy when the call is captured, fixed in the graph
    gws = svo.BatchWorkspace()  # the graph keeps its own workspace: later casts on `ws` leave it alone
    gstream = torch.cuda.Stream(dev)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(gstream):
        gws.cast(items, gcfg, gstream.cuda_stream)
        torch.cuda.synchronize()
        with torch.cuda.graph(graph, stream=gstream):
            gws.cast(items, gcfg, gstream.cuda_stream)
    torch.cuda.synchronize()
    dev_out_clear(dev_out)
    graph.replay()
    torch.cuda.synchronize()
    checks.append(("batched launch replayed from a CUDA graph", host_fields(svo, dev_out)))

    clocks = ClockSampler(0).start()
    for _ in range(args.warmup):
        serial()
        batched()
        graph.replay()
    torch.cuda.synchronize()
    reps = interleaved_repeats({"serial": serial, "batched": batched, "graph": graph.replay}, args.steps,
                               REPEATS, stream, torch)
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
    del cnt

    # end to end: host rays in, batched launches, host hits out (pinned buffers, copies in the timed region):
    # the batch cut into 4 groups of consecutive items, each copy-in, launch and copy-out on its own stream
    # with its own workspace, so one group's copies overlap another group's launch
    pin_in = {k: torch.from_numpy(c).pin_memory() for k, c in zip(RAY_KEYS, host_cols)}
    pin_out = {k: torch.empty(total, dtype=v.dtype).pin_memory() for k, v in dev_out.items()}
    base = dev_cols["ox"].data_ptr()
    offs = [(it[1]["ox"] - base) // 4 for it in items]
    n_groups, groups, cur_g, acc = 4, [], [], 0
    for it, off in zip(items, offs):
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
                for k in RAY_KEYS:
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
    checks.append(("host buffers, 4 pipelined groups", {k: v.numpy().view(svo.HIT_FIELDS[k]).copy()
                                                        for k, v in pin_out.items()}))

    # every item against the oracle's cast of its rays
    parity, cpu = None, None
    if ofut is not None:
        trees = [f.result() for f in ofut]
        opool.shutdown()
        threads = os.cpu_count() or 1
        ref = {k: np.zeros(total, dtype=t) for k, t in oracle.HIT_FIELDS.items()}
        cpu_s = 0.0
        for i, tr in enumerate(trees):
            a, b = int(begins[i]), int(begins[i + 1])
            t0 = time.perf_counter()
            r = tr.cast(all_o[a:b], all_d[a:b], threads=threads)
            cpu_s += time.perf_counter() - t0
            for k in ref:
                ref[k][a:b] = r[k]
        del trees
        parity = merge_parity([compare_hits(got, ref, label) for label, got in checks])
        parity["items_checked"] = len(items)
        cpu = {"value": round(total / cpu_s / 1e6, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
               "sample": "every ray of the 64 scenes, once (%.1fs on %d threads)" % (cpu_s, threads)}
    checks.clear()

    peak, peak_src = measured_peak()
    graph_sp, serial_sp, batched_sp = spread(total, reps["graph"]), spread(total, reps["serial"]), spread(total, reps["batched"])
    graph_ms = graph_sp["ms_per_step"]
    rec = {
        "metric": "Mrays/s", "value": graph_sp["value"], "unit": "Mrays/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": graph_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "multiscene64", "scenes": len(specs), "items": len(items), "rays_per_step": total,
                   "sizes": sorted({sp["size"] for sp in specs}), "brick_dims": sorted({sp["brick_dim"] for sp in specs}),
                   "voxels_inserted": n_voxels, "gen_s": round(gen_s, 1), "build_s": round(build_s, 1),
                   "l2": "rays %.0f MB + hits %.0f MB per step (larger than L2)" % (total * 24 / 1e6, total * 34 / 1e6),
                   "timed": "the batched cast replayed from a CUDA graph (one persistent launch; with sort_key 1 the "
                            "ray sort's six launches too), median of %d repeats of %d steps" % (REPEATS, args.steps),
                   "ray_order": "per scene: camera rays as rows of the image (8 x 4 ray blocks per warp), "
                                "random rays in order or sorted by direction octant and entry point (autotune.sort_key)",
                   "graph": graph_sp,
                   "serial_plain": dict(serial_sp, launches_per_step=len(items)),
                   "batched": batched_sp,
                   "graph_vs_serial": versus(graph_sp, serial_sp),
                   "autotune": dict(cfg_record(cfg), cached=tune_info["cached"], sweep_ms=tune_info.get("sweep_ms"))},
        "roofline": {"bound": "hbm", "achieved": round(alg / (graph_ms / 1e3) / 1e9, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(alg / (graph_ms / 1e3) / 1e9 / peak, 4), "traffic": None, "peak_source": peak_src,
                     "alg_bytes_per_launch": alg, "alg_bytes_per_ray": round(alg / total, 2)},
        "cpu_baseline": cpu,
        "e2e": {"value": round(total / e2e_s / 1e6, 3), "unit": "Mrays/s", "h2d_bytes_per_step": total * 24,
                "d2h_bytes_per_step": total * sum(OUT_BYTES.values()),
                "how": "4 groups of items, each copy-in, batched launch, copy-out on its own stream"},
        "gpu_launches": args.steps * batched_launches(items, gcfg.sort_key),
        "clocks": clk,
        "parity": parity,
    }
    del dev_cols, dev_out, graph
    torch.cuda.empty_cache()
    return rec


def dev_out_clear(d):
    for v in d.values():
        v.zero_()


# ---- comparison (c): served requests --------------------------------------------------------------
SERVE_STRIDE = 1024  # every request: its pixels first, first + 1024, ... are checked against the oracle
SERVE_FULL_EVERY = 500  # every 500th request also returns every hit field and is checked in full
SERVE_FIELDS = ("status", "albedo")  # what every request returns to host memory


def served_scenes(svo, w):
    rng = np.random.default_rng(w["seed"])
    sizes = [int(v) for v in rng.permutation(np.repeat([256, 512, 1024, 2048], w["served"] // 4))]
    recipes = [(S, w["seed"] + 31 * i, float(rng.uniform(0.01, 0.05))) for i, S in enumerate(sizes)]
    return rng, sizes, recipes


def served_requests(rng, sizes, w):
    n_req = w["requests"]
    arrivals = np.cumsum(rng.exponential(1.0 / w["rate"], n_req))
    reqs = []
    for _ in range(n_req):
        j = int(rng.integers(0, len(sizes)))
        S = float(sizes[j])
        a, el = rng.uniform(0, 2 * np.pi), rng.uniform(0.35, 0.7)
        eye = [S / 2 + 1.4 * S * np.cos(el) * np.cos(a), S / 2 + 1.4 * S * np.sin(el), S / 2 + 1.4 * S * np.cos(el) * np.sin(a)]
        target = [S / 2 + rng.uniform(-0.1, 0.1) * S, S / 2, S / 2 + rng.uniform(-0.1, 0.1) * S]
        wd, ht = RESOLUTIONS[int(rng.integers(0, len(RESOLUTIONS)))]
        reqs.append((j, eye, target, 60.0, wd, ht))
    return arrivals, reqs


def run_served(args, w):
    """Served load: Poisson camera requests over 16 scenes under a device budget that forces evictions,
    continuous batching vs serial dispatch, paced and at capacity, repeated; every request checked against
    the oracle on a strided sample of its pixels, every 500th request on all of its pixels and fields."""
    import concurrent.futures as cf
    import torch
    import shocovox_gb300 as svo
    from oracle import oracle
    torch.cuda.set_device(0)
    rng, sizes, recipes = served_scenes(svo, w)
    t0 = time.perf_counter()
    all_ops = [svo.gen_scene(4, S, 8, seed, occupancy=occ) for S, seed, occ in recipes]
    scenes = []
    for (S, _, _), ops in zip(recipes, all_ops):
        t = svo.Octree(S, 8)
        t.apply_ops(ops)
        scenes.append(t)
    build_s = time.perf_counter() - t0
    # device image of every scene, measured by one upload
    image = []
    for t in scenes:
        t.upload()
        image.append(int(t.stats()["device_bytes"]))
        t.release_device()
    budget = int(w["budget_frac"] * sum(image))
    arrivals, reqs = served_requests(rng, sizes, w)
    n_req = len(reqs)
    total_rays = sum(r[4] * r[5] for r in reqs)
    firsts = [(k * 7919) % SERVE_STRIDE for k in range(n_req)]
    full_ids = list(range(0, n_req, SERVE_FULL_EVERY))

    # oracle references (built and cast on host threads while nothing runs on the GPU)
    oref_sample, oref_full = None, None
    if not args.no_parity:
        def build_oracle(i):
            t = oracle.Tree(recipes[i][0], 8)
            t.apply_ops(all_ops[i])
            return t
        with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
            otrees = list(ex.map(build_oracle, range(len(scenes))))
        threads = os.cpu_count() or 1
        oref_sample = [None] * n_req
        for j, tr in enumerate(otrees):
            ks = [k for k, r in enumerate(reqs) if r[0] == j]
            if not ks:
                continue
            o_d = [oracle.gen_camera_rays_strided(reqs[k][1], reqs[k][2], reqs[k][3], reqs[k][4], reqs[k][5], firsts[k],
                                                  SERVE_STRIDE) for k in ks]
            r = tr.cast(np.concatenate([x[0] for x in o_d]), np.concatenate([x[1] for x in o_d]), threads=threads)
            at = 0
            for k, x in zip(ks, o_d):
                m = len(x[0])
                oref_sample[k] = {f: r[f][at:at + m] for f in SERVE_FIELDS}
                at += m
        oref_full = {}
        for k in full_ids:
            j, eye, target, fov, wd, ht = reqs[k]
            o, d = oracle.gen_camera_rays(eye, target, fov, wd, ht)
            oref_full[k] = otrees[j].cast(o, d, threads=threads)
        del otrees

    # pinned result buffers (SERVE_FIELDS per ray), reused round-robin by later requests; the full-record
    # requests get buffers of their own with every field
    ring = 48
    maxn = max(r[4] * r[5] for r in reqs)
    bufs = [{"status": torch.empty(maxn, dtype=torch.uint8).pin_memory().numpy(),
             "albedo": torch.empty(maxn, dtype=torch.int32).pin_memory().numpy().view(np.uint32)} for _ in range(ring)]
    full_fields = ID_FIELDS + FLOAT_FIELDS
    tnp = {np.uint8: torch.uint8, np.uint32: torch.int32, np.float32: torch.float32}
    full_bufs = {k: {f: torch.empty(reqs[k][4] * reqs[k][5], dtype=tnp[svo.HIT_FIELDS[f]]).pin_memory().numpy().view(
        svo.HIT_FIELDS[f]) for f in full_fields} for k in full_ids}

    def serve(srv, paced):
        # the Python loop below drives the native server: a collection of the interpreter's heap in the
        # middle of it (the process holds the earlier workloads' objects) would stall submissions, so the
        # heap is collected before the run and the collector is off during it
        gc.collect()
        gc.disable()
        try:
            return serve_run(srv, paced)
        finally:
            gc.enable()

    def serve_run(srv, paced):
        for t in scenes:  # every run starts with no scene resident
            t.release_device()
        ids = [srv.add_scene(t) for t in scenes]
        assert ids == list(range(len(scenes)))
        # warm-up: the launch path exercised once per scene (scenes past the budget are evicted again)
        for j in range(len(scenes)):
            srv.wait(srv.submit(j, [0.0, float(sizes[j]), 0.0], [sizes[j] / 2] * 3, 60.0, 64, 64,
                                out={k: v[:4096] for k, v in bufs[0].items()}))
        st0 = srv.stats()
        sample = [None] * n_req
        start = srv.now()
        rids, res = [], [None] * n_req

        def out_of(k):  # the host arrays request k writes
            if k in full_bufs:
                return full_bufs[k]
            return {f: v[:reqs[k][4] * reqs[k][5]] for f, v in bufs[k % ring].items()}

        def finish(k):
            res[k] = srv.wait(rids[k], 600.0)
            b = out_of(k)
            sample[k] = {f: b[f][firsts[k]::SERVE_STRIDE].copy() for f in SERVE_FIELDS}

        for k, r in enumerate(reqs):
            if k >= ring:  # the result buffers of request k - ring are reused: it must be done
                finish(k - ring)
            if paced:
                delay = start + arrivals[k] - srv.now()
                if delay > 0:
                    time.sleep(delay)
            rids.append(srv.submit(*r, out=out_of(k)))
        for k in range(max(0, n_req - ring), n_req):
            finish(k)
        if paced:  # from the scheduled arrival: a submission the loop made late still counts its wait
            lat = np.array([x["done_s"] - (start + arrivals[k]) for k, x in enumerate(res)])
        else:
            lat = np.array([x["done_s"] - x["submit_s"] for x in res])
        span = max(x["done_s"] for x in res) - (start if paced else min(x["submit_s"] for x in res))
        st = srv.stats()
        srv.close()
        checks = []
        if oref_sample is not None:
            got = {f: np.concatenate([sample[k][f] for k in range(n_req)]) for f in SERVE_FIELDS}
            ref = {f: np.concatenate([oref_sample[k][f] for k in range(n_req)]) for f in SERVE_FIELDS}
            checks.append(compare_hits(got, ref, "every request, pixels first + 1024 i (status, albedo)"))
            for k in full_ids:
                checks.append(compare_hits(full_bufs[k], oref_full[k], "request %d, every pixel and field" % k))
        return {"value": round(total_rays / span / 1e6, 3), "p50_ms": round(float(np.percentile(lat, 50)) * 1e3, 3),
                "p99_ms": round(float(np.percentile(lat, 99)) * 1e3, 3), "span_s": round(span, 3),
                "launches": st["launches"] - st0["launches"], "uploads": st["uploads"] - st0["uploads"],
                "evictions": st["evictions"] - st0["evictions"],
                "mean_batch": round(float(np.mean([x["batch_requests"] for x in res])), 2),
                "parity": merge_parity(checks)}

    clocks = ClockSampler(0, interval_ms=500).start()
    runs = {"served": [], "serial_dispatch": [], "capacity_served": [], "capacity_serial_dispatch": []}
    for _ in range(w["repeats"]):
        # paced: launches of at most 4 M rays keep a large request from delaying the next ones
        runs["served"].append(serve(svo.Server(budget_bytes=budget, max_batch_requests=64, max_batch_rays=1 << 22,
                                               max_inflight=3), paced=True))
        runs["serial_dispatch"].append(serve(svo.Server(budget_bytes=budget, max_batch_requests=1, max_inflight=1),
                                             paced=True))
        # capacity: the same requests submitted as fast as result buffers free up (48 outstanding)
        runs["capacity_served"].append(serve(svo.Server(budget_bytes=budget, max_batch_requests=64,
                                                        max_batch_rays=1 << 25, max_inflight=3), paced=False))
        runs["capacity_serial_dispatch"].append(serve(svo.Server(budget_bytes=budget, max_batch_requests=1,
                                                                 max_inflight=1), paced=False))
    clk = clocks.stop()

    def summary(rs):
        v = np.array([r["value"] for r in rs])
        return {"value": round(float(np.median(v)), 3), "min": round(float(v.min()), 3), "max": round(float(v.max()), 3),
                "p50_ms": round(float(np.median([r["p50_ms"] for r in rs])), 3),
                "p99_ms": round(float(np.median([r["p99_ms"] for r in rs])), 3),
                "p99_ms_per_repeat": [r["p99_ms"] for r in rs], "repeats": len(rs),
                "uploads": [r["uploads"] for r in rs], "evictions": [r["evictions"] for r in rs],
                "launches": [r["launches"] for r in rs], "span_s": [r["span_s"] for r in rs],
                "mean_batch": [r["mean_batch"] for r in rs]}

    sm = {k: summary(v) for k, v in runs.items()}
    parity = merge_parity([r["parity"] for v in runs.values() for r in v])
    srv_ = sm["served"]
    return {
        "metric": "Mrays/s", "value": srv_["value"], "unit": "Mrays/s", "n_gpus": 1, "steps": n_req,
        "warmup": len(scenes), "ms_per_step": round(float(np.median([r["span_s"] for r in runs["served"]])) / n_req * 1e3, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "served16", "scenes": len(scenes), "sizes": sizes, "requests": n_req,
                   "arrival_rate_per_s": w["rate"], "rays": total_rays, "build_s": round(build_s, 1),
                   "scene_image_bytes": image, "budget_bytes": budget,
                   "budget": "half the sum of the 16 scene images, so scenes are evicted and uploaded again while "
                             "requests run (the box-recipe scenes total %.1f MB)" % (sum(image) / 1e6),
                   "outputs": "status + albedo of every pixel to pinned host memory; every %dth request also every "
                              "hit field" % SERVE_FULL_EVERY,
                   "latency": "paced: scheduled arrival -> result in host memory; capacity: submission -> result",
                   "server_config": {"served": "max_batch_requests 64, max_batch_rays 2^22, max_inflight 3",
                                     "capacity_served": "max_batch_requests 64, max_batch_rays 2^25, max_inflight 3",
                                     "serial_dispatch": "max_batch_requests 1, max_inflight 1 (one request per launch)"},
                   "served": srv_, "serial_dispatch": sm["serial_dispatch"],
                   "capacity_served": sm["capacity_served"], "capacity_serial_dispatch": sm["capacity_serial_dispatch"],
                   "served_vs_serial": versus(sm["served"], sm["serial_dispatch"]),
                   "capacity_vs_serial": versus(sm["capacity_served"], sm["capacity_serial_dispatch"]),
                   "p50_ms": srv_["p50_ms"], "p99_ms": srv_["p99_ms"]},
        "roofline": None, "cpu_baseline": None,
        "e2e": {"value": srv_["value"], "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(total_rays * 5 / n_req)},
        "gpu_launches": srv_["launches"][0] if srv_["launches"] else 0, "clocks": clk,
        "parity": parity,
    }


# ---- f2 / f3 workloads --------------------------------------------------------------------------
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
    clocks = ClockSampler(0).start()
    for _ in range(args.warmup):
        render()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        render()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    frames = img.cpu().numpy()
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
    rays = {k: torch.from_numpy(c).to(dev) for k, c in zip(RAY_KEYS, cols)}
    rp = {k: v.data_ptr() for k, v in rays.items()}
    outs = device_outputs(torch, svo, n, dev, ("status", "albedo", "nx", "ny", "nz"))
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

    cpu, parity = None, None
    if not args.no_parity:
        from oracle import oracle
        ot = oracle.Tree(w["size"], w["brick_dim"])
        ot.apply_ops(ops)
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        ref_frames = []
        bad_ref = 0
        for vp in vps:
            d = {"origin": list(vp.origin), "direction": list(vp.direction), "up": list(vp.up), "width": vp.width,
                 "height": vp.height, "fov": vp.fov, "light": list(vp.light), "background": vp.background}
            fr, b = ot.render_viewport(d, W, H, threads=threads)
            ref_frames.append(fr)
            bad_ref += b
        cpu_s = time.perf_counter() - t0
        mism = int(np.any(np.stack(ref_frames) != frames, axis=-1).sum())
        parity = {"pixels_checked": n, "mismatches": mism, "unshaded_pixels_oracle": int(bad_ref),
                  "what": "every RGBA8 pixel of the 4 frames against the oracle's restatement of cpu_render.rs"}
        cpu = {"value": round(n / cpu_s / 1e6, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
               "sample": "the 4 frames rendered once (%.1fs on %d threads)" % (cpu_s, threads)}
    peak, peak_src = measured_peak()
    achieved = alg / (ms / 1e3) / 1e9
    return {
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
                     "frac": round(achieved / peak, 4), "traffic": profile_traffic("viewport512").get("dram_bytes_per_launch"),
                     "peak_source": peak_src, "alg_bytes_per_launch": alg, "alg_bytes_per_ray": round(alg / n, 2)},
        "cpu_baseline": cpu,
        "e2e": {"value": round(n / e2e_s / 1e6, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": n * 4,
                "paths": {"one_launch_then_copy": round(n / e2e_one_s / 1e6, 3),
                          "two_streams_of_two_frames": round(n / e2e_pairs_s / 1e6, 3)}},
        "gpu_launches": args.steps, "clocks": clk, "parity": parity,
    }


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
    rays = {k: torch.from_numpy(c).to(dev) for k, c in zip(RAY_KEYS, cols)}
    rp = {k: v.data_ptr() for k, v in rays.items()}
    out = device_outputs(torch, svo, n, dev, OUT_FIELDS)
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
    clocks = ClockSampler(0).start()
    ms = timed(lambda: scene.cast_lod(rp, hp, n, vd, s, row_length=row))
    timed_out = host_fields(svo, out)
    max_ms = timed(lambda: scene.cast_lod(rp, hp, n, float(np.finfo(np.float32).max), s, row_length=row))
    plain_ms = timed(lambda: scene.cast(rp, hp, n, s, row_length=row))
    lod_plain_order_ms = timed(lambda: scene.cast_lod(rp, hp, n, vd, s))
    # end to end: rays from pinned host memory, status + albedo back, copies in the timed region
    pin_in = {k: torch.from_numpy(c).pin_memory() for k, c in zip(RAY_KEYS, cols)}
    pin_out = {k: torch.empty(n, dtype=out[k].dtype).pin_memory() for k in ("status", "albedo")}

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
    cpu, parity = None, None
    if not args.no_parity:
        from oracle import oracle
        ot = oracle.Tree(w["size"], w["brick_dim"])
        ot.apply_ops(ops)
        ot.mip_switch(True)
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        ref = ot.cast(origins, dirs, threads=threads, viewing_distance=vd)
        cpu_s = time.perf_counter() - t0
        parity = merge_parity([compare_hits(timed_out, ref, "timed svo_cast_lod_rows launch")])
        cpu = {"value": round(n / cpu_s / 1e6, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
               "sample": "the whole %d-ray batch, once (%.1fs on %d threads)" % (n, cpu_s, threads)}
    peak, peak_src = measured_peak()
    achieved = alg / (ms / 1e3) / 1e9
    st_ = scene.stats()
    return {
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
                     "frac": round(achieved / peak, 4), "traffic": profile_traffic("lod512").get("dram_bytes_per_launch"),
                     "peak_source": peak_src, "alg_bytes_per_launch": alg, "alg_bytes_per_ray": round(alg / n, 2)},
        "cpu_baseline": cpu,
        "e2e": {"value": round(n / e2e_s / 1e6, 3), "unit": "Mrays/s", "h2d_bytes_per_step": n * 24,
                "d2h_bytes_per_step": n * 5,
                "how": "per camera image on its own stream: rays in, svo_cast_lod_rows, status + albedo out"},
        "gpu_launches": args.steps, "clocks": clk, "parity": parity,
    }


# ---- the reference arm: the oracle's CPU cast, no product code -----------------------------------
def product_code_loaded():
    """Whether this process has the product package imported or its library mapped."""
    if any(m == "shocovox_gb300" or m.startswith("shocovox_gb300.") for m in sys.modules):
        return True
    try:
        with open("/proc/self/maps") as f:
            return "libsvo.so" in f.read()
    except OSError:
        return False


def run_reference(args, w):
    rank, _, world = dist_env()
    if rank != 0:
        return
    from oracle import oracle
    t0 = time.perf_counter()
    ops = scene_ops(oracle, w)  # the oracle's own generators: the same ops and rays, no product code
    tree = oracle.Tree(w["size"], w["brick_dim"])
    tree.apply_ops(ops)
    origins, dirs = make_rays(oracle, w)
    setup_s = time.perf_counter() - t0
    threads = os.cpu_count() or 1
    n = len(origins)
    for _ in range(args.warmup):
        tree.cast(origins, dirs, threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        tree.cast(origins, dirs, threads=threads)
    dt = time.perf_counter() - t0
    value = n * args.steps / dt / 1e6
    sample = "the whole %d-ray batch every step (oracle scene, rays and tree built in %.1fs)" % (n, setup_s)
    print(json.dumps({
        "impl": "reference", "metric": "Mrays/s", "value": round(value, 4), "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "rays_per_step": n, "voxels_inserted": int(len(ops)),
                   "note": "CPU oracle cast (a restatement of the reference's get_by_ray; the Rust crate cannot be "
                           "built here), all host threads, scene and rays from the oracle's generators",
                   "product_code_loaded": product_code_loaded()},
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
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle checks (and the CPU baseline)")
    ap.add_argument("--no-comparisons", action="store_true",
                    help="skip the incoherent1024 / multiscene64 / served16 comparisons of the default run")
    ap.add_argument("--no-variants", action="store_true", help="skip the persistent-kernel autotune sweep")
    ap.add_argument("--refill", type=int, default=0,
                    help="svo_set_refill for the timed plain cast: park a warp's rays below this many in flight")
    ap.add_argument("--staging-depth", type=int, default=0,
                    help="svo_set_staging_depth for the timed plain cast: top levels staged in shared memory")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        if "multi" in w or "served" in w or "viewport" in w or "lod" in w:
            print(json.dumps({"impl": "reference", "unavailable": "the reference arm times the single-scene workloads "
                                                                  "(terrain512, heightfield128, incoherent1024)"}))
            return
        run_reference(args, w)
        return
    pg = None
    if "multi" in w:
        rec = run_multiscene(args, w)
    elif "served" in w:
        rec = run_served(args, w)
    elif "viewport" in w:
        rec = run_viewport(args, w)
    elif "lod" in w:
        rec = run_lod(args, w)
    else:
        rec, pg = run_single(args, w, args.workload)
        _, _, world = dist_env()
        if args.workload == "terrain512" and world == 1 and not args.no_comparisons:
            ns = {}
            # served16 before multiscene64: after the 64-scene workload, the serving loop in the same process
            # ran 15-20% slower (measured, cause not found), which a process of its own does not show
            for name, fn in (("incoherent1024", lambda: compare_incoherent(args)),
                             ("served16", lambda: run_served(args, WORKLOADS["served16"])),
                             ("multiscene64", lambda: run_multiscene(args, WORKLOADS["multiscene64"]))):
                try:
                    ns[name] = fn()
                except Exception as e:  # recorded in the line (and fails the run), the other parts still report
                    ns[name] = {"error": "%s: %s" % (type(e).__name__, e)}
            rec["comparisons"] = ns
    rank, _, _ = dist_env()
    if rank == 0:
        print(json.dumps(rec))
    if pg:
        pg.destroy_process_group()
    if parity_failed(rec):
        sys.stderr.write("bench: a result differs from the oracle (see the parity records)\n")
        sys.exit(1)


if __name__ == "__main__":
    main()
