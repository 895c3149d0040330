"""Benchmark: path samples/s of the GB300 path tracer on the 1.31M-triangle
displaced-icosphere scene (1024x1024, 64 spp, max depth 16, procedural sky),
plus the reference CPU path (the oracle restatement) timed on the host.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

A step is one full render of the scene: 1024*1024*64 = 67,108,864 path
samples through PathTracingMIS.  `value` is measured with the scene and the
film resident in device memory; `e2e` is the same render through the C ABI
into a host film buffer (device->host film copy and the per-call host->device
uploads inside the timed region).  Multi-GPU runs are weak-scaled replicas:
rank r renders the same image with its own sample indices [r*spp, (r+1)*spp),
no collective in the timed region.
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

CONFIG = dict(level=8, width=1024, height=1024, spp=64, max_depth=16, env=(1024, 512), seed=0)
# --workload volume: 128^3 fBm grid medium + homogeneous slab + sphere light, VolPathTracing
VOLUME = dict(volume=True, width=512, height=512, spp=128, max_depth=64, res=128, seed=0)
VOLUME_WORKLOAD = "volume_grid_128cube_fbm_slab_spherelight_512x512_128spp_depth64"
# --workload smooth: the Cornell room furnished with every BSDF family but
# RoughDielectric: Conductor tall box, Dielectric short box, Mirror sphere,
# TwoSides Diffuse and RoughConductor panels, LayeredBSDF left wall,
# SmoothLayered right wall; PathTracingMIS
SMOOTH = dict(smooth=True, width=1024, height=1024, spp=16, max_depth=12, seed=0)
SMOOTH_WORKLOAD = "cornell_smooth_bsdfs_1024x1024_16spp_depth12"
# --small: the same scene at 512x512, 8 spp, for profiler captures only
SMALL = dict(width=512, height=512, spp=8)
WORKLOAD = "displaced_icosphere_1310720tri_1024x1024_64spp_depth16_sky1024x512"
METRIC = "path samples/s"
UNIT = "samples/s"
S_NODE = {8: 80,   # bytes per compressed 8-wide node fetch (origin, exponents, links, 8 quantised boxes)
          4: 112,  # bytes per 4-wide node fetch (four child boxes + links; the 16-byte pad is not read)
          2: 64}   # bytes per BVH2 node fetch (two child boxes + links)
S_TRI = 36         # bytes per triangle test (three float3 vertices)
S_RAY_IN = 32      # origin, direction, tmin, tmax
S_HIT_OUT = 16     # t, u, v, triangle id


def _peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi sampling during the timed region.  Start it before the
    warm-up (nvidia-smi takes a moment to print its first row) and bracket the
    timed region with begin() / end(): only rows stamped inside it count, or,
    for a region shorter than the sampling interval, the rows next to it."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None
        self.window = None

    def begin(self):
        self.window = [time.time(), None]

    def end(self):
        if self.window:
            self.window[1] = time.time()

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.time(), [c.strip() for c in line.split(",")]))

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        rows = self.rows
        if self.window and self.window[1] is not None and rows:
            a, b = self.window
            inside = [r for t, r in rows if a <= t <= b + 0.06]
            if not inside:   # a region shorter than the interval: the rows on either side
                before = [r for t, r in rows if t < a][-1:]
                after = [r for t, r in rows if t > b][:1]
                inside = before + after
            rows = inside
        else:
            rows = [r for _, r in rows]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                for k, n in enumerate(names):
                    if r[5 + k].lower() == "active":
                        reasons.add(n)
            except Exception:
                continue
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _workload_name():
    if CONFIG.get("volume"):
        return VOLUME_WORKLOAD
    if CONFIG.get("smooth"):
        return SMOOTH_WORKLOAD
    return WORKLOAD


def make_scene():
    from raytracer_gb300 import scenes, desc as D
    if CONFIG.get("smooth"):
        s = scenes.cornell_smooth(CONFIG["width"], CONFIG["height"], max_depth=CONFIG["max_depth"])
        s.meshes[1]["bsdf"] = s.add_bsdf(D.bsdf(D.BSDF_LAYERED, eta=(1.1, 0.9, 0.7), k=(3.0, 2.5, 2.0)))
        s.meshes[2]["bsdf"] = s.add_bsdf(D.bsdf(D.BSDF_SMOOTH_LAYERED, albedo=(0.12, 0.45, 0.15), eta_int=1.5))
        return s
    if CONFIG.get("volume"):
        return scenes.volume_grid(CONFIG["width"], CONFIG["height"], res=CONFIG["res"], seed=CONFIG["seed"],
                                  max_depth=CONFIG["max_depth"])
    return scenes.displaced_icosphere(level=CONFIG["level"], width=CONFIG["width"], height=CONFIG["height"],
                                      seed=CONFIG["seed"], env_size=CONFIG["env"], max_depth=CONFIG["max_depth"])


def _config(data):
    """The workload, identical in both arms' JSON lines: the scene, the
    render and how the timed inputs relate to L2."""
    W, H = CONFIG["width"], CONFIG["height"]
    return {"workload": _workload_name(),
            "integrator": "VolPathTracing" if CONFIG.get("volume") else "PathTracingMIS",
            "triangles": data.n_triangles, "resolution": [W, H], "spp": CONFIG["spp"],
            "max_depth": CONFIG["max_depth"], "samples_per_step": W * H * CONFIG["spp"],
            "filter": getattr(_ARGS, "filter", "box"),
            "parallelism": "replicas" if int(os.environ.get("WORLD_SIZE", "1")) > 1 else "single",
            "l2": "inputs larger than L2: the scene (BVH, triangles, materials, maps) and the wavefront path "
                  "state (246 bytes per path in flight, 342 for VolPathTracing) live in HBM"}


_ARGS = None


def _tile_sample(ntiles, n, tiles_x):
    """n tiles spread evenly over the job grid: tiles t0 + k * stride in
    raster order with the stride about ntiles / n and coprime with the grid
    width, so the sample walks a diagonal lattice through every row band and
    column (sky, sphere and ground in proportion), not the frame's centre."""
    import math
    n = max(1, min(n, ntiles))
    stride = max(1, ntiles // n)
    while stride > 1 and math.gcd(stride, tiles_x) != 1:
        stride -= 1
    t0 = stride // 2
    n = min(n, (ntiles - 1 - t0) // stride + 1)
    return t0, n, stride


def cpu_oracle_rate(scene, target_s=15.0, threads=None):
    """Time the CPU oracle (the reference path restated in C) on a bounded
    sample: whole 32x32 tiles at the full spp, spread evenly over the frame,
    as many as take about target_s."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    threads = threads or os.cpu_count() or 1
    t0 = time.time()
    o = O.OracleScene(scene)
    build_s = time.time() - t0
    W, H = scene.camera["width"], scene.camera["height"]
    tiles_x = (W + 31) // 32
    ntiles = tiles_x * ((H + 31) // 32)
    # calibration on a spread sample of one tile per thread
    cal0, cal, cstride = _tile_sample(ntiles, max(1, min(threads, 16)), tiles_x)
    t0 = time.time()
    o.render_tiles_strided(CONFIG["spp"], cal0, cal, cstride, seed=1, threads=threads)
    dt = max(time.time() - t0, 1e-3)
    per_tile = dt / cal * min(threads, cal) / threads
    n = int(max(threads, min(ntiles, target_s / max(per_tile, 1e-4))))
    tile0, n, stride = _tile_sample(ntiles, n, tiles_x)
    return o, tile0, n, stride, build_s


def _sample_desc(tile0, n, stride, ntiles, spp, threads, extra=""):
    return ("%d of %d 32x32 tiles spread over the frame (tiles %d + %d k), %d path samples, full %d spp, "
            "%d threads%s" % (n, ntiles, tile0, stride, n * 32 * 32 * spp, spp, threads, extra))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    scene = make_scene()
    threads = os.cpu_count() or 1
    o, tile0, n, stride, build_s = cpu_oracle_rate(scene, target_s=args.cpu_seconds)
    spp = CONFIG["spp"]
    for _ in range(max(0, min(args.warmup, 1))):
        o.render_tiles_strided(spp, tile0, max(1, n // 8), stride, seed=3, threads=threads)
    times = []
    for k in range(args.steps):
        t0 = time.time()
        o.render_tiles_strided(spp, tile0, n, stride, seed=4 + k, threads=threads)
        times.append(time.time() - t0)
    samples = n * 32 * 32 * spp
    value = samples * len(times) / sum(times)
    W, H = CONFIG["width"], CONFIG["height"]
    ntiles = ((W + 31) // 32) * ((H + 31) // 32)
    sample_desc = _sample_desc(tile0, n, stride, ntiles, spp, threads, " per step")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * float(np.mean(times)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded scene generator, no dataset)",
            "config": _config(scene),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample_desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "notes": "reference CPU path = the oracle's C restatement of the integrator with the reference's "
                     "two-level SAH BVH, whose per-path radiance is bit-identical to the reference's own "
                     "PathTracingMIS compiled from its sources (pin tests); the GPU machine has no copy of "
                     "those sources, so the restatement is what runs everywhere; oracle scene build %.1f s "
                     "not timed" % build_s}
    print(json.dumps(line))


def batched_block(ctx_factory, n_jobs=64):
    """The 64-scene batch (its jobs' scenes, resolutions and sample counts
    from the batch distribution), rendered into device films allocated once:
    one rt_render per job one after the other (plain) against rt_batch_render
    as one multi-scene wavefront.  Films compared bit for bit."""
    import torch
    import raytracer_gb300 as R
    t0 = time.time()
    jobs = _batch_jobs(n_jobs)
    ctx = ctx_factory()
    scs = [R.Scene(ctx, s) for s, _ in jobs]
    prep = time.time() - t0
    work = [(g, spp, dict(seed=k)) for k, (g, (_, spp)) in enumerate(zip(scs, jobs))]
    total = sum(g.width * g.height * spp for g, spp, _ in work)
    dev = [torch.zeros((g.height, g.width, 4), dtype=torch.float32, device="cuda") for g, _, _ in work]
    ptrs = [f.data_ptr() for f in dev]

    def timed(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t

    def plain_run():
        for (g, spp, o), p in zip(work, ptrs):
            g.render(spp, film=p, **o)
    plain_run()
    plain_s = min(timed(plain_run), timed(plain_run))
    plain = [f.cpu().numpy().copy() for f in dev]
    ctx.set_tuning(batch_wavefront=1)
    ctx.batch_render(work, device_films=ptrs)
    wave_s = min(timed(lambda: ctx.batch_render(work, device_films=ptrs)) for _ in range(2))
    same = all(np.array_equal(f.cpu().numpy(), p) for f, p in zip(dev, plain))
    for g in scs:
        g.close()
    ctx.close()
    return {"jobs": len(work), "total_samples": total, "plain_samples_per_s": total / plain_s,
            "batched_samples_per_s": total / wave_s, "speedup": plain_s / wave_s, "films_equal": same,
            "form": "one multi-scene wavefront (rt_batch_render, batch_wavefront=1) vs one rt_render per job",
            "prep_s": round(prep, 1)}


def served_block(ctx_factory, rate=5.0, n_jobs=30, pool_pt=8, target=0.02, cap=4096):
    """Served jobs at one Poisson arrival rate: continuous batching against
    one job at a time, same arrivals, p50/p99 latency to completion (time to
    target) and the true RMSE of the finished films against 4096-spp GPU
    renders, on the displayed image (pixel means clipped to [0, 1])."""
    ctx = ctx_factory()
    pool, refs = _serve_pool(ctx, pool_pt, 2)
    rng = np.random.default_rng(7)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_jobs))
    picks = [(int(pool_pt + rng.integers(2)) if rng.random() < 0.2 else int(rng.integers(pool_pt)), j)
             for j in range(n_jobs)]
    res = {"rate_jobs_per_s": rate, "jobs": n_jobs, "target_rmse": target, "rmse_space": "display ([0, 1] clipped)",
           "spp_cap": cap, "device_budget_gb": SERVE_BUDGET / 1e9,
           "pool": "%d scenes of the batch distribution + 2 grid-medium scenes, 4096-spp references" % pool_pt}
    for form in ("plain", "batched"):
        res[form] = _serve_run(ctx, pool, refs, picks, arrivals, form, target, cap, 4)
    for g in pool:
        g.close()
    ctx.close()
    return res


def run_gpu(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from raytracer_gb300 import build as B
    B.build()
    import raytracer_gb300 as R
    t0 = time.time()
    data = make_scene()
    if args.filter != "box":
        from raytracer_gb300 import desc as D
        data.camera["filter"] = (D.gaussian_filter(1.5, 1.5) if args.filter == "gaussian"
                                 else D.mitchell_filter(2.0, 1.0))
    gen_s = time.time() - t0
    ctx = R.Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    t0 = time.time()
    scene = R.Scene(ctx, data)
    upload_s = time.time() - t0
    info = scene.info()
    W, H, spp = CONFIG["width"], CONFIG["height"], CONFIG["spp"]
    film = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    samples_per_step = W * H * spp
    batch_paths = min(samples_per_step, args.wave_paths or (1 << 26))
    sbase = rank * spp

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    ctx.set_bvh_width(args.bvh_width)
    if args.wave_paths:
        ctx.set_wave_paths(args.wave_paths)
    ctx.set_ray_sort(args.ray_sort)
    if args.sort_threshold:
        ctx.set_tuning(sort_threshold=args.sort_threshold)
    ctx.set_tuning(volpath_wavefront=args.volpath_wavefront)
    # counting pass (traversal statistics for the roofline; not timed)
    ctx.set_profiling(2)
    scene.render(8, seed=99, film=film.data_ptr())
    cstats = ctx.stats()
    pre_launches = cstats["launches"]
    # graph launches (--graphs 1) time the steps without per-kernel events;
    # the kernel split then comes from as many kernel-by-kernel profiled
    # steps after the timed region
    ctx.set_profiling(0 if args.graphs else 1)
    ctx.set_graphs(args.graphs)
    clocks = ClockSampler(local)
    clocks.start()   # before the warm-up: its first rows arrive after a moment
    for _ in range(args.warmup):
        scene.render(spp, seed=7, sample_begin=sbase, film=film.data_ptr())
        pre_launches += ctx.stats()["launches"]
    barrier()
    agg = {}
    launches = 0
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.nvtx.range_push("timed")   # profilers can select the timed launches by this range
    clocks.begin()
    e0.record(stream)
    for k in range(args.steps):
        scene.render(spp, seed=1000 + k, sample_begin=sbase, film=film.data_ptr())
        st = ctx.stats()
        launches += st["launches"]
        for key in ("trace_closest_ms", "trace_any_ms", "shade_ms", "resolve_ms", "sort_ms", "volpath_ms", "camera_ms",
                    "film_ms",
                    "closest_rays",
                    "shadow_rays", "trace_closest_launches", "trace_any_launches", "paths", "nan_samples"):
            agg[key] = agg.get(key, 0) + st[key]
    e1.record(stream)
    torch.cuda.nvtx.range_pop()
    barrier()
    clocks.end()
    clk = clocks.stop()
    if args.graphs:
        ctx.set_graphs(0)
        ctx.set_profiling(1)
        eager = {}
        for k in range(args.steps):
            scene.render(spp, seed=1000 + k, sample_begin=sbase, film=film.data_ptr())
            st = ctx.stats()
            for key in ("trace_closest_ms", "trace_any_ms", "shade_ms", "resolve_ms", "sort_ms", "volpath_ms",
                        "camera_ms", "film_ms", "trace_closest_launches", "trace_any_launches"):
                eager[key] = eager.get(key, 0) + st[key]
        agg.update(eager)
    dev_ms = e0.elapsed_time(e1)
    t_local = dev_ms / 1000.0
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([t_local], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_local = float(t.item())
    value = samples_per_step * args.steps * world / t_local
    # end to end through the C ABI with a host film: one page-locked buffer
    # that every step's film is copied into, as a host render loop reuses
    ctx.set_profiling(0)
    host_film = torch.empty((H, W, 4), dtype=torch.float32, pin_memory=True).numpy()
    barrier()
    t0 = time.perf_counter()
    for k in range(0 if args.small else args.steps):
        scene.render(spp, seed=2000 + k, sample_begin=sbase, out=host_film)
    barrier()
    e2e_s = max(time.perf_counter() - t0, 1e-9)
    e2e_value = samples_per_step * args.steps * world / e2e_s
    d2h = W * H * 16
    h2d = 64 + 4 * (len(data.lights) + 1)
    # roofline of the dominant kernel
    # single kernels (shade = the four per-BSDF shade kernels of a round)
    kern = {"trace_closest": agg["trace_closest_ms"], "trace_any": agg["trace_any_ms"],
            "resolve": agg["resolve_ms"], "shade": agg["shade_ms"] - agg["resolve_ms"], "sort": agg["sort_ms"]}
    if CONFIG.get("volume"):
        kern = {"volpath": agg["volpath_ms"]}
    dom = max(kern, key=kern.get)
    peaks, src = _peaks()
    rays_c, rays_a = agg["closest_rays"], agg["shadow_rays"]
    nodes_pr_c = cstats["nodes_closest"] / max(cstats["closest_rays"], 1)
    tris_pr_c = cstats["tris_closest"] / max(cstats["closest_rays"], 1)
    nodes_pr_a = cstats["nodes_any"] / max(cstats["shadow_rays"], 1)
    tris_pr_a = cstats["tris_any"] / max(cstats["shadow_rays"], 1)
    if dom == "trace_closest":
        per_ray = S_RAY_IN + S_HIT_OUT + nodes_pr_c * S_NODE[args.bvh_width] + tris_pr_c * S_TRI
        algo_bytes = rays_c * per_ray
        nl = agg["trace_closest_launches"]
    elif dom == "trace_any":
        per_ray = S_RAY_IN + 4 + nodes_pr_a * S_NODE[args.bvh_width] + tris_pr_a * S_TRI
        algo_bytes = rays_a * per_ray
        nl = agg["trace_any_launches"]
    elif dom in ("shade", "resolve"):
        # per path vertex: path state read + write (2 x 64 B), ray queue
        # write + read (2 x 32 B), material parameters (64 B)
        per_ray = 2 * 64 + 2 * 32 + 64
        algo_bytes = rays_c * per_ray
        nl = max(agg["trace_closest_launches"], 1)
    else:
        # persistent VolPath megakernel: path state stays in registers; the
        # streamed bytes are the camera ray and the film (the grid and the
        # BVH of 36 triangles stay in L2), so an HBM roofline says little
        per_ray = 32 + 16
        algo_bytes = agg["paths"] * per_ray
        nl = args.steps * max(1, int(round(agg["paths"] / max(args.steps, 1) / (1 << 22))))
    per_launch_bytes = algo_bytes / max(nl, 1)
    avg_launch_s = kern[dom] / 1000.0 / max(nl, 1)
    achieved = per_launch_bytes / max(avg_launch_s, 1e-12) / 1e9
    # DRAM traffic per launch: bytes per ray measured by ncu on the small
    # case of the same scene (profiles/trace_traffic.json) x rays per launch
    traffic = None
    tf = os.path.join(ROOT, "profiles", "trace_traffic.json")
    if dom in ("trace_closest", "trace_any") and args.bvh_width == 2 and not CONFIG.get("volume") \
            and os.path.exists(tf):
        try:
            tj = json.load(open(tf))
            key, rays = ("closest_bytes_per_ray", rays_c) if dom == "trace_closest" else ("any_bytes_per_ray", rays_a)
            traffic = tj[key] * rays / max(nl, 1)
        except Exception:
            traffic = None
    dram_gbs = traffic / max(avg_launch_s, 1e-12) / 1e9 if traffic is not None else None
    dram_frac = dram_gbs / peaks.get("hbm_gbs", 1) if dram_gbs is not None else None
    bound = "latency/L2" if dom in ("trace_closest", "trace_any") else "latency"
    rays_per_s = (rays_c + rays_a) * world / t_local
    res = {}
    if rank == 0 and not args.small and args.forms and not CONFIG.get("volume") and not CONFIG.get("smooth"):
        # the batched and served forms on the same GPU, after the timed region
        scene.close()
        del film
        torch.cuda.empty_cache()
        try:
            res["batched"] = batched_block(lambda: R.Context(local))
        except Exception as ex:
            res["batched"] = {"failed": str(ex)}
        try:
            res["served"] = served_block(lambda: R.Context(local))
        except Exception as ex:
            res["served"] = {"failed": str(ex)}
    if rank == 0 and not args.small:
        try:
            cpu_o, tile0, n, stride, _ = cpu_oracle_rate(data, target_s=args.cpu_seconds)
            threads = os.cpu_count() or 1
            t0 = time.time()
            cpu_o.render_tiles_strided(spp, tile0, n, stride, seed=5, threads=threads)
            cdt = time.time() - t0
            cpu_samples = n * 32 * 32 * spp
            res["cpu_baseline"] = {"value": cpu_samples / cdt, "unit": UNIT, "cores": threads, "kind": "port",
                                   "sample": _sample_desc(tile0, n, stride, ((W + 31) // 32) * ((H + 31) // 32),
                                                          spp, threads, ", %.1f s" % cdt)}
        except Exception as ex:  # the baseline never blocks the GPU line
            res["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                   "sample": "failed: %s" % ex}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded scene generator: %s; no dataset)" % (
                    "fBm grid medium" if CONFIG.get("volume") else
                    "furnished Cornell room" if CONFIG.get("smooth") else "displaced icosphere + procedural sky"),
                "config": _config(data),
                "tuning": {"bvh_width": args.bvh_width, "graphs": args.graphs,
                           "sort_threshold": args.sort_threshold, "volpath_wavefront": args.volpath_wavefront,
                           "wave_paths": batch_paths},
                "setup": {"scene_device_mb": round(info["device_bytes"] / 1e6, 1),
                          "path_state_gb_per_batch": round(batch_paths * 205 / 1e9, 2),
                          "scene_gen_s": round(gen_s, 2), "scene_build_upload_s": round(upload_s, 2)},
                "e2e": None if args.small else {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                                                "d2h_bytes_per_step": d2h},
                "roofline": {"bound": bound, "achieved": achieved, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                             "frac": achieved / peaks.get("hbm_gbs", 1), "traffic": traffic,
                             "dram_gbs": dram_gbs, "dram_frac": dram_frac,
                             "kernel": dom, "peak_source": src, "peak_kind": "HBM copy bandwidth (of measured)",
                             "algorithmic_bytes_per_ray": per_ray, "launches": nl,
                             "avg_launch_ms": avg_launch_s * 1000,
                             "note": "frac = algorithmic bytes (node + triangle fetches, ray in, hit out) per "
                                     "launch / launch time / HBM peak; most node fetches hit L2, so it is a "
                                     "memory-side request rate, not DRAM throughput. dram_frac = ncu DRAM "
                                     "bytes per launch / launch time / HBM peak. The kernel is latency-bound "
                                     "(dependent node fetches, divergent lanes)"},
                "mrays_per_s": rays_per_s / 1e6,
                "kernel_ms": {k: round(v / args.steps, 3) for k, v in kern.items()},
                "kernel_ms_source": ("kernel-by-kernel profiled steps after the graph-launched timed region"
                                     if args.graphs else "CUDA events in the timed region"),
                "traversal": {"nodes_per_closest_ray": nodes_pr_c, "tris_per_closest_ray": tris_pr_c,
                              "nodes_per_shadow_ray": nodes_pr_a, "tris_per_shadow_ray": tris_pr_a},
                "gpu_launches": launches, "launches_before_timed": pre_launches,
                "rays_per_step": {"closest": rays_c / args.steps, "shadow": rays_a / args.steps},
                "clocks": clk}
        line.update(res)
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def _batch_jobs(n):
    from raytracer_gb300 import scenes
    env, _ = scenes.sky_env(1024, 512)
    return [scenes.batch_job(k, env) for k in range(n)]


def run_batch(args):
    """64 independent scenes: plain (one rt_render per job, one after the
    other) against rt_batch_render as one wavefront spanning the scenes, on
    several lanes (a render per job each), and under the autotuner's choice;
    same films.  The timed runs render into device films allocated
    once (the tuner times the same way); `e2e` is the fastest configuration
    again into host films (device-to-host copies and host allocation
    included)."""
    import torch
    import raytracer_gb300 as R
    torch.cuda.init()
    t0 = time.time()
    jobs = _batch_jobs(args.batch_jobs)
    gen_s = time.time() - t0
    ctx = R.Context(0)
    t0 = time.time()
    scs = [R.Scene(ctx, s) for s, _ in jobs]
    upload_s = time.time() - t0
    work = [(g, spp, dict(seed=k)) for k, (g, (_, spp)) in enumerate(zip(scs, jobs))]
    total = sum(g.width * g.height * spp for g, spp, _ in work)
    dev = [torch.zeros((g.height, g.width, 4), dtype=torch.float32, device="cuda") for g, _, _ in work]
    ptrs = [f.data_ptr() for f in dev]

    def timed(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t

    def films_now():
        return [f.cpu().numpy().copy() for f in dev]

    # warm-up: every scene once at 1 spp (tile tables, wavefront buffers)
    ctx.batch_render([(g, 1, dict(seed=0)) for g, _, _ in work])
    clocks = ClockSampler(0)
    clocks.start()

    def plain_run():
        for (g, spp, o), p in zip(work, ptrs):
            g.render(spp, film=p, **o)
    plain_run()   # untimed: the context's path buffers at their largest
    plain_s = timed(plain_run)
    plain = films_now()
    res = {}
    default_tuning = ctx.get_tuning()
    # every job as its own rt_render on 2, 4, 8 worker lanes
    ctx.set_tuning(batch_wavefront=0)
    for lanes in [int(x) for x in args.lanes.split(",")]:
        ctx.set_lanes(lanes)
        ctx.batch_render(work, device_films=ptrs)   # untimed: grows the new lanes' path buffers
        dt = timed(lambda: ctx.batch_render(work, device_films=ptrs))
        res[lanes] = (dt, all(np.array_equal(a, b) for a, b in zip(films_now(), plain)))
    best = min(res, key=lambda k: res[k][0])
    best_tuning = dict(default_tuning, lanes=best, batch_wavefront=0)
    best_s = res[best][0]
    # all jobs in one wavefront: each launch's path slots span the scenes
    ctx.set_tuning(**dict(default_tuning, batch_wavefront=1))
    ctx.batch_render(work, device_films=ptrs)   # untimed: path buffers at the batch capacity
    wave_s = timed(lambda: ctx.batch_render(work, device_films=ptrs))
    wave_st = ctx.stats()
    one_wave = {"value": total / wave_s, "seconds": wave_s, "launches": wave_st["launches"],
                "films_equal_plain": all(np.array_equal(a, b) for a, b in zip(films_now(), plain))}
    if wave_s < best_s:
        best_s, best_tuning = wave_s, dict(default_tuning, batch_wavefront=1)
    # the autotuner on the workload itself (as a farm tunes on its first
    # batch and keeps the tuning for the next ones), from the best form
    # above, then a fresh timed run of the whole batch under its choice
    tuned = None
    if not args.no_autotune:
        ctx.set_tuning(**best_tuning)
        t0 = time.perf_counter()
        choice, sample_sps = ctx.autotune(work, max_trials=args.tune_trials)
        tune_s = time.perf_counter() - t0
        ctx.batch_render(work, device_films=ptrs)   # untimed: buffers and graphs of the choice
        dt = timed(lambda: ctx.batch_render(work, device_films=ptrs))
        tuned = {"value": total / dt, "seconds": dt, "tuning": choice, "tune_seconds": tune_s,
                 "sample_jobs": len(work), "sample_samples_per_s": sample_sps,
                 "films_equal_plain": all(np.array_equal(a, b) for a, b in zip(films_now(), plain))}
        if dt < best_s:
            best_s, best_tuning = dt, choice
    # end to end: the fastest configuration into host films
    ctx.set_tuning(**best_tuning)
    ctx.batch_render(work)
    t0 = time.perf_counter()
    host = ctx.batch_render(work)
    e2e_s = time.perf_counter() - t0
    e2e_same = all(np.array_equal(a, b) for a, b in zip(host, plain))
    ctx.set_tuning(**default_tuning)
    clk = clocks.stop()
    d2h = int(sum(g.width * g.height * 16 for g, _, _ in work))
    line = {"metric": METRIC, "value": total / best_s, "unit": UNIT, "n_gpus": 1, "higher_is_better": True,
            "workload": "batch%d" % len(jobs), "dtype": "f32", "data": "synthetic (seeded scenes)",
            "config": {"jobs": len(jobs), "total_samples": total,
                       "triangles": int(sum(s.n_triangles for s, _ in jobs)),
                       "pixels": int(sum(g.width * g.height for g in scs)), "max_depth": 12,
                       "films": "device (allocated once)",
                       "scene_gen_s": round(gen_s, 2), "scene_build_upload_s": round(upload_s, 2)},
            "plain": {"value": total / plain_s, "seconds": plain_s},
            "batched": {str(k): {"value": total / v[0], "seconds": v[0], "films_equal_plain": v[1]}
                        for k, v in res.items()},
            "one_wavefront": one_wave,
            "autotuned": tuned, "default_tuning": default_tuning, "best_tuning": best_tuning,
            "best_lanes": best, "speedup_vs_plain": plain_s / best_s,
            "e2e": {"value": total / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": d2h,
                    "films_equal_plain": e2e_same},
            "clocks": clk}
    print(json.dumps(line))


def _serve_pool(ctx, n_pt, n_vol, ref_spp=4096):
    """The served stream's scene pool: n_pt scenes of the 64-scene batch
    distribution (seeded displaced icospheres, 1e3-5e5 triangles, 128^2 to
    1024^2, the sky map) and n_vol 256x256 grid-medium scenes, each with its
    ref_spp-sample GPU render as the RMSE reference."""
    import raytracer_gb300 as R
    from raytracer_gb300 import scenes
    env, _ = scenes.sky_env(1024, 512)
    pool = []
    for k in range(n_pt):
        s, _ = scenes.batch_job(1000 + k, env)
        pool.append(R.Scene(ctx, s))
    for k in range(n_vol):
        pool.append(R.Scene(ctx, scenes.volume_grid(256, 256, res=128, seed=k)))
    refs = [R.post_process(g.render(ref_spp, seed=999)) for g in pool]
    return pool, refs


SERVE_BUDGET = 150 * 10 ** 9   # device bytes a server may hold for admitted jobs (scenes, films, path state)


def _serve_run(ctx, pool, refs, picks, arrivals, form, target, cap, lanes):
    """Submit the jobs at their arrival times to a server of the given form;
    per job: latency to completion (queue + run), samples rendered and the
    true RMSE of its film against the pool scene's reference."""
    import raytracer_gb300 as R
    srv = R.Server(ctx, lanes=1 if form == "plain" else lanes, lanes_only=form != "batched", rmse_display=True,
                   device_budget_bytes=SERVE_BUDGET)
    t0 = time.perf_counter()
    ids = []
    for (pi, seed), ta in zip(picks, arrivals):
        dt = ta - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        ids.append(srv.submit(pool[pi], cap, target_rmse=target, seed=seed))
    lat, samples, rmse, rmse_lin, spp = [], 0, [], [], []
    for j, (pi, _) in zip(ids, picks):
        info, film = srv.wait(j)
        lat.append(info["queue_ms"] + info["run_ms"])
        g = pool[pi]
        samples += g.width * g.height * info["spp_done"]
        spp.append(info["spp_done"])
        img = R.post_process(film)
        rmse.append(float(np.sqrt(np.mean((np.clip(img, 0, 1) - np.clip(refs[pi], 0, 1)) ** 2))))
        rmse_lin.append(float(np.sqrt(np.mean((img - refs[pi]) ** 2))))
    wall = time.perf_counter() - t0
    srv.stop()
    rmse = np.array(rmse)
    # the reference renders carry noise of their own (about 0.01 on the
    # displayed image), so a film that meets the target measures up to
    # sqrt(0.02^2 + 0.01^2) against them: 1.25x the target is the bar
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "jobs_per_s": len(ids) / wall, "samples_per_s": samples / wall,
            "spp_p50": float(np.median(spp)), "spp_max": int(np.max(spp)),
            "true_rmse_p50": float(np.median(rmse)), "true_rmse_p90": float(np.percentile(rmse, 90)),
            "met_target_frac": float(np.mean(rmse <= target * 1.25)),
            "linear_rmse_p50": float(np.median(rmse_lin))}


def run_serve(args):
    """Open-loop Poisson arrivals at each rate, the same trace for three
    server forms: plain (one job at a time), lanes (every job a render of
    its own on 4 lanes) and batched (continuous batching: the chunks of all
    admitted jobs in one multi-scene wavefront per step).  Jobs render
    progressively to a target RMSE; latency is submission to completion,
    and each finished film's true RMSE is measured against its scene's
    4096-spp GPU render."""
    import torch
    import raytracer_gb300 as R
    torch.cuda.init()
    ctx = R.Context(0)
    t0 = time.time()
    pool, refs = _serve_pool(ctx, args.serve_pool, max(1, args.serve_pool // 6))
    prep_s = time.time() - t0
    n_pt = args.serve_pool
    out = {"metric": "job latency", "unit": "ms", "workload": "serve", "higher_is_better": False,
           "target_rmse": args.target_rmse, "spp_cap": args.spp_cap, "jobs_per_rate": args.serve_jobs,
           "device_budget_gb": SERVE_BUDGET / 1e9,
           "pool": {"path_mis_scenes": n_pt, "volume_scenes": len(pool) - n_pt, "reference_spp": 4096,
                    "prep_s": round(prep_s, 1)},
           "rates": {}}
    forms = [f for f in args.serve_forms.split(",")]
    for lam in [float(x) for x in args.rates.split(",")]:
        rng = np.random.default_rng(int(lam * 10))
        arrivals = np.cumsum(rng.exponential(1.0 / lam, args.serve_jobs))
        picks = [(int(n_pt + rng.integers(len(pool) - n_pt)) if rng.random() < 0.2 else int(rng.integers(n_pt)), j)
                 for j in range(args.serve_jobs)]
        out["rates"][str(lam)] = {f: _serve_run(ctx, pool, refs, picks, arrivals, f, args.target_rmse, args.spp_cap,
                                                args.serve_lanes) for f in forms}
        print(json.dumps({"rate": lam, **out["rates"][str(lam)]}), file=sys.stderr, flush=True)
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--forms", type=int, default=1, choices=[0, 1],
                    help="add the batched (64 scenes) and served (one arrival rate) blocks to the line")
    ap.add_argument("--small", action="store_true",
                    help="profiler case: same scene at 512x512, 8 spp, no CPU baseline, no e2e")
    ap.add_argument("--bvh-width", type=int, default=2, choices=[2, 4, 8],
                    help="traversal tree: binary BVH (default) or compressed 8-wide BVH")
    ap.add_argument("--workload", default="icosphere", choices=["icosphere", "volume", "smooth", "batch", "serve"],
                    help="icosphere: the headline single-scene render; batch: 64 scenes, plain vs "
                         "rt_batch_render; serve: Poisson arrivals through rt_server")
    ap.add_argument("--wave-paths", type=int, default=0, help="paths per wavefront batch (0: library default)")
    ap.add_argument("--ray-sort", type=int, default=0, choices=[0, 1], help="regroup rays before each trace")
    ap.add_argument("--batch-jobs", type=int, default=64)
    ap.add_argument("--lanes", default="2,4,8", help="batch: lane counts to time")
    ap.add_argument("--no-autotune", action="store_true", help="batch: skip the autotuned run")
    ap.add_argument("--tune-trials", type=int, default=20, help="batch: autotuner trial budget")
    ap.add_argument("--graphs", type=int, default=0, choices=[0, 1],
                    help="launch each wavefront batch as a CUDA graph (render and serve workloads)")
    ap.add_argument("--sort-threshold", type=int, default=0,
                    help="bounces with fewer closest-hit rays shade unsorted (0: always sorted by material)")
    ap.add_argument("--volpath-wavefront", type=int, default=1, choices=[0, 1],
                    help="VolPathTracing as a wavefront of kernels (1) or one persistent kernel (0)")
    ap.add_argument("--filter", default="box", choices=["box", "gaussian", "mitchell"],
                    help="reconstruction filter of the rendered scene (box: radius 0.5)")
    ap.add_argument("--rates", default="5,10,20,50,100,200", help="serve: arrival rates (jobs/s)")
    ap.add_argument("--serve-jobs", type=int, default=100, help="serve: jobs per arrival rate")
    ap.add_argument("--serve-pool", type=int, default=24, help="serve: scenes of the batch distribution in the pool")
    ap.add_argument("--serve-forms", default="plain,lanes,batched", help="serve: server forms to time")
    ap.add_argument("--serve-lanes", type=int, default=4)
    ap.add_argument("--target-rmse", type=float, default=0.02)
    ap.add_argument("--spp-cap", type=int, default=4096)
    args = ap.parse_args()
    global _ARGS
    _ARGS = args
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "volume":
        CONFIG.clear()
        CONFIG.update(VOLUME)
    if args.workload == "smooth":
        CONFIG.clear()
        CONFIG.update(SMOOTH)
    if args.small:
        CONFIG.update(SMALL)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
