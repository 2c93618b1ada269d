"""Benchmark of the path-tracing pass: Mrays/s on the instanced 1920x1080 workload.

Workload (default, one GPU): 16 seeded meshes (~4.9M unique triangles, noise-displaced
icospheres and heightfield grids) in 1024 instances (~68M instanced triangles), a 2048x1024
RGBA32F procedural sky with a 0.5 degree sun disc, 1920x1080 pinhole camera, 64 samples
per pixel, 8 bounces, the reference's Russian roulette (contribution factor 4).  A step is
one full frame: invalidate + 64 dispatches' worth of samples, so every step renders the
same 132.7M paths.  Mrays/s counts traversal queries (primary + extension rays).

  value  device-resident: scene, environment and image stay in HBM; CUDA events bracket K
         steps on the launching stream.  The scene (~0.8 GB) and the path queues exceed L2,
         so no flush is needed between steps.
  e2e    the same frames through the C ABI with host buffers: the camera struct goes in and
         the 33 MB RGBA32F image comes back to pinned host memory inside every step.

The line also carries `quality` (relMSE of 16/64/256 spp against a 16,384-spp render, plain
and with environment next-event estimation),
`serving` (render-job server p50/p99 under Poisson loads) and `cache` (the learned radiance
cache: online training along a seeded camera spline, then relMSE and frame time of cache
mode against plain 16/64 spp at the last camera, with the MLP kernels' tensor-core rate).

--impl reference times the CPU restatement of the reference pass (oracle/, all host
threads) on crops of the same frame.  --gpus N runs N independent replicas (one frame each,
weak scaling); there is no data-path collective.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "Mrays/s (primary + extension rays), 1920x1080 64spp 8 bounces"
# DRAM bytes (read + write) per traversal query of k_trace_wave, from one ncu capture of the
# same scene at 480x270, 4 spp (bounce-0 launch: 518,400 rays, 74.1 MB read + 6.0 MB
# written); the roofline scales it to a full launch by the launch's rays
TRACE_DRAM_BYTES_PER_RAY = 154.6
UNIT = "Mrays/s"
WORKLOAD = "instanced 16 meshes / 1024 instances, 1920x1080, 64 spp, 8 bounces, equirect sky"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU work per baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--spp", type=int, default=64)
    p.add_argument("--width", type=int, default=1920, help="smaller frames for profiling runs only")
    p.add_argument("--height", type=int, default=1080)
    p.add_argument("--batch-paths", type=int, default=0, help="paths per wavefront batch (0: library default)")
    p.add_argument("--no-serving", action="store_true", help="skip the render-job serving report")
    p.add_argument("--serving-loads", type=str, default="10:60,30:90,60:120",
                   help="rate:jobs pairs of Poisson loads for the serving report")
    p.add_argument("--no-cache", action="store_true", help="skip the radiance-cache report")
    p.add_argument("--env-nee", action="store_true",
                   help="time the opt-in environment-NEE estimator instead of the reference's (rays counted "
                        "are the closest-hit queries; no CPU baseline or roofline: the oracle has no NEE)")
    p.add_argument("--all-configs", action="store_true",
                   help="instead of the benchmark line, measure the other workloads (spheres 256x256 16 spp, "
                        "1M-triangle soup traversal) on GPU and CPU and print them as one JSON line")
    p.add_argument("--cache-frames", type=int, default=300, help="1-spp frames of online training on the camera path")
    p.add_argument("--cache-ref-spp", type=int, default=16384, help="samples of the cache report's reference image")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peaks_all():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


def measured_peaks():
    p = measured_peaks_all()
    return float(p.get("hbm_gbs", 6800.0)), ("fallback" if p.get("fallback") else "measured")


def build_workload(args):
    from nbounce_gb300 import scenes
    return scenes.instanced_scene(spp=args.spp, width=args.width, height=args.height)


def cpu_baseline(desc, sobol, seconds, threads):
    """The oracle (binary32 restatement of the reference pass) on a centred crop of the frame,
    sized from a calibration run to take about `seconds`.  Returns a dict for the JSON line
    plus the reference work counters per ray."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    osc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    build_s = time.perf_counter() - t0
    W, H, spp = desc.width, desc.height, desc.spp

    def run(w, h):
        x0, y0 = (W - w) // 2, (H - h) // 2
        t = time.perf_counter()
        _, rays, _, _ = osc.render(desc.clip_to_world, W, H, sobol, 1, spp, bounces=desc.bounces,
                                   env_texels=desc.env_texels, region=(x0, y0, w, h), threads=threads)
        return rays, time.perf_counter() - t

    rays, dt = run(16, 16)
    scale = max(1.0, seconds / max(dt, 1e-3))
    side = int(16 * scale ** 0.5) // 8 * 8
    w, h = min(W, max(16, side * 2)), min(H, max(16, side // 2))
    rays, dt = run(w, h)
    per_ray = osc.work_per_ray()
    return {"value": rays / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"centred {w}x{h} crop of the 1920x1080 frame, {spp} spp, {rays} rays in {dt:.1f} s "
                      f"(oracle scene build {build_s:.1f} s, not timed)"}, per_ray, osc


def rel_mse(img, ref):
    """mean over pixels and channels of (x - ref)^2 / (ref^2 + 1e-2), over the pixels where both
    images are finite: the reference shading divides 0 by 0 at exactly grazing angles
    (pathtracing.wgsl:119-125 with cos = 0), and a NaN sample stays in a pixel's running mean,
    so a long reference render can hold a few NaN pixels (counted by nonfinite_pixels)."""
    x = img[..., :3].astype(np.float64)
    r = ref[..., :3].astype(np.float64)
    ok = np.all(np.isfinite(x), axis=-1) & np.all(np.isfinite(r), axis=-1)
    return float(np.mean(((x - r) ** 2 / (r * r + 1e-2))[ok]))


def nonfinite_pixels(img):
    return int(np.sum(~np.all(np.isfinite(img[..., :3]), axis=-1)))


def quality_report(args, ref_spp=16384, width=480, height=270):
    """relMSE of the benchmark frame's 64-spp estimate against a 16,384-spp render of the same
    camera and scene (FP32, this GPU), at 480x270 so the reference takes seconds."""
    import nbounce_gb300 as nb
    from nbounce_gb300 import scenes
    desc = scenes.instanced_scene(spp=args.spp, width=width, height=height)
    scene = nb.SceneBuffers.from_desc(desc)
    env = nb.EnvMap(texels=desc.env_texels)
    cam = nb.camera_struct(desc.world_to_clip, desc.clip_to_world)
    table = nb.sobol_burley_table(ref_spp, 17)
    pt = nb.Pathtracer(width, height, nb.Globals(bounces=desc.bounces), sobol_table=table)
    t = time.perf_counter()
    pt.render(scene, cam, env, ref_spp)
    ref = pt.download()
    ref_s = time.perf_counter() - t
    out = {"resolution": [width, height], "reference_spp": ref_spp, "reference_s": round(ref_s, 2),
           "reference": "FP32 GPU render, same camera/scene, Sobol rows 1..16384"}
    for spp in (16, 64, 256):
        pt.invalidate()
        pt.render(scene, cam, env, spp)
        out[f"relmse_{spp}spp"] = round(rel_mse(pt.download(), ref), 6)
    # the same frames with environment next-event estimation (MIS), an opt-in estimator
    pt.set_sampling(env_nee=True)
    for spp in (16, 64, 256):
        pt.invalidate()
        pt.render(scene, cam, env, spp)
        out[f"nee_relmse_{spp}spp"] = round(rel_mse(pt.download(), ref), 6)
    return out


def serving_report(args):
    """Render-job serving (continuous batching): 8 resident instanced scenes of ~10K to ~5M
    unique triangles, one shared 2048x1024 sky, seeded Poisson arrivals; resolution uniform
    over {256^2, 512^2, 1024x768, 1920x1080}, spp uniform over {1, 4, 16, 64}, 8 bounces,
    120 GB admission budget.  The mix costs ~17M paths per job on average, so the arrival
    rates are given beside the measured saturation throughput."""
    import nbounce_gb300 as nb
    from nbounce_gb300 import scenes, server
    scales = [1 / 512, 1 / 128, 1 / 64, 1 / 16, 1 / 8, 1 / 4, 1 / 2, 1.0]
    descs = [scenes.instanced_scene(seed=0x5EED1 + 97 * k, scale=s, width=64, height=64, env_size=(16, 8))
             for k, s in enumerate(scales)]
    bufs = [nb.SceneBuffers.from_desc(d) for d in descs]
    sky = nb.EnvMap(texels=scenes.sky_envmap(0x5EED9, 2048, 1024))
    srv = server.RenderServer(hbm_budget_bytes=120 << 30, paths_per_wave=1 << 25)
    slots = [srv.add_scene(b) for b in bufs]
    env = srv.add_env(sky)
    eye, target = (0.0, 14.0, 62.0), (0.0, -2.0, 0.0)
    cams = [lambda w, h: scenes.camera_matrices(eye, target, w, h)] * len(descs)
    server.run_load(srv, slots, env, cams, server.make_trace(8, 1000.0, len(descs), seed=1))  # warm-up
    out = {"scenes_unique_triangles": [int(d.n_triangles_unique) for d in descs], "budget_gb": 120,
           "paths_per_wave": 1 << 25, "loads": []}
    def rounded(r):
        return {k: (rounded(v) if isinstance(v, dict) else round(v, 3) if isinstance(v, float) else v)
                for k, v in r.items()}

    for rate, n_jobs in args.serving_loads:
        r = server.run_load(srv, slots, env, cams, server.make_trace(n_jobs, rate, len(descs), seed=int(rate)))
        r["rate_jobs_per_s"] = rate
        out["loads"].append(rounded(r))
    # per-job estimator options: the middle load again, each job drawn from {reference,
    # environment NEE, radiance cache}; the caches of the scenes are created by a warm-up mix
    options = (0, server.L.NB_JOB_ENV_NEE, server.L.NB_JOB_CACHE)
    server.run_load(srv, slots, env, cams, server.make_trace(16, 1000.0, len(descs), seed=2, options=options))
    rate, n_jobs = args.serving_loads[len(args.serving_loads) // 2]
    r = server.run_load(srv, slots, env, cams,
                        server.make_trace(n_jobs, rate, len(descs), seed=int(rate), options=options))
    r["rate_jobs_per_s"] = rate
    out["mixed_options"] = rounded(r)
    srv.close()
    return out


# Algorithmic FLOPs of the radiance-cache MLP (64 -> 5 x 64 -> 3): a lookup is 5 * 64 * 64 +
# 3 * 64 = 20,672 multiply-adds; a training record adds the backward pass, 4 * 4096 + 3 * 64 =
# 16,576 for the hidden-layer gradients and 20,672 for the weight gradients.
MLP_FLOP_PER_QUERY = 2 * 20672
MLP_FLOP_PER_RECORD = 2 * (20672 + 16576 + 20672)


def cache_report(args, desc, scene, env, stream):
    """Learned radiance cache on the benchmark scene at the benchmark resolution: the cache
    trains online for args.cache_frames one-sample frames while the camera moves along a
    seeded spline (scenes.camera_path), then the last camera's frame is rendered with the
    cache at 1, 4 and 16 spp and without it at 16 and 64 spp.  Every image is scored by
    relMSE against an args.cache_ref_spp-sample plain render of that camera; frame times are
    CUDA-event times of whole frames (render call: trace, shade, cache lookups, training,
    accumulate).  Modes: "primary" ends every path at its primary hit (spread < 0), "spread"
    uses the spread rule with c = 0.01."""
    import torch
    import nbounce_gb300 as nb
    from nbounce_gb300 import scenes
    W, H = desc.width, desc.height
    sh = stream.cuda_stream
    path = scenes.camera_path(args.cache_frames)
    cams = [nb.camera_struct(*scenes.camera_matrices(e, t, W, H)) for e, t in path]
    last = cams[-1]

    def frame(pt, cam, spp):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        pt.invalidate()
        a.record(stream)
        pt.render(scene, cam, env, spp, stream=sh)
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b)

    ref_pt = nb.Pathtracer(W, H, nb.Globals(bounces=desc.bounces), sobol_table=nb.sobol_burley_table(args.cache_ref_spp, 17))
    t = time.perf_counter()
    ref_pt.render(scene, last, env, args.cache_ref_spp, stream=sh)
    ref = ref_pt.download(stream=sh)
    ref_s = time.perf_counter() - t
    ref_pt.close()
    out = {"resolution": [W, H], "frames": args.cache_frames, "camera": "scenes.camera_path(seed 0x5EEDC), last frame",
           "reference": f"plain FP32 GPU render, {args.cache_ref_spp} spp, {ref_s:.1f} s", "plain": {}, "modes": {}}
    plain = nb.Pathtracer(W, H, nb.Globals(bounces=desc.bounces))
    for spp in (16, 64):
        frame(plain, last, spp)
        ms = frame(plain, last, spp)
        out["plain"][f"{spp}spp"] = {"relmse": round(rel_mse(plain.download(stream=sh), ref), 5), "ms": round(ms, 2)}
    # environment next-event estimation (no cache): the opt-in estimator aimed at the sun disc
    out["nee"] = {}
    plain.set_sampling(env_nee=True)
    for spp in (4, 16, 64):
        frame(plain, last, spp)
        ms = frame(plain, last, spp)
        out["nee"][f"{spp}spp"] = {"relmse": round(rel_mse(plain.download(stream=sh), ref), 5), "ms": round(ms, 2)}
    plain.close()
    peak = measured_peaks_all().get("bf16_tflops")
    for name, cfg in (("primary", dict(spread=-1.0)), ("spread", dict(spread=0.01))):
        cache = nb.RadianceCache(seed=0x5EEDC, **cfg)
        pt = nb.Pathtracer(W, H, nb.Globals(bounces=desc.bounces))
        pt.set_cache(cache)
        # training along the path; the last `timed` frames also record per-kernel times and
        # cache counters (steady state: the training-path density has adapted to the budget)
        timed = min(20, len(cams))
        train_ms, queries, records = [], 0, 0
        for k, cam in enumerate(cams):
            if k == len(cams) - timed:
                pt.enable_timing(True)
                pt.kernel_times(reset=True, stream=sh)
            train_ms.append(frame(pt, cam, 1))
            if k >= len(cams) - timed:
                st = cache.stats(stream=sh)
                queries += st["queries"]
                records += st["records_used"]
        kt = pt.kernel_times(reset=True, stream=sh)
        pt.enable_timing(False)
        m = {"config": cache.config, "train_frame_ms_median": round(statistics.median(train_ms), 3),
             "kernel_ms_per_frame": {k: round(kt[k] / timed, 3) for k in ("raygen_ms", "trace_ms", "shade_ms",
                                                                          "cache_infer_ms", "cache_train_ms",
                                                                          "accumulate_ms")},
             "per_frame": {"queries": queries // timed, "records_used": records // timed,
                           "stride": st["stride"], "loss": round(st["loss"], 4)}}
        for spp in (1, 4, 16):
            ms = frame(pt, last, spp)
            m[f"{spp}spp"] = {"relmse": round(rel_mse(pt.download(stream=sh), ref), 5), "ms": round(ms, 2)}
        infer_tf = queries * MLP_FLOP_PER_QUERY / (kt["cache_infer_ms"] / 1e3) / 1e12
        train_tf = records * MLP_FLOP_PER_RECORD / (kt["cache_train_ms"] / 1e3) / 1e12
        m["mlp_roofline"] = {"bound": "tensor", "unit": "TFLOP/s", "peak": peak,
                             "infer_achieved": round(infer_tf, 1), "infer_frac": round(infer_tf / peak, 4) if peak else None,
                             "train_achieved": round(train_tf, 2), "train_frac": round(train_tf / peak, 5) if peak else None,
                             "note": "algorithmic FLOPs (41,344 per lookup, 115,840 per training record) over the "
                                     "timed cache_infer / cache_train launches of the last 20 training frames "
                                     "(train includes record gathering and the Adam launches)"}
        out["modes"][name] = m
        pt.close()
        cache.close()
    p64 = out["plain"]["64spp"]
    best = None
    for name, m in out["modes"].items():
        for spp in (1, 4, 16):
            r = m[f"{spp}spp"]
            if r["relmse"] <= p64["relmse"] and (best is None or r["ms"] < best[2]):
                best = (name, spp, r["ms"], r["relmse"])
    out["at_plain64_relmse"] = None if best is None else {
        "mode": best[0], "spp": best[1], "ms": best[2], "relmse": best[3],
        "frame_time_ratio": round(p64["ms"] / best[2], 2)}
    return out


def configs_report(args):
    """GPU and CPU (oracle, all host threads) numbers of the two other workloads:
    spheres: 64 icospheres + ground, 256x256, 16 spp, 6 bounces, constant sky; Mrays/s, frame
             ms and relMSE against a 16,384-spp render of the same frame
    soup:    1M-triangle soup (edges ~0.02 in [-1,1]^3), 16,777,216 rays, coherent (1024 x 16384
             pinhole grid) and incoherent (uniform origins and directions), closest and any hit;
             GPU on device-resident rays, CPU on a 262,144-ray prefix of the same rays."""
    import torch
    import nbounce_gb300 as nb
    from nbounce_gb300 import scenes
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    out = {"cpu_threads": threads}
    # spheres
    desc = scenes.spheres_scene(width=256, height=256, spp=16, bounces=6)
    scene = nb.SceneBuffers.from_desc(desc)
    env = nb.EnvMap(desc.env_color)
    cam = nb.camera_struct(desc.world_to_clip, desc.clip_to_world)
    ref_pt = nb.Pathtracer(256, 256, nb.Globals(bounces=6), sobol_table=nb.sobol_burley_table(16384, 17))
    ref_pt.render(scene, cam, env, 16384)
    ref = ref_pt.download()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def gpu_frames(rr_start):
        pt = nb.Pathtracer(256, 256, nb.Globals(bounces=6))
        pt.set_rr_start_bounce(rr_start)
        for _ in range(3):
            pt.invalidate()
            pt.render(scene, cam, env, 16)
        torch.cuda.synchronize()
        a.record()
        for _ in range(10):
            pt.invalidate()
            pt.render(scene, cam, env, 16)
        b.record()
        b.synchronize()
        return a.elapsed_time(b) / 10, pt.last_stats()[0], pt.download()

    ms, rays, img = gpu_frames(0)
    ms3, rays3, img3 = gpu_frames(3)
    osc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    t = time.perf_counter()
    cimg, crays, _, _ = osc.render(desc.clip_to_world, 256, 256, nb.sobol_burley_table(), 1, 16, bounces=6,
                                   env=desc.env_color, threads=threads)
    cs = time.perf_counter() - t
    out["spheres_256_16spp"] = {
        "gpu": {"mrays_s": round(rays / ms / 1e3, 1), "frame_ms": round(ms, 3), "rays": int(rays),
                "relmse": round(rel_mse(img, ref), 5), "nonfinite_pixels": nonfinite_pixels(img)},
        "cpu": {"mrays_s": round(crays / cs / 1e6, 2), "frame_ms": round(cs * 1e3, 1), "rays": int(crays),
                "relmse": round(rel_mse(cimg, ref), 5), "nonfinite_pixels": nonfinite_pixels(cimg)},
        "gpu_rr_from_bounce_3": {"mrays_s": round(rays3 / ms3 / 1e3, 1), "frame_ms": round(ms3, 3),
                                 "rays": int(rays3), "relmse": round(rel_mse(img3, ref), 5)},
        "rr": "reference schedule (cf 4) unless stated; the variant disables roulette before bounce 3",
        "reference": "16,384-spp plain GPU render", "reference_nonfinite_pixels": nonfinite_pixels(ref)}
    # soup traversal
    desc = scenes.soup_scene(1 << 20)
    soup = nb.SceneBuffers.from_desc(desc)
    osc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    n = 1 << 24
    res = {}
    for kind in ("coherent", "incoherent"):
        rays = scenes.coherent_rays(1024, 16384) if kind == "coherent" else scenes.incoherent_rays(n, seed=0x5EED3)
        d_rays = torch.from_numpy(rays).cuda()
        hits = torch.empty((n, 4), dtype=torch.float32, device="cuda")
        inst = torch.empty(n, dtype=torch.int32, device="cuda")
        for any_hit in (False, True):
            for _ in range(3):
                soup.trace_device(d_rays.data_ptr(), n, hits.data_ptr(), inst.data_ptr(), any_hit=any_hit)
            a.record()
            for _ in range(5):
                soup.trace_device(d_rays.data_ptr(), n, hits.data_ptr(), inst.data_ptr(), any_hit=any_hit)
            b.record()
            b.synchronize()
            gms = a.elapsed_time(b) / 5
            m = 1 << 18
            t = time.perf_counter()
            osc.trace(rays[:m], any_hit=any_hit, threads=threads)
            cs = time.perf_counter() - t
            res[f"{kind}_{'any' if any_hit else 'closest'}"] = {
                "gpu_mrays_s": round(n / gms / 1e3, 1), "gpu_ms": round(gms, 3), "cpu_mrays_s": round(m / cs / 1e6, 2),
                "ratio": round((n / gms / 1e3) / (m / cs / 1e6), 1)}
        del d_rays, hits, inst
    out["soup_1m_16m_rays"] = res
    return out


def run_ours(args):
    import torch
    import nbounce_gb300 as nb

    rank, world, local = dist_env()
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    desc = build_workload(args)
    t0 = time.perf_counter()
    scene = nb.SceneBuffers.from_desc(desc, dedup=True)
    build_s = time.perf_counter() - t0
    env = nb.EnvMap(texels=desc.env_texels)
    cam = nb.camera_struct(desc.world_to_clip, desc.clip_to_world)
    pt = nb.Pathtracer(desc.width, desc.height, nb.Globals(bounces=desc.bounces))
    if args.batch_paths:
        pt.set_batch_paths(args.batch_paths)
    if args.env_nee:
        pt.set_sampling(env_nee=True)
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream

    def step():
        pt.invalidate()
        pt.render(scene, cam, env, desc.spp, stream=sh)

    for _ in range(max(3, args.warmup)):
        step()
    rays_per_step, status = pt.last_stats(stream=sh)
    if status:
        raise RuntimeError(f"device status {status}")

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # device-resident timing, per-kernel events on the launch stream
    pt.enable_timing(True)
    pt.kernel_times(reset=True, stream=sh)
    torch.cuda.synchronize()
    barrier()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        start.record(stream)
        for _ in range(args.steps):
            step()
        stop.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = start.elapsed_time(stop)
    kt = pt.kernel_times(reset=True, stream=sh)
    pt.enable_timing(False)

    # end-to-end through the C ABI with host buffers
    host_img = torch.empty((desc.height, desc.width, 4), dtype=torch.float32, pin_memory=True)
    host_np = host_img.numpy()
    torch.cuda.synchronize()
    barrier()
    t = time.perf_counter()
    for _ in range(args.steps):
        step()
        pt.download(out=host_np, stream=sh)
    e2e_s = time.perf_counter() - t
    barrier()

    t_max = ms
    e2e_max = e2e_s
    if world > 1:
        v = torch.tensor([ms, e2e_s], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(v, op=torch.distributed.ReduceOp.MAX)
        t_max, e2e_max = float(v[0]), float(v[1])
    total_rays = rays_per_step * args.steps * world
    value = total_rays / (t_max / 1e3) / 1e6
    e2e_value = total_rays / e2e_max / 1e6
    if rank != 0:
        return None
    launches_per_step = sum(kt[k] for k in ("raygen_launches", "trace_launches", "shade_launches",
                                             "accumulate_launches")) / args.steps
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": round(t_max / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
        "config": {"workload": WORKLOAD, "width": desc.width, "height": desc.height, "spp": desc.spp,
                   "bounces": desc.bounces, "unique_triangles": int(desc.n_triangles_unique),
                   "instanced_triangles": int(desc.n_triangles_instanced), "instances": len(desc.instances),
                   "rays_per_step": int(rays_per_step), "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (scene ~0.8 GB + path queues), no flush",
                   "scene_build_s": round(build_s, 2),
                   "estimator": "environment NEE (opt-in)" if args.env_nee else "reference"},
        "e2e": {"value": round(e2e_value, 2), "unit": UNIT, "h2d_bytes_per_step": 128,
                "d2h_bytes_per_step": int(desc.width * desc.height * 16)},
        "gpu_launches": int(round(launches_per_step * args.steps)),
        "kernel_ms_per_step": {k: round(kt[k] / args.steps, 3) for k in ("raygen_ms", "trace_ms", "shade_ms",
                                                                       "accumulate_ms")},
        "clocks": clocks.summary(),
    }
    if not args.no_serving and world == 1:
        line["quality"] = quality_report(args)
        line["serving"] = serving_report(args)
    if not args.no_cache and world == 1:
        line["cache"] = cache_report(args, desc, scene, env, stream)
    peak, peak_kind = measured_peaks()
    sobol = nb.sobol_burley_table()
    if not args.no_cpu_baseline and not args.env_nee:
        base, per_ray, _ = cpu_baseline(desc, sobol, args.cpu_seconds, os.cpu_count() or 1)
        line["cpu_baseline"] = base
        n_aabb, n_tri, n_inst = per_ray
        bytes_per_ray = 32.0 * n_aabb + 48.0 * n_tri + 128.0 * n_inst  # reference-layout bytes per query
        trace_launches = max(1, kt["trace_launches"])
        avg_launch_ms = kt["trace_ms"] / trace_launches
        rays_per_launch = rays_per_step * args.steps / trace_launches
        achieved = bytes_per_ray * rays_per_launch / (avg_launch_ms / 1e3) / 1e9
        line["roofline"] = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                            "frac": round(achieved / peak, 4),
                            "traffic": round(TRACE_DRAM_BYTES_PER_RAY * rays_per_launch),
                            "traffic_note": "ncu dram bytes per ray of the 480x270 capture x rays per launch",
                            "note": "achieved counts the reference algorithm's bytes per query (binary BVH: 32 B "
                                    "per box test, 48 per triangle, 128 per instance, counted by the oracle); "
                                    "the device traversal fetches ~1.2-2.0 KB per ray (8-wide nodes, mostly "
                                    "L1/L2 hits) and ~155 B from DRAM (traffic), hence frac > 1: the kernel is "
                                    "latency-bound, not HBM-bound",
                            "kernel": "k_trace_wave", "peak_kind": f"{peak_kind} hbm_gbs (burst copy)",
                            "bytes_per_ray": round(bytes_per_ray, 1),
                            "work_per_ray": {"n_aabb": round(n_aabb, 2), "n_tri": round(n_tri, 2),
                                             "n_inst": round(n_inst, 2)}}
    return line


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return None
    import nbounce_gb300 as nb
    desc = build_workload(args)
    sobol = nb.sobol_burley_table()
    threads = os.cpu_count() or 1
    base, per_ray, osc = cpu_baseline(desc, sobol, min(args.cpu_seconds, 10.0), threads)
    # time steps: each step one crop sample of the same frame
    W, H = desc.width, desc.height
    w, h = 64, 32
    x0, y0 = (W - w) // 2, (H - h) // 2
    for _ in range(args.warmup):
        osc.render(desc.clip_to_world, W, H, sobol, 1, desc.spp, bounces=desc.bounces, env_texels=desc.env_texels,
                   region=(x0, y0, w, h), threads=threads)
    total_rays, t = 0, time.perf_counter()
    for _ in range(args.steps):
        _, rays, _, _ = osc.render(desc.clip_to_world, W, H, sobol, 1, desc.spp, bounces=desc.bounces,
                                   env_texels=desc.env_texels, region=(x0, y0, w, h), threads=threads)
        total_rays += rays
    dt = time.perf_counter() - t
    value = total_rays / dt / 1e6
    return {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "width": W, "height": H, "spp": desc.spp, "bounces": desc.bounces,
                       "step_sample": f"centred {w}x{h} crop per step"},
            "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"centred {w}x{h} crop of the frame per step, {desc.spp} spp"},
            "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    args.serving_loads = [(float(a), int(b)) for a, b in (x.split(":") for x in args.serving_loads.split(","))]
    if args.all_configs:
        line = configs_report(args)
    else:
        line = run_reference(args) if args.impl == "reference" else run_ours(args)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
