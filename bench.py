"""Benchmark of the path-tracing pass: Mrays/s on the instanced 1920x1080 workload.

Workload (default, one GPU): 16 seeded meshes (~4.9M unique triangles, noise-displaced
icospheres and heightfield grids) in 1024 instances (~68M instanced triangles), a 2048x1024
RGBA32F procedural sky with a 0.5 degree sun disc, 1920x1080 pinhole camera, 64 samples
per pixel, 8 bounces, the reference's Russian roulette (contribution factor 4).  A step is
one full frame: invalidate + 64 dispatches' worth of samples, so every step renders the
same 132.7M paths.  Mrays/s counts traversal queries (primary + extension rays).

  value     device-resident: scene, environment and image stay in HBM; CUDA events bracket
            K steps on the launching stream.  The scene (~0.8 GB) and the path queues exceed
            L2, so no flush is needed between steps.
  e2e       the same frames through the C ABI with host buffers: the camera struct goes in
            and the 33 MB RGBA32F image comes back to pinned host memory inside every step.
  roofline  the traversal kernel against the measured HBM copy peak, counting the bytes the
            device's own layout fetches (instrumented counters of one extra frame outside the
            timed region); the kernel is bound by the latency of its dependent loads, which
            the record states.

The line also carries `quality` (relMSE of the benchmark frame at 16/64/256/1024 spp, plain
and with environment next-event estimation, and of a 16,384-spp GPU render, against the
binary64 16,384-spp oracle truth on 24 stratified tiles, tests/golden/truth_*.npz), `serving`
(render-job server p50/p99 under Poisson loads of 50-400 jobs/s) and `cache` (the learned
radiance cache: online training along a seeded camera spline, then relMSE and frame time of
cache mode against plain 16/64 spp at the last camera, judged by that camera's binary64
truth, with the MLP kernels' tensor-core rate).

--impl reference times the CPU restatement of the reference pass (oracle/ only, all host
threads) on the same 24 stratified tiles of the same frame per step.  --gpus N starts N ranks
(one per GPU, via torch.distributed.run) unless it already runs under a launcher; each rank
renders its own frame (replicas, weak scaling, no data-path collective), or with
--shard-frame one frame is split into contiguous Sobol row ranges and merged by one
all-reduce on the device (strong scaling).
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
# DRAM bytes (read + write) per traversal query of k_trace_wave over all bounces of a frame,
# from one ncu capture of the same scene at 480x270, 64 spp (nine launches, 12,435,256 rays,
# 1,015.3 MB read + 486.2 MB written); the roofline scales it to a launch by the launch's rays
TRACE_DRAM_BYTES_PER_RAY = 120.7
# issue utilisation of the same capture (smsp__issue_active.avg.pct_of_peak_sustained_active):
# camera rays (k_trace_wave<1,0,0>) and bounce 1 (the lane-refill kernel)
TRACE_ISSUE_ACTIVE_PCT = {"camera_rays": 77.4, "bounce_1": 75.3}
UNIT = "Mrays/s"
WORKLOAD = "instanced 16 meshes / 1024 instances, 1920x1080, 64 spp, 8 bounces, equirect sky"
# bytes the device layout fetches per unit of traversal work (nb_trace_counters): an 8-wide
# node, a triangle record, an instance record, a stack entry written and read back; plus the
# ray read from the queue (two float4) and the hit written (float4 + instance id)
NODE_BYTES, TRI_BYTES, INST_BYTES, PUSH_BYTES, RAY_IO_BYTES = 80, 48, 64, 16, 52
TRUTH_DIR = os.path.join(ROOT, "tests", "golden")


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
    p.add_argument("--serving-loads", type=str, default="50:1000,100:1000,200:1000,400:1000",
                   help="rate:jobs pairs of Poisson loads for the serving report")
    p.add_argument("--serving-queue", type=int, default=64,
                   help="jobs the server lets wait for admission; submissions beyond are rejected (0: no limit)")
    p.add_argument("--shard-frame", action="store_true",
                   help="with N ranks: split each frame's samples over the ranks and merge on the device")
    p.add_argument("--no-cache", action="store_true", help="skip the radiance-cache report")
    p.add_argument("--env-nee", action="store_true",
                   help="time the opt-in environment-NEE estimator instead of the reference's (rays counted "
                        "are the closest-hit queries; no CPU baseline or roofline: the oracle has no NEE)")
    p.add_argument("--all-configs", action="store_true",
                   help="instead of the benchmark line, measure the other workloads (spheres 256x256 16 spp, "
                        "1M-triangle soup traversal) on GPU and CPU and print them as one JSON line")
    p.add_argument("--cache-frames", type=int, default=300, help="1-spp frames of online training on the camera path")
    p.add_argument("--train-bench", action="store_true",
                   help="instead of the benchmark line, time radiance-cache Adam steps of 16,384 seeded rows on both "
                        "tensor-core paths (tcgen05 and mma.sync) and print them as one JSON line")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def launch_ranks(n, script, argv):
    """Runs `script argv` as n local ranks under torch.distributed.run (rendezvous on
    127.0.0.1); the ranks inherit stdout, so rank 0's JSON line is this process's output.
    Returns the launcher's exit code."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr=127.0.0.1", f"--master-port={free_port()}", script, *argv]
    return subprocess.call(cmd)


def workload_config(desc, world, shard=False):
    """The workload as both arms name it (identical dicts for the same frame)."""
    return {"workload": WORKLOAD, "width": desc.width, "height": desc.height, "spp": desc.spp,
            "bounces": desc.bounces, "unique_triangles": int(desc.n_triangles_unique),
            "instanced_triangles": int(desc.n_triangles_instanced), "instances": len(desc.instances),
            "parallelism": (f"sample shards x{world}" if shard else f"replicas x{world}"),
            "l2": "inputs larger than L2 (scene ~0.8 GB + path queues), no flush",
            "rr": "reference schedule (contribution factor 4)"}


def load_truth(name):
    """The binary64 16,384-spp oracle image (tests/golden/make_truth.py), or None."""
    path = os.path.join(TRUTH_DIR, f"truth_{name}.npz")
    if not os.path.exists(path):
        return None
    d = np.load(path)
    return {k: d[k] for k in d.files}


def truth_matches(desc, truth):
    """The truth was made from the same seeded scene: counts equal, binary64 sums of the
    positions and transforms equal to 1e-9 relative (numpy's transcendental functions may
    round differently on another host)."""
    from nbounce_gb300 import scenes
    fp = scenes.scene_fingerprint(desc)
    t = truth["fingerprint"]
    return (int(t[0]) == fp["triangles"] and int(t[1]) == fp["instances"]
            and abs(t[2] - fp["pos_sum"]) <= 1e-9 * max(1.0, abs(fp["pos_sum"]))
            and abs(t[3] - fp["l2w_sum"]) <= 1e-9 * max(1.0, abs(fp["l2w_sum"])))


def tiles_of(img, tiles):
    return np.stack([img[y:y + h, x:x + w, :3] for (x, y, w, h) in np.asarray(tiles).tolist()])


def rel_mse_truth(img, truth):
    """relMSE of a full image's truth tiles against the binary64 truth."""
    return rel_mse(tiles_of(img, truth["tiles"]), truth["rgb"])


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


def cpu_sample_tiles(desc):
    """The CPU timing sample: 24 tiles of 16 x 16 pixels, one centred in each cell of a 6 x 4
    grid over the frame (scenes.stratified_tiles), so every part of the frame counts alike."""
    from nbounce_gb300 import scenes
    return scenes.stratified_tiles(desc.width, desc.height)


class OracleFrame:
    """The oracle (binary32 restatement of the reference pass; oracle/ only) on the benchmark
    frame: one step renders the sample tiles at the frame's samples per pixel with all host
    threads.  Nothing here loads the GPU library."""

    def __init__(self, desc, threads):
        from oracle import oracle as O
        t0 = time.perf_counter()
        self.osc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
        self.build_s = time.perf_counter() - t0
        self.sobol = O.sobol_table()
        self.desc, self.threads = desc, threads
        self.tiles = cpu_sample_tiles(desc)
        self.counters = np.zeros(4, np.float64)  # rays, n_aabb, n_tri, n_inst of the last step

    def step(self):
        d = self.desc
        rays, self.counters = 0, np.zeros(4, np.float64)
        for (x0, y0, w, h) in self.tiles:
            _, r, _, _ = self.osc.render(d.clip_to_world, d.width, d.height, self.sobol, 1, d.spp, bounces=d.bounces,
                                         env_texels=d.env_texels, region=(x0, y0, w, h), threads=self.threads)
            rays += r
            self.counters += self.osc.last_counters
        return rays

    def sample_text(self):
        n = len(self.tiles)
        s = self.tiles[0][2]
        return (f"{n} tiles of {s}x{s} pixels, one centred in each cell of a 6x4 grid over the "
                f"{self.desc.width}x{self.desc.height} frame, {self.desc.spp} spp")

    def work_per_ray(self):
        """Reference work counters per traversal query (raytracing_sw.wgsl:187,207-208,227,261,280)."""
        rays = max(self.counters[0], 1.0)
        return self.counters[1] / rays, self.counters[2] / rays, self.counters[3] / rays


def cpu_baseline(desc, seconds, threads):
    """The oracle timed on the host cores over repeated CPU sample steps (about `seconds` of
    work, after one warm-up step).  Returns the JSON dict and the OracleFrame."""
    of = OracleFrame(desc, threads)
    of.step()
    rays, n, t = 0, 0, time.perf_counter()
    while True:
        rays += of.step()
        n += 1
        if time.perf_counter() - t >= seconds:
            break
    dt = time.perf_counter() - t
    return {"value": rays / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{of.sample_text()}, {n} steps: {rays} rays in {dt:.1f} s (oracle scene build "
                      f"{of.build_s:.1f} s, not timed)"}, of


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


def truth_note(truth, name):
    return {"truth": f"binary64 oracle render at {int(truth['spp'])} spp (tests/golden/truth_{name}.npz): "
                     f"{len(truth['tiles'])} tile(s) of {int(truth['tiles'][0][2])}x{int(truth['tiles'][0][3])}",
            "truth_made_by": f"{truth['command']} ({int(truth['cores'])} {truth['host']} threads, "
                             f"{float(truth['seconds']):.0f} s)"}


def quality_report(args, desc, scene, env, stream):
    """relMSE of the benchmark frame itself (1920x1080, benchmark camera, 8 bounces) against
    the binary64 16,384-spp oracle truth on its 24 stratified tiles: GPU renders at 16, 64,
    256 and 1024 spp (plain and with environment NEE), and a GPU render of the truth's own
    16,384 samples, which measures how far the binary32 GPU pass and the binary64 oracle
    are apart on identical samples."""
    import nbounce_gb300 as nb
    truth = load_truth("instanced_1080p")
    if truth is None:
        return {"unavailable": "tests/golden/truth_instanced_1080p.npz is missing"}
    if not truth_matches(desc, truth) or desc.width != int(truth["width"]) or desc.height != int(truth["height"]):
        return {"unavailable": "the truth image was made from another scene or frame size"}
    sh = stream.cuda_stream
    cam = nb.camera_struct(desc.world_to_clip, desc.clip_to_world)
    ref_spp = int(truth["spp"])
    pt = nb.Pathtracer(desc.width, desc.height, nb.Globals(bounces=desc.bounces),
                       sobol_table=nb.sobol_burley_table(ref_spp, 17))
    out = {"resolution": [desc.width, desc.height], **truth_note(truth, "instanced_1080p")}

    def score(spp):
        pt.invalidate()
        pt.render(scene, cam, env, spp, stream=sh)
        return round(rel_mse_truth(pt.download(stream=sh), truth), 6)

    for spp in (16, 64, 256, 1024):
        out[f"relmse_{spp}spp"] = score(spp)
    t = time.perf_counter()
    out[f"gpu_{ref_spp}spp_vs_truth_relmse"] = score(ref_spp)
    out[f"gpu_{ref_spp}spp_s"] = round(time.perf_counter() - t, 2)
    # the same frames with environment next-event estimation (MIS), an opt-in estimator
    pt.set_sampling(env_nee=True)
    for spp in (16, 64, 256):
        out[f"nee_relmse_{spp}spp"] = score(spp)
    pt.close()
    return out


def serving_report(args):
    """Render-job serving (continuous batching): 8 resident instanced scenes of ~10K to ~5M
    unique triangles, one shared 2048x1024 sky, seeded Poisson arrivals at 50, 100, 200 and
    400 jobs/s (1,000 jobs each); resolution uniform over {256^2, 512^2, 1024x768, 1920x1080},
    spp uniform over {1, 4, 16, 64}, 8 bounces, 120 GB admission budget.  The mix costs ~17M
    paths (~25M traversal queries) per job on average, so one GPU saturates near 60-70 jobs/s;
    beyond that the server sheds load: at most args.serving_queue jobs wait for admission and
    further submissions are rejected (NB_ERR_BUSY).  Per load: p50/p99 of submit -> finish and
    of queue time of the admitted jobs, admitted / rejected counts, the queued and active job
    counts over time, GPU busy fraction and completed jobs per second."""
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
    idle_bytes = srv.stats()["bytes_in_use"]
    srv.set_queue_limit(args.serving_queue)
    out = {"scenes_unique_triangles": [int(d.n_triangles_unique) for d in descs], "budget_gb": 120,
           "paths_per_wave": 1 << 25, "queue_limit": args.serving_queue, "idle_bytes": int(idle_bytes),
           "admission": "jobs wait in arrival order while their images fit the budget and the wave has job slots; "
                        "beyond the queue limit submissions are rejected with NB_ERR_BUSY (load shedding)",
           "loads": []}

    def rounded(r):
        if isinstance(r, dict):
            return {k: rounded(v) for k, v in r.items()}
        if isinstance(r, list):
            return [rounded(v) for v in r]
        return round(r, 3) if isinstance(r, float) else r

    for rate, n_jobs in args.serving_loads:
        r = server.run_load(srv, slots, env, cams, server.make_trace(n_jobs, rate, len(descs), seed=int(rate)))
        r["rate_jobs_per_s"] = rate
        out["loads"].append(rounded(r))
    # per-job estimator options: each job drawn from {reference, environment NEE, radiance
    # cache} at 50 jobs/s; the caches of the scenes are created by a warm-up mix
    options = (0, server.L.NB_JOB_ENV_NEE, server.L.NB_JOB_CACHE)
    server.run_load(srv, slots, env, cams, server.make_trace(16, 1000.0, len(descs), seed=2, options=options))
    r = server.run_load(srv, slots, env, cams, server.make_trace(600, 50.0, len(descs), seed=50, options=options))
    r["rate_jobs_per_s"] = 50.0
    out["mixed_options"] = rounded(r)
    out["bytes_in_use_after_all"] = int(srv.stats()["bytes_in_use"])
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
    relMSE against the binary64 16,384-spp oracle truth of that camera on 24 stratified
    tiles (tests/golden/truth_instanced_cache.npz); frame times are
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

    truth = load_truth("instanced_cache")
    if truth is None or not truth_matches(desc, truth) or (W, H) != (int(truth["width"]), int(truth["height"])):
        return {"unavailable": "tests/golden/truth_instanced_cache.npz is missing or from another scene"}

    def score(img):
        return round(rel_mse_truth(img, truth), 5)

    out = {"resolution": [W, H], "frames": args.cache_frames, "camera": "scenes.camera_path(seed 0x5EEDC), last frame",
           **truth_note(truth, "instanced_cache"), "plain": {}, "modes": {}}
    plain = nb.Pathtracer(W, H, nb.Globals(bounces=desc.bounces))
    for spp in (16, 64):
        frame(plain, last, spp)
        ms = frame(plain, last, spp)
        out["plain"][f"{spp}spp"] = {"relmse": score(plain.download(stream=sh)), "ms": round(ms, 2)}
    # environment next-event estimation (no cache): the opt-in estimator aimed at the sun disc
    out["nee"] = {}
    plain.set_sampling(env_nee=True)
    for spp in (4, 16, 64):
        frame(plain, last, spp)
        ms = frame(plain, last, spp)
        out["nee"][f"{spp}spp"] = {"relmse": score(plain.download(stream=sh)), "ms": round(ms, 2)}
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
            m[f"{spp}spp"] = {"relmse": score(pt.download(stream=sh)), "ms": round(ms, 2)}
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
             ms and relMSE against the binary64 16,384-spp oracle truth of the full frame
             (tests/golden/truth_spheres_256.npz), plus a GPU render of the truth's own samples
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
    truth = load_truth("spheres_256")
    if truth is not None and not truth_matches(desc, truth):
        truth = None

    def score(img):
        return None if truth is None else round(rel_mse_truth(img, truth), 6)

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
    full = None
    if truth is not None:
        ref_pt = nb.Pathtracer(256, 256, nb.Globals(bounces=6), sobol_table=nb.sobol_burley_table(int(truth["spp"]), 17))
        ref_pt.render(scene, cam, env, int(truth["spp"]))
        full = ref_pt.download()
    osc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    t = time.perf_counter()
    cimg, crays, _, _ = osc.render(desc.clip_to_world, 256, 256, O.sobol_table(), 1, 16, bounces=6,
                                   env=desc.env_color, threads=threads)
    cs = time.perf_counter() - t
    out["spheres_256_16spp"] = {
        "gpu": {"mrays_s": round(rays / ms / 1e3, 1), "frame_ms": round(ms, 3), "rays": int(rays),
                "relmse": score(img), "nonfinite_pixels": nonfinite_pixels(img),
                "bit_equal_to_oracle_pixels": round(float(np.mean(np.all(img == cimg, axis=-1))), 5)},
        "cpu": {"mrays_s": round(crays / cs / 1e6, 2), "frame_ms": round(cs * 1e3, 1), "rays": int(crays),
                "relmse": score(cimg), "nonfinite_pixels": nonfinite_pixels(cimg)},
        "gpu_rr_from_bounce_3": {"mrays_s": round(rays3 / ms3 / 1e3, 1), "frame_ms": round(ms3, 3),
                                 "rays": int(rays3), "relmse": score(img3)},
        "gpu_truth_samples_vs_truth_relmse": None if full is None else score(full),
        "rr": "reference schedule (cf 4) unless stated; the variant disables roulette before bounce 3",
        **(truth_note(truth, "spheres_256") if truth is not None else {"truth": "unavailable"})}
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
            gms = {}
            for incoherent in (False, True):  # warps of 32 neighbours vs lane refill (NB_TRACE_INCOHERENT)
                for _ in range(3):
                    soup.trace_device(d_rays.data_ptr(), n, hits.data_ptr(), inst.data_ptr(), any_hit=any_hit,
                                      incoherent=incoherent)
                a.record()
                for _ in range(5):
                    soup.trace_device(d_rays.data_ptr(), n, hits.data_ptr(), inst.data_ptr(), any_hit=any_hit,
                                      incoherent=incoherent)
                b.record()
                b.synchronize()
                gms[incoherent] = a.elapsed_time(b) / 5
            m = 1 << 18
            t = time.perf_counter()
            osc.trace(rays[:m], any_hit=any_hit, threads=threads)
            cs = time.perf_counter() - t
            best = min(gms.values())
            res[f"{kind}_{'any' if any_hit else 'closest'}"] = {
                "gpu_mrays_s": round(n / best / 1e3, 1), "gpu_ms": round(best, 3),
                "gpu_ms_warp_of_neighbours": round(gms[False], 3), "gpu_ms_lane_refill": round(gms[True], 3),
                "cpu_mrays_s": round(m / cs / 1e6, 2), "ratio": round((n / best / 1e3) / (m / cs / 1e6), 1)}
        del d_rays, hits, inst
    out["soup_1m_16m_rays"] = res
    return out


class _DeviceView:
    """A torch view of a device buffer the library owns (no copy)."""

    def __init__(self, ptr, shape):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": "<f4", "data": (int(ptr), False),
                                         "version": 3}


def trace_roofline(pt, scene, cam, env, desc, kt, steps, rays_per_step, sh, of):
    """Roofline of the traversal kernel from one instrumented frame outside the timed region.

    achieved = the bytes the device's own layout fetches per trace launch (80 B per 8-wide node
    test, 48 B per triangle test, 64 B per instance entry, 16 B per stack entry written and read
    back, 52 B of ray in / hit out), counted by nb_trace_counters, divided by the timed average
    trace launch duration; peak = the measured HBM copy bandwidth.  Most of those bytes are
    served by L1 and L2, so frac is the kernel's distance from the memory roofline, and the
    kernel itself is bound by the latency of its dependent loads (bound "latency")."""
    pt.enable_trace_counters(True)
    pt.invalidate()
    pt.render(scene, cam, env, desc.spp, stream=sh)
    c = pt.trace_counters(desc.bounces + 1, reset=True, stream=sh)
    pt.enable_trace_counters(False)

    def bytes_of(x):
        return (NODE_BYTES * (x["tlas_node_tests"] + x["blas_node_tests"]) + TRI_BYTES * x["triangle_tests"]
                + INST_BYTES * x["instance_entries"] + PUSH_BYTES * x["stack_pushes"] + RAY_IO_BYTES * x["rays"])

    def per_ray(xs):
        r = max(1, sum(x["rays"] for x in xs))
        keys = ("tlas_node_tests", "blas_node_tests", "triangle_tests", "instance_entries", "stack_pushes")
        return {**{k: round(sum(x[k] for x in xs) / r, 3) for k in keys},
                "bytes": round(sum(bytes_of(x) for x in xs) / r, 1), "rays": int(r)}

    def lanes(xs):
        # how a warp's 32 lanes share the node steps (the instrumented kernel's warp-step counts)
        tot = {k: sum(x[k] for x in xs) for k in ("warp_steps", "lane_steps", "leaf_steps", "leaf_lanes",
                                                   "leaf_warp_triangles", "triangle_tests")}
        ws, ls = max(1, tot["warp_steps"]), max(1, tot["leaf_steps"])
        return {"lanes_per_step": round(tot["lane_steps"] / ws, 2),
                "leaf_step_frac": round(tot["leaf_steps"] / ws, 3),
                "leaf_lanes_per_leaf_step": round(tot["leaf_lanes"] / ls, 2),
                "warp_triangle_iterations_per_leaf_step": round(tot["leaf_warp_triangles"] / ls, 2),
                "leaf_loop_lane_use": round(tot["triangle_tests"] / max(1, 32 * tot["leaf_warp_triangles"]), 3)}

    counted_rays = sum(x["rays"] for x in c)
    total_bytes = sum(bytes_of(x) for x in c)
    launches = max(1, kt["trace_launches"]) / steps
    avg_launch_ms = kt["trace_ms"] / max(1, kt["trace_launches"])
    bytes_per_launch = total_bytes / launches
    achieved = bytes_per_launch / (avg_launch_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    rays_per_launch = rays_per_step / launches
    line = {"bound": "latency", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": round(TRACE_DRAM_BYTES_PER_RAY * rays_per_launch),
            "kernel": "k_trace_wave", "peak_kind": f"{peak_kind} hbm_gbs (copy)",
            "bytes_per_launch": round(bytes_per_launch), "avg_launch_ms": round(avg_launch_ms, 4),
            "counted_rays_per_step": int(counted_rays),
            "device_work_per_ray": {"bounce_0": per_ray(c[:1]), "bounces_1_plus": per_ray(c[1:])},
            "warp_lanes": {"bounce_0": lanes(c[:1]), "bounces_1_plus": lanes(c[1:])},
            "rays_per_bounce": [x["rays"] for x in c],
            "traffic_note": "ncu dram bytes per ray of all trace launches of the 480x270 64-spp small case "
                            "(profiles/k_trace_wave__instanced_480x270_64spp.md) x rays per launch",
            "issue_active_pct": TRACE_ISSUE_ACTIVE_PCT,
            "note": "achieved = bytes the 8-wide device layout fetches (instrumented counters of one extra "
                    "frame) / timed trace launch time, against the HBM copy peak; mostly L1/L2 hits.  The "
                    "binding limit is instruction issue (issue_active_pct: the schedulers issue in 75-77% of "
                    "cycles, ncu on the 480x270 64-spp case) with SIMT divergence, not DRAM bandwidth"}
    if of is not None:
        n_aabb, n_tri, n_inst = of.work_per_ray()
        line["reference_algorithm"] = {
            "bytes_per_ray": round(32.0 * n_aabb + 48.0 * n_tri + 128.0 * n_inst, 1),
            "n_aabb": round(n_aabb, 2), "n_tri": round(n_tri, 2), "n_inst": round(n_inst, 2),
            "note": "the reference's binary-BVH work per query (32 B per box test, 48 per triangle, 128 per "
                    "instance), counted by the oracle on the CPU sample: the work the device layout replaces"}
    return line


def train_bench(args, rows=16384, warm=10, steps=100):
    """Radiance-cache training on its own: Adam steps over `rows` seeded encoded rows (targets a
    smooth function the network can fit), per tensor-core path; CUDA-event time per step
    (each step returns its loss to the host, so the time includes that synchronisation)."""
    import torch
    import nbounce_gb300 as nb
    from nbounce_gb300 import _lib as L
    rng = np.random.default_rng(0)
    x = rng.uniform(-1.0, 1.0, (rows, 64)).astype(np.float32)
    x[:, 62], x[:, 63] = 1.0, 0.0
    y = (0.5 + 0.4 * np.sin(x[:, :3] * 2.0 + x[:, 3:6])).astype(np.float32)
    X, Y = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    out = {"rows_per_step": rows, "steps": steps, "flop_per_step": rows * MLP_FLOP_PER_RECORD}
    for name, tp in (("tcgen05", L.NB_CACHE_TCGEN05), ("mma_sync", L.NB_CACHE_MMA_SYNC)):
        c = nb.RadianceCache(seed=9, learning_rate=5e-3, tensor_path=tp)
        for _ in range(warm):
            c.train_step(X, Y, rows)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        losses = [c.train_step(X, Y, rows) for _ in range(steps)]
        b.record()
        b.synchronize()
        out[name] = {"ms_per_step": round(a.elapsed_time(b) / steps, 4), "final_loss": round(losses[-1], 6)}
        c.close()
    return out


def run_ours(args):
    import torch
    import nbounce_gb300 as nb
    from nbounce_gb300 import replicas

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    grouped = world > 1 or args.shard_frame  # --shard-frame merges over NCCL even with one rank
    if grouped:
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        os.environ.setdefault("MASTER_PORT", str(free_port()))
        torch.distributed.init_process_group("nccl", rank=rank, world_size=world,
                                             device_id=torch.device("cuda", local))
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
    shard = args.shard_frame
    first, count = replicas.shard_samples(desc.spp, rank, world) if shard else (1, desc.spp)
    ptr, w, h = pt.output_texture()
    image = torch.as_tensor(_DeviceView(ptr, (h, w, 4)), device=dev)

    def step():
        pt.invalidate()
        if shard:
            # rows first..first+count-1 continue a running mean that starts from a zero image
            image.zero_()
            g = pt.globals
            g.sample = first - 1
            pt.globals = g
        pt.render(scene, cam, env, count, stream=sh)
        if shard:
            return replicas.merge_running_means_distributed(image, first + count - 1, count)
        return image

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
        img = step()
        if shard:
            host_img.copy_(img)
        else:
            pt.download(out=host_np, stream=sh)
    e2e_s = time.perf_counter() - t
    barrier()

    t_max = ms
    e2e_max = e2e_s
    total_rays = rays_per_step * args.steps
    if world > 1:
        v = torch.tensor([ms, e2e_s], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(v, op=torch.distributed.ReduceOp.MAX)
        r = torch.tensor([float(total_rays)], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(r)
        t_max, e2e_max, total_rays = float(v[0]), float(v[1]), float(r[0])
    value = total_rays / (t_max / 1e3) / 1e6
    e2e_value = total_rays / e2e_max / 1e6
    if rank != 0:
        if grouped:
            torch.distributed.destroy_process_group()
        return None
    launches_per_step = sum(kt[k] for k in ("raygen_launches", "trace_launches", "shade_launches",
                                             "accumulate_launches")) / args.steps
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": round(t_max / args.steps, 3), "higher_is_better": True,
        "scaling": "strong" if shard else "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scene generator)",
        "config": workload_config(desc, world, shard),
        "workload_stats": {"rays_per_step": int(total_rays / args.steps), "scene_build_s": round(build_s, 2),
                           "estimator": "environment NEE (opt-in)" if args.env_nee else "reference"},
        "e2e": {"value": round(e2e_value, 2), "unit": UNIT, "h2d_bytes_per_step": 128,
                "d2h_bytes_per_step": int(desc.width * desc.height * 16)},
        "gpu_launches": int(round(launches_per_step * args.steps)),
        "kernel_ms_per_step": {k: round(kt[k] / args.steps, 3) for k in ("raygen_ms", "trace_ms", "shade_ms",
                                                                       "accumulate_ms")},
        "clocks": clocks.summary(),
    }
    of = None
    if not args.no_cpu_baseline and not args.env_nee and world == 1:
        base, of = cpu_baseline(desc, args.cpu_seconds, os.cpu_count() or 1)
        line["cpu_baseline"] = base
    if not args.env_nee and world == 1:
        line["roofline"] = trace_roofline(pt, scene, cam, env, desc, kt, args.steps, rays_per_step, sh, of)
    if not args.no_serving and world == 1:
        line["quality"] = quality_report(args, desc, scene, env, stream)
        line["serving"] = serving_report(args)
    if not args.no_cache and world == 1:
        line["cache"] = cache_report(args, desc, scene, env, stream)
    if grouped:
        torch.distributed.destroy_process_group()
    return line


def run_reference(args):
    """The reference arm: the oracle (the CPU restatement of the reference pass; oracle/ only,
    libnbounce.so is never loaded) on all host threads, each step one CPU sample of the same
    frame (24 stratified 16x16 tiles at 64 spp).  Under a launcher only rank 0 runs."""
    rank, world, _ = dist_env()
    if rank != 0:
        return None
    desc = build_workload(args)
    threads = os.cpu_count() or 1
    of = OracleFrame(desc, threads)
    for _ in range(args.warmup):
        of.step()
    total_rays, t = 0, time.perf_counter()
    for _ in range(args.steps):
        total_rays += of.step()
    dt = time.perf_counter() - t
    value = total_rays / dt / 1e6
    return {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
            "impl": "reference", "config": workload_config(desc, world),
            "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{of.sample_text()} per step: {total_rays} rays in {dt:.1f} s"},
            "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ and not args.all_configs:
        sys.exit(launch_ranks(args.gpus, os.path.abspath(__file__), sys.argv[1:]))
    args.serving_loads = [(float(a), int(b)) for a, b in (x.split(":") for x in args.serving_loads.split(","))]
    if args.all_configs:
        line = configs_report(args)
    elif args.train_bench:
        line = train_bench(args)
    else:
        line = run_reference(args) if args.impl == "reference" else run_ours(args)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
