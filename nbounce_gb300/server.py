"""Render-job server (continuous batching) over the C ABI, and a seeded load generator.

``RenderServer`` wraps nb_server_*: resident scenes and environments are registered once,
jobs (scene, camera, resolution, spp, bounces) are submitted from any thread, the native
scheduler batches their samples into shared wavefronts, and each job reports submit /
admit / finish times on the server clock.  ``run_load`` replays a Poisson arrival trace and
returns p50/p99 job latency and throughput.
"""
import ctypes as C
import threading
import time

import numpy as np

from . import _lib as L
from ._lib import check, lib
from .pathtracer import camera_struct


class RenderServer:
    def __init__(self, hbm_budget_bytes=120 << 30, paths_per_wave=1 << 25):
        h = C.c_void_p()
        check(lib().nb_server_create(int(hbm_budget_bytes), int(paths_per_wave), C.byref(h)))
        self._h = h
        self._keep = []

    def add_scene(self, scene):
        slot = C.c_uint32()
        check(lib().nb_server_add_scene(self._h, scene.handle, C.byref(slot)))
        self._keep.append(scene)
        return slot.value

    def add_env(self, env):
        slot = C.c_uint32()
        check(lib().nb_server_add_env(self._h, env.handle, C.byref(slot)))
        self._keep.append(env)
        return slot.value

    def submit(self, scene, env, world_to_clip, clip_to_world, width, height, spp, bounces=8,
               contribution_factor=4.0, out=None, flags=0):
        """Queues a job; `out` (h, w, 4) float32 receives the image when it finishes.

        `flags`: NB_JOB_ENV_NEE (environment next-event estimation) or NB_JOB_CACHE (the
        server's radiance cache of the scene), 0 for the reference estimator."""
        d = L.NbJobDesc()
        d.scene, d.env = scene, env
        d.camera = camera_struct(world_to_clip, clip_to_world)
        d.width, d.height, d.spp, d.bounces = width, height, spp, bounces
        d.contribution_factor = contribution_factor
        d.flags = flags
        d.host_out = None if out is None else out.ctypes.data
        jid = C.c_uint64()
        check(lib().nb_server_submit(self._h, C.byref(d), C.byref(jid)))
        return jid.value

    def set_cache_config(self, **fields):
        """Configuration of the radiance caches created from now on for NB_JOB_CACHE jobs:
        nb_cache_default_config with the given fields replaced (no fields: the defaults)."""
        cfg = L.NbCacheConfig()
        lib().nb_cache_default_config(C.byref(cfg))
        for k, v in fields.items():
            if not hasattr(cfg, k):
                raise AttributeError(f"nb_cache_config has no field {k!r}")
            setattr(cfg, k, v)
        check(lib().nb_server_set_cache_config(self._h, C.byref(cfg) if fields else None))

    def wait(self, job, timeout_ms=-1):
        info = L.NbJobInfo()
        st = lib().nb_server_wait(self._h, job, int(timeout_ms), C.byref(info))
        if st not in (L.NB_OK, L.NB_ERR_TIMEOUT):
            check(st)
        return {k: getattr(info, k) for k, _ in L.NbJobInfo._fields_}

    def fetch(self, job, width, height):
        out = np.empty((height, width, 4), np.float32)
        check(lib().nb_server_fetch(self._h, job, out.ctypes.data_as(C.c_void_p)))
        return out

    def release(self, job):
        check(lib().nb_server_release(self._h, job))

    def stats(self):
        s = L.NbServerStats()
        check(lib().nb_server_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in L.NbServerStats._fields_}

    def close(self):
        if self._h:
            lib().nb_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


RESOLUTIONS = ((256, 256), (512, 512), (1024, 768), (1920, 1080))
SPPS = (1, 4, 16, 64)


def make_trace(n_jobs, rate_per_s, n_scenes, seed=0x5EED4, resolutions=RESOLUTIONS, spps=SPPS, options=None):
    """Seeded Poisson arrivals: (arrival_s, scene, (w, h), spp, flags) per job.

    `options`: job flags drawn uniformly per job (from a second seeded stream, so that the
    arrivals, scenes, sizes and sample counts equal those of the same trace without them);
    None: every job uses the reference estimator (flags 0)."""
    rng = np.random.default_rng(seed)
    opt_rng = np.random.default_rng(seed ^ 0x0F7105)
    t = np.cumsum(rng.exponential(1.0 / rate_per_s, n_jobs))
    out = []
    for k in range(n_jobs):
        w, h = resolutions[rng.integers(len(resolutions))]
        flags = 0 if options is None else int(options[opt_rng.integers(len(options))])
        out.append((float(t[k]), int(rng.integers(n_scenes)), (int(w), int(h)), int(spps[rng.integers(len(spps))]),
                    flags))
    return out


OPTION_NAMES = {0: "reference", L.NB_JOB_ENV_NEE: "env_nee", L.NB_JOB_CACHE: "cache"}


def run_load(server, scene_slots, env_slot, cameras, trace, bounces=8):
    """Replays `trace` against the server; returns latency percentiles and throughput."""
    jobs = []
    outs = []
    t0 = time.perf_counter()
    stats0 = server.stats()
    for arrival, scene, (w, h), spp, flags in trace:
        delay = arrival - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        out = np.empty((h, w, 4), np.float32)
        w2c, c2w = cameras[scene](w, h)
        jobs.append(server.submit(scene_slots[scene], env_slot, w2c, c2w, w, h, spp, bounces, out=out, flags=flags))
        outs.append(out)
    infos = [server.wait(j) for j in jobs]
    wall = time.perf_counter() - t0
    stats1 = server.stats()
    for j in jobs:
        server.release(j)
    lat = np.array([i["finish_ms"] - i["submit_ms"] for i in infos])
    queue = np.array([i["admit_ms"] - i["submit_ms"] for i in infos])
    rays = stats1["rays"] - stats0["rays"]
    busy = stats1["gpu_busy_ms"] - stats0["gpu_busy_ms"]
    flags = np.array([job[4] for job in trace])
    by_option = {}
    for f in sorted(set(flags.tolist())):
        sel = lat[flags == f]
        by_option[OPTION_NAMES.get(f, str(f))] = {"jobs": int(sel.size), "p50_ms": float(np.percentile(sel, 50)),
                                                  "p99_ms": float(np.percentile(sel, 99))}
    extra = {"by_option": by_option} if len(by_option) > 1 else {}
    return {**extra, "jobs": len(jobs), "failed": int(sum(i["status"] != 0 for i in infos)),
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "p99_queue_ms": float(np.percentile(queue, 99)),
            "wall_s": wall, "rays": int(rays), "mrays_per_s_wall": rays / wall / 1e6,
            "mrays_per_s_busy": rays / max(busy, 1e-9) / 1e3, "gpu_busy_frac": busy / 1e3 / wall,
            "waves": int(stats1["waves"] - stats0["waves"]), "peak_bytes": int(stats1["peak_bytes_in_use"])}
