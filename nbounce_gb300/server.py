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
               contribution_factor=4.0, out=None, flags=0, deadline_ms=0, busy_ok=False):
        """Queues a job; `out` (h, w, 4) float32 receives the image when it finishes.

        `flags`: NB_JOB_ENV_NEE (environment next-event estimation) or NB_JOB_CACHE (the
        server's radiance cache of the scene), 0 for the reference estimator.  `deadline_ms`:
        the job fails with NB_ERR_EXPIRED if unfinished this long after submission (0: none).
        With busy_ok, a full queue returns None instead of raising (the job was shed)."""
        d = L.NbJobDesc()
        d.scene, d.env = scene, env
        d.camera = camera_struct(world_to_clip, clip_to_world)
        d.width, d.height, d.spp, d.bounces = width, height, spp, bounces
        d.contribution_factor = contribution_factor
        d.flags = flags
        d.deadline_ms = int(deadline_ms)
        d.host_out = None if out is None else out.ctypes.data
        jid = C.c_uint64()
        st = lib().nb_server_submit(self._h, C.byref(d), C.byref(jid))
        if st == L.NB_ERR_BUSY and busy_ok:
            return None
        check(st)
        return jid.value

    def set_queue_limit(self, max_queued):
        """At most max_queued jobs wait for admission; submissions beyond get NB_ERR_BUSY (0: no limit)."""
        check(lib().nb_server_set_queue_limit(self._h, int(max_queued)))

    def cancel(self, job):
        """Cancels an unfinished job; it finishes with NB_ERR_CANCELLED."""
        check(lib().nb_server_cancel(self._h, job))

    def fail_alloc(self, nth):
        """Test hook: the nth job-image allocation from now on fails as an out-of-memory one."""
        check(lib().nb_server_fail_alloc(self._h, int(nth)))

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
        """The job's info once it finished (info["status"] is its outcome, NB_OK or the
        error it failed with), or with done = 0 after timeout_ms."""
        info = L.NbJobInfo()
        st = lib().nb_server_wait(self._h, job, int(timeout_ms), C.byref(info))
        if st not in (L.NB_OK, L.NB_ERR_TIMEOUT) and not info.done:
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


def run_load(server, scene_slots, env_slot, cameras, trace, bounces=8, sample_every_s=0.05):
    """Replays `trace` against the server; returns latency percentiles and throughput.

    Jobs the server sheds (NB_ERR_BUSY: its queue limit is reached) are counted as rejected
    and not retried.  Latency is submit -> finish of the admitted jobs, queue time submit ->
    admit.  A sampler thread records the server's queued / active job counts over the run.
    Finished jobs are waited for and released in submission order by a second thread, so
    their host images are dropped as they complete."""
    import queue as Q
    outs = {}
    submitted = Q.Queue()
    infos = []
    series = []
    t0 = time.perf_counter()
    stats0 = server.stats()
    stop = threading.Event()

    def waiter():
        while True:
            j = submitted.get()
            if j is None:
                return
            infos.append(server.wait(j))
            server.release(j)
            outs.pop(j, None)

    def sampler():
        while not stop.is_set():
            st = server.stats()
            series.append((time.perf_counter() - t0, st["queued"], st["active"]))
            stop.wait(sample_every_s)

    threads = [threading.Thread(target=waiter, daemon=True), threading.Thread(target=sampler, daemon=True)]
    for th in threads:
        th.start()
    flags_kept, rejected = [], 0
    for arrival, scene, (w, h), spp, flags in trace:
        delay = arrival - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        out = np.empty((h, w, 4), np.float32)
        w2c, c2w = cameras[scene](w, h)
        j = server.submit(scene_slots[scene], env_slot, w2c, c2w, w, h, spp, bounces, out=out, flags=flags,
                          busy_ok=True)
        if j is None:
            rejected += 1
            continue
        outs[j] = out
        flags_kept.append(flags)
        submitted.put(j)
    submitted.put(None)
    threads[0].join()
    wall = time.perf_counter() - t0
    stop.set()
    threads[1].join()
    stats1 = server.stats()
    ok = np.array([i["status"] == 0 for i in infos], bool)
    lat = np.array([i["finish_ms"] - i["submit_ms"] for i in infos])[ok]
    queue = np.array([i["admit_ms"] - i["submit_ms"] for i in infos])[ok]
    rays = stats1["rays"] - stats0["rays"]
    busy = stats1["gpu_busy_ms"] - stats0["gpu_busy_ms"]
    flags = np.array(flags_kept)[ok]
    by_option = {}
    for f in sorted(set(flags.tolist())):
        sel = lat[flags == f]
        by_option[OPTION_NAMES.get(f, str(f))] = {"jobs": int(sel.size), "p50_ms": float(np.percentile(sel, 50)),
                                                  "p99_ms": float(np.percentile(sel, 99))}
    extra = {"by_option": by_option} if len(by_option) > 1 else {}
    q = np.array([s[1] for s in series] or [0])
    a = np.array([s[2] for s in series] or [0])
    step = max(1, len(series) // 24)
    pct = (lambda x, p: float(np.percentile(x, p)) if x.size else None)
    return {**extra, "jobs": len(trace), "admitted": len(infos), "rejected": rejected,
            "failed": int((~ok).sum()), "completed": int(ok.sum()),
            "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99), "mean_ms": float(lat.mean()) if lat.size else None,
            "p50_queue_ms": pct(queue, 50), "p99_queue_ms": pct(queue, 99),
            "queued_max": int(q.max()), "queued_mean": float(q.mean()), "active_max": int(a.max()),
            "queue_series": [[round(t, 2), int(qq), int(aa)] for t, qq, aa in series[::step]],
            "wall_s": wall, "rays": int(rays), "mrays_per_s_wall": rays / wall / 1e6,
            "mrays_per_s_busy": rays / max(busy, 1e-9) / 1e3, "gpu_busy_frac": busy / 1e3 / wall,
            "jobs_per_s_completed": float(ok.sum()) / wall,
            "waves": int(stats1["waves"] - stats0["waves"]), "peak_bytes": int(stats1["peak_bytes_in_use"]),
            "bytes_in_use_after": int(stats1["bytes_in_use"])}
