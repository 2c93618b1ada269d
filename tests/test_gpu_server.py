"""Render-job server: continuous batching on the GPU.

Each job's image must be bit-identical to rendering the same job alone with the
Pathtracer (every path depends only on its job, pixel and sample; samples reach the image in
order), whatever it was batched with; admission must respect the HBM budget.
"""
import numpy as np
import pytest

import nbounce_gb300 as nb
from nbounce_gb300 import _lib as L
from nbounce_gb300 import scenes
from nbounce_gb300.server import RenderServer

pytestmark = pytest.mark.gpu

PATH_BYTES = 11 * 16 + 4  # per path of the server's buffers (queues, hits, radiance, shadow rays)


def fixed_bytes(paths):
    return paths * PATH_BYTES + 2 * 64 * 4 + 1024 * 17 * 16 + 2 * 64 * 4 + 16 + 8


@pytest.fixture(scope="module")
def world():
    sph = scenes.spheres_scene(width=48, height=32, spp=3, bounces=6)
    ins = scenes.instanced_scene(n_instances=64, width=40, height=24, spp=2, bounces=8, env_size=(64, 32),
                                 scale=1 / 128)
    s0 = nb.SceneBuffers.from_desc(sph)
    s1 = nb.SceneBuffers.from_desc(ins)
    e0 = nb.EnvMap(sph.env_color)
    e1 = nb.EnvMap(texels=ins.env_texels)
    return dict(descs=(sph, ins), scenes=(s0, s1), envs=(e0, e1))


def alone(world, k, w, h, spp, bounces, env_nee=False):
    w2c, c2w = scenes.camera_matrices(*CAMS[k], w, h)
    pt = nb.Pathtracer(w, h, nb.Globals(bounces=bounces))
    pt.set_sampling(env_nee=env_nee)
    pt.render(world["scenes"][k], nb.camera_struct(w2c, c2w), world["envs"][k], spp)
    return pt.download()


CAMS = {0: ((0.0, 6.0, 34.0), (0.0, -1.0, 0.0)), 1: ((0.0, 14.0, 62.0), (0.0, -2.0, 0.0))}
JOBS = [(0, 48, 32, 3, 6), (1, 40, 24, 2, 8), (0, 64, 64, 5, 4), (1, 32, 32, 1, 8), (0, 16, 48, 7, 6),
        (1, 80, 40, 3, 2)]


def submit_all(srv, slots, env_slots, outs):
    ids = []
    for (k, w, h, spp, b), out in zip(JOBS, outs):
        w2c, c2w = scenes.camera_matrices(*CAMS[k], w, h)
        ids.append(srv.submit(slots[k], env_slots[k], w2c, c2w, w, h, spp, b, out=out))
    return ids


def test_mixed_jobs_equal_jobs_rendered_alone(world):
    paths = 1 << 14  # small waves: every job is split over several waves and shares them
    srv = RenderServer(hbm_budget_bytes=1 << 30, paths_per_wave=paths)
    slots = [srv.add_scene(s) for s in world["scenes"]]
    env_slots = [srv.add_env(e) for e in world["envs"]]
    outs = [np.full((h, w, 4), np.nan, np.float32) for (_, w, h, _, _) in JOBS]
    ids = submit_all(srv, slots, env_slots, outs)
    infos = [srv.wait(j, timeout_ms=120000) for j in ids]
    assert all(i["done"] == 1 and i["status"] == 0 for i in infos)
    st = srv.stats()
    assert st["jobs_done"] == len(JOBS) and st["waves"] > 1
    for (k, w, h, spp, b), out in zip(JOBS, outs):
        ref = alone(world, k, w, h, spp, b)
        assert np.array_equal(out, ref), (k, w, h, spp, b)
    srv.close()


def test_budget_limits_admission_and_all_jobs_finish(world):
    paths = 1 << 14
    biggest = max(w * h for (_, w, h, _, _) in JOBS) * 16
    budget = fixed_bytes(paths) + 2 * biggest
    srv = RenderServer(hbm_budget_bytes=budget, paths_per_wave=paths)
    slots = [srv.add_scene(s) for s in world["scenes"]]
    env_slots = [srv.add_env(e) for e in world["envs"]]
    outs = [np.zeros((h, w, 4), np.float32) for (_, w, h, _, _) in JOBS]
    ids = submit_all(srv, slots, env_slots, outs)
    infos = [srv.wait(j, timeout_ms=120000) for j in ids]
    assert all(i["done"] == 1 and i["status"] == 0 for i in infos)
    st = srv.stats()
    assert st["peak_bytes_in_use"] <= budget
    assert all(np.isfinite(o).all() and (o[..., 3] == 1.0).all() for o in outs)
    srv.close()


def test_invalid_jobs_are_rejected(world):
    paths = 1 << 12
    srv = RenderServer(hbm_budget_bytes=fixed_bytes(paths) + 32 * 32 * 16, paths_per_wave=paths)
    slot = srv.add_scene(world["scenes"][0])
    env = srv.add_env(world["envs"][0])
    w2c, c2w = scenes.camera_matrices(*CAMS[0], 32, 32)
    with pytest.raises(nb.NbError) as e:
        srv.submit(slot + 5, env, w2c, c2w, 32, 32, 1)
    assert e.value.status == 1
    with pytest.raises(nb.NbError) as e:  # larger than one wave's paths
        srv.submit(slot, env, w2c, c2w, 128, 64, 1)
    assert e.value.status == 1
    with pytest.raises(nb.NbError) as e:  # fits one wave (2304 <= 4096 paths), not the budget
        srv.submit(slot, env, w2c, c2w, 48, 48, 1)
    assert e.value.status == 2
    job = srv.submit(slot, env, w2c, c2w, 32, 32, 2)
    info = srv.wait(job, timeout_ms=60000)
    assert info["done"] == 1
    img = srv.fetch(job, 32, 32)
    assert np.array_equal(img, alone(world, 0, 32, 32, 2, 8))
    srv.close()


def test_nee_jobs_share_waves_and_equal_jobs_rendered_alone(world):
    """NB_JOB_ENV_NEE jobs ride in the same waves as reference-estimator jobs; every image
    equals its job rendered alone with the matching sampling mode."""
    paths = 1 << 14
    srv = RenderServer(hbm_budget_bytes=1 << 30, paths_per_wave=paths)
    slots = [srv.add_scene(s) for s in world["scenes"]]
    env_slots = [srv.add_env(e) for e in world["envs"]]
    flags = [L.NB_JOB_ENV_NEE if i % 2 else 0 for i in range(len(JOBS))]
    outs = [np.full((h, w, 4), np.nan, np.float32) for (_, w, h, _, _) in JOBS]
    ids = []
    for (k, w, h, spp, b), out, f in zip(JOBS, outs, flags):
        w2c, c2w = scenes.camera_matrices(*CAMS[k], w, h)
        ids.append(srv.submit(slots[k], env_slots[k], w2c, c2w, w, h, spp, b, out=out, flags=f))
    infos = [srv.wait(j, timeout_ms=120000) for j in ids]
    assert all(i["done"] == 1 and i["status"] == 0 for i in infos)
    assert srv.stats()["waves"] > 1
    for (k, w, h, spp, b), out, f in zip(JOBS, outs, flags):
        ref = alone(world, k, w, h, spp, b, env_nee=bool(f))
        assert np.array_equal(out, ref), (k, w, h, spp, b, f)
    # the NEE estimator changes the image (same job, other estimator)
    k, w, h, spp, b = JOBS[1]
    assert not np.array_equal(outs[1], alone(world, k, w, h, spp, b))
    srv.close()


def test_cache_jobs_run_beside_plain_jobs(world):
    """NB_JOB_CACHE jobs run in cache waves (one scene each) alternated with ordinary waves:
    they finish with finite images, and the ordinary jobs' images stay equal to rendering them
    alone."""
    paths = 1 << 14
    srv = RenderServer(hbm_budget_bytes=1 << 30, paths_per_wave=paths)
    slots = [srv.add_scene(s) for s in world["scenes"]]
    env_slots = [srv.add_env(e) for e in world["envs"]]
    flags = [L.NB_JOB_CACHE if i in (1, 2, 3) else 0 for i in range(len(JOBS))]  # 1 and 3 share a scene
    outs = [np.full((h, w, 4), np.nan, np.float32) for (_, w, h, _, _) in JOBS]
    ids = []
    for (k, w, h, spp, b), out, f in zip(JOBS, outs, flags):
        w2c, c2w = scenes.camera_matrices(*CAMS[k], w, h)
        ids.append(srv.submit(slots[k], env_slots[k], w2c, c2w, w, h, spp, b, out=out, flags=f))
    infos = [srv.wait(j, timeout_ms=120000) for j in ids]
    assert all(i["done"] == 1 and i["status"] == 0 for i in infos)
    for (k, w, h, spp, b), out, f in zip(JOBS, outs, flags):
        if f:
            assert np.isfinite(out).all() and (out[..., :3] >= 0).all() and (out[..., 3] == 1.0).all()
            assert out[..., :3].mean() > 0
        else:
            assert np.array_equal(out, alone(world, k, w, h, spp, b)), (k, w, h, spp, b)
    srv.close()


def test_job_flags_are_validated(world):
    paths = 1 << 12
    srv = RenderServer(hbm_budget_bytes=1 << 30, paths_per_wave=paths)
    slot = srv.add_scene(world["scenes"][0])
    env = srv.add_env(world["envs"][0])
    w2c, c2w = scenes.camera_matrices(*CAMS[0], 32, 32)
    for bad in (4, 1 << 31, L.NB_JOB_ENV_NEE | L.NB_JOB_CACHE):
        with pytest.raises(nb.NbError) as e:
            srv.submit(slot, env, w2c, c2w, 32, 32, 1, flags=bad)
        assert e.value.status == 1
    srv.close()


def test_rejected_cache_config_fails_only_the_cache_jobs(world):
    """A cache configuration nb_cache_create rejects is found when the scene's cache is
    created: that scene's cache jobs fail with its status, every other job completes with its
    usual image, and a later valid configuration serves new cache jobs."""
    paths = 1 << 14
    srv = RenderServer(hbm_budget_bytes=1 << 30, paths_per_wave=paths)
    slots = [srv.add_scene(s) for s in world["scenes"]]
    env_slots = [srv.add_env(e) for e in world["envs"]]
    srv.set_cache_config(train_steps=1000)  # above the 64 steps a cache accepts
    flags = [L.NB_JOB_CACHE if i in (1, 3) else 0 for i in range(len(JOBS))]  # both on scene 1
    outs = [np.full((h, w, 4), np.nan, np.float32) for (_, w, h, _, _) in JOBS]
    ids = []
    for (k, w, h, spp, b), out, f in zip(JOBS, outs, flags):
        w2c, c2w = scenes.camera_matrices(*CAMS[k], w, h)
        ids.append(srv.submit(slots[k], env_slots[k], w2c, c2w, w, h, spp, b, out=out, flags=f))
    for jid, (k, w, h, spp, b), out, f in zip(ids, JOBS, outs, flags):
        if f:
            info = srv.wait(jid, timeout_ms=120000)
            assert info["done"] == 1 and info["status"] == 1
        else:
            info = srv.wait(jid, timeout_ms=120000)
            assert info["done"] == 1 and info["status"] == 0
            assert np.array_equal(out, alone(world, k, w, h, spp, b)), (k, w, h, spp, b)
    assert srv.stats()["jobs_failed"] == 2
    srv.set_cache_config(tensor_path=L.NB_CACHE_MMA_SYNC)
    k, w, h, spp, b = JOBS[1]
    w2c, c2w = scenes.camera_matrices(*CAMS[k], w, h)
    out = np.full((h, w, 4), np.nan, np.float32)
    jid = srv.submit(slots[k], env_slots[k], w2c, c2w, w, h, spp, b, out=out, flags=L.NB_JOB_CACHE)
    info = srv.wait(jid, timeout_ms=120000)
    assert info["status"] == 0 and np.isfinite(out).all() and (out[..., 3] == 1.0).all()
    srv.close()


def test_concurrent_submitters_get_their_own_images(world):
    """nb_server_submit / _wait are thread-safe: four host threads submit and wait at the same
    time; every job ends with the image of the same job rendered alone."""
    import threading
    paths = 1 << 14
    srv = RenderServer(hbm_budget_bytes=1 << 30, paths_per_wave=paths)
    slots = [srv.add_scene(s) for s in world["scenes"]]
    env_slots = [srv.add_env(e) for e in world["envs"]]
    results, errors = {}, []

    def worker(t):
        try:
            for n in range(3):
                k, w, h, spp, b = JOBS[(t + 2 * n) % len(JOBS)]
                w2c, c2w = scenes.camera_matrices(*CAMS[k], w, h)
                out = np.full((h, w, 4), np.nan, np.float32)
                jid = srv.submit(slots[k], env_slots[k], w2c, c2w, w, h, spp, b, out=out,
                                 flags=L.NB_JOB_ENV_NEE if (t + n) % 3 == 0 else 0)
                info = srv.wait(jid, timeout_ms=120000)
                results[(t, n)] = (info, out, (k, w, h, spp, b), (t + n) % 3 == 0)
        except Exception as e:  # surfaced below
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    assert len(results) == 12
    for info, out, job, nee in results.values():
        assert info["done"] == 1 and info["status"] == 0
        assert np.array_equal(out, alone(world, *job, env_nee=nee)), job
    assert srv.stats()["jobs_done"] == 12
    srv.close()


def test_burst_of_small_jobs_completes_and_frees_its_memory(world):
    """Four hundred small jobs submitted at once (sizes, sample counts and estimators mixed):
    every job completes, admission never exceeds the budget, and once the images are delivered
    and the jobs released the server holds only its fixed buffers again."""
    paths = 1 << 15
    budget = fixed_bytes(paths) + 64 * 64 * 16 * 24  # room for ~24 of the largest images at once
    srv = RenderServer(hbm_budget_bytes=budget, paths_per_wave=paths)
    slots = [srv.add_scene(s) for s in world["scenes"]]
    env_slots = [srv.add_env(e) for e in world["envs"]]
    rng = np.random.default_rng(17)
    idle = srv.stats()["bytes_in_use"]
    jobs = []
    for n in range(400):
        k = int(rng.integers(2))
        w, h = int(rng.integers(8, 65)), int(rng.integers(8, 65))
        spp, b = int(rng.integers(1, 5)), int(rng.integers(0, 9))
        flags = [0, L.NB_JOB_ENV_NEE, L.NB_JOB_CACHE][int(rng.integers(3))]
        w2c, c2w = scenes.camera_matrices(*CAMS[k], w, h)
        jobs.append((srv.submit(slots[k], env_slots[k], w2c, c2w, w, h, spp, b, flags=flags), w, h))
    for jid, w, h in jobs:
        info = srv.wait(jid, timeout_ms=300000)
        assert info["done"] == 1 and info["status"] == 0
        img = srv.fetch(jid, w, h)
        assert np.isfinite(img).all() and (img[..., 3] == 1.0).all()
        srv.release(jid)
    st = srv.stats()
    assert st["jobs_done"] == 400 and st["jobs_failed"] == 0
    assert st["peak_bytes_in_use"] <= budget
    assert st["bytes_in_use"] == idle
    srv.close()


def test_cancelled_expired_and_out_of_memory_jobs_fail_alone(world):
    """Host-side failure cases (no GPU fault is involved): a job whose image allocation fails
    (nb_server_fail_alloc arms the second allocation to fail as cudaMallocAsync does when
    memory runs out), a job cancelled while it waits in the queue, a job cancelled after some
    of its waves ran, and a job whose deadline passes.  Each finishes with its own status; the
    other jobs' images equal the same jobs rendered alone; once every job is released the
    server holds only its fixed buffers again."""
    import time
    paths = 1 << 12
    budget = fixed_bytes(paths) + 64 * 64 * 16 + 4 * 32 * 32 * 16  # one 64x64 image at a time
    srv = RenderServer(hbm_budget_bytes=budget, paths_per_wave=paths)
    slots = [srv.add_scene(s) for s in world["scenes"]]
    env_slots = [srv.add_env(e) for e in world["envs"]]
    idle = srv.stats()["bytes_in_use"]
    srv.fail_alloc(2)
    jobs = {"a": (0, 32, 32, 3, 6, 0), "oom": (1, 32, 32, 2, 8, 0), "big": (0, 64, 64, 1000, 6, 0),
            "queued": (1, 64, 64, 4, 8, 0), "late": (0, 24, 24, 1000, 6, 1), "f": (1, 40, 24, 2, 8, 0)}
    ids, outs = {}, {}
    for name, (k, w, h, spp, b, deadline) in jobs.items():
        w2c, c2w = scenes.camera_matrices(*CAMS[k], w, h)
        outs[name] = np.full((h, w, 4), np.nan, np.float32)
        ids[name] = srv.submit(slots[k], env_slots[k], w2c, c2w, w, h, spp, b, out=outs[name],
                               deadline_ms=deadline)
        if name == "queued":  # waits behind "big"'s image for budget
            srv.cancel(ids[name])
    t0 = time.time()
    while srv.stats()["waves"] < 3 and time.time() - t0 < 60:
        time.sleep(0.001)
    srv.cancel(ids["big"])
    infos = {n: srv.wait(j, timeout_ms=120000) for n, j in ids.items()}
    assert all(i["done"] == 1 for i in infos.values())
    want = {"a": 0, "oom": L.NB_ERR_OOM, "big": L.NB_ERR_CANCELLED, "queued": L.NB_ERR_CANCELLED,
            "late": L.NB_ERR_EXPIRED, "f": 0}
    assert {n: i["status"] for n, i in infos.items()} == want
    for name in ("a", "f"):
        k, w, h, spp, b, _ = jobs[name]
        assert np.array_equal(outs[name], alone(world, k, w, h, spp, b)), name
    with pytest.raises(nb.NbError) as e:  # a finished job cannot be cancelled
        srv.cancel(ids["a"])
    assert e.value.status == L.NB_ERR_INVALID_ARG
    st = srv.stats()
    assert (st["jobs_cancelled"], st["jobs_expired"], st["jobs_failed"], st["jobs_done"]) == (2, 1, 4, 2)
    for j in ids.values():
        srv.release(j)
    assert srv.stats()["bytes_in_use"] == idle
    srv.close()  # waits for the cancelled jobs' waves still on the GPU


def test_overload_sheds_jobs_and_returns_to_idle(world):
    """Two hundred jobs submitted back to back against a queue limit of 8: submissions beyond
    the limit are rejected with NB_ERR_BUSY at once, every admitted job completes (no stall),
    and after the jobs are released the server's device memory is back to its idle level."""
    paths = 1 << 14
    srv = RenderServer(hbm_budget_bytes=1 << 30, paths_per_wave=paths)
    slots = [srv.add_scene(s) for s in world["scenes"]]
    env_slots = [srv.add_env(e) for e in world["envs"]]
    srv.set_queue_limit(8)
    idle = srv.stats()["bytes_in_use"]
    rng = np.random.default_rng(5)
    accepted, rejected = [], 0
    for n in range(200):
        k = int(rng.integers(2))
        w, h = int(rng.integers(16, 65)), int(rng.integers(16, 65))
        w2c, c2w = scenes.camera_matrices(*CAMS[k], w, h)
        jid = srv.submit(slots[k], env_slots[k], w2c, c2w, w, h, int(rng.integers(1, 9)), 8, busy_ok=True)
        if jid is None:
            rejected += 1
        else:
            accepted.append(jid)
    assert rejected > 0 and len(accepted) >= 8
    for jid in accepted:
        info = srv.wait(jid, timeout_ms=120000)
        assert info["done"] == 1 and info["status"] == 0
        srv.release(jid)
    st = srv.stats()
    assert st["jobs_rejected"] == rejected and st["jobs_submitted"] == len(accepted)
    assert st["jobs_done"] == len(accepted) and st["queued"] == 0 and st["active"] == 0
    assert st["bytes_in_use"] == idle
    srv.close()
