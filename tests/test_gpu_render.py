"""Parity of the full pass (ray generation, traversal, shading, Russian roulette,
accumulation) against the oracle's binary32 restatement of pathtracing.wgsl.

Both sides evaluate the same arithmetic contract, so pixels are expected to be bit-equal;
a pixel differs only where one of its paths met a traversal near-tie and diverged.  Bar:
>= 99% of pixels bit-equal and relMSE (mean of (x-ref)^2/(ref^2+1e-2)) <= 1e-4.
"""
import numpy as np
import pytest

import nbounce_gb300 as nb
from nbounce_gb300 import scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu

EXACT_FRAC = 0.99
REL_MSE = 1e-4


def rel_mse(a, b):
    return float(np.mean((a[..., :3].astype(np.float64) - b[..., :3]) ** 2 / (b[..., :3].astype(np.float64) ** 2 + 1e-2)))


def gpu_render(desc, spp, dedup=True, env=None, dispatch_one_by_one=False, sobol=None):
    scene = nb.SceneBuffers.from_desc(desc, dedup=dedup)
    envmap = env or nb.EnvMap(desc.env_color, desc.env_texels)
    cam = nb.camera_struct(desc.world_to_clip, desc.clip_to_world)
    pt = nb.Pathtracer(desc.width, desc.height, nb.Globals(bounces=desc.bounces), sobol_table=sobol)
    if dispatch_one_by_one:
        for _ in range(spp):
            pt.dispatch(scene, cam, envmap)
    else:
        pt.render(scene, cam, envmap, spp)
    img = pt.download()
    rays, status = pt.last_stats()
    return img, rays, status, pt


@pytest.fixture(scope="module")
def spheres():
    desc = scenes.spheres_scene(width=64, height=64, spp=4, bounces=6)
    orc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    return desc, orc


def test_spheres_image_matches_oracle(spheres):
    desc, orc = spheres
    img, rays, status, _ = gpu_render(desc, desc.spp)
    assert status == 0
    ref, ref_rays, _, ovf = orc.render(desc.clip_to_world, desc.width, desc.height, nb.sobol_burley_table(), 1,
                                       desc.spp, bounces=desc.bounces, env=desc.env_color)
    assert not ovf
    exact = np.mean(np.all(img == ref, axis=-1))
    assert exact >= EXACT_FRAC, exact
    assert rel_mse(img, ref) <= REL_MSE
    # one traversal query per loop iteration on both sides (near-tie paths may differ)
    assert abs(rays - ref_rays) <= 0.001 * ref_rays


def test_dispatch_sequence_equals_batched_render(spheres):
    desc, _ = spheres
    a, ra, _, _ = gpu_render(desc, 3, dispatch_one_by_one=True)
    b, rb, _, pt = gpu_render(desc, 3)
    assert np.array_equal(a, b)
    assert pt.sample_count == 3 and abs(pt.globals.weight - 1.0 / 3.0) < 1e-7


def test_invalidate_restarts_accumulation(spheres):
    desc, _ = spheres
    first, _, _, _ = gpu_render(desc, 1)
    scene = nb.SceneBuffers.from_desc(desc)
    env = nb.EnvMap(desc.env_color)
    cam = nb.camera_struct(desc.world_to_clip, desc.clip_to_world)
    pt = nb.Pathtracer(desc.width, desc.height, nb.Globals(bounces=desc.bounces))
    pt.render(scene, cam, env, 2)
    pt.invalidate()
    assert pt.sample_count == 0
    pt.dispatch(scene, cam, env)  # weight 1: the old content is discarded (pathtracer.rs:234-235)
    assert np.array_equal(pt.download(), first)


def test_sample_budget_is_enforced(spheres):
    desc, _ = spheres
    table = nb.sobol_burley_table(3, 17)
    scene = nb.SceneBuffers.from_desc(desc)
    env = nb.EnvMap(desc.env_color)
    cam = nb.camera_struct(desc.world_to_clip, desc.clip_to_world)
    pt = nb.Pathtracer(desc.width, desc.height, nb.Globals(bounces=desc.bounces), sobol_table=table)
    assert pt.max_sample_count == 3
    pt.render(scene, cam, env, 5)
    assert pt.sample_count == 3
    with pytest.raises(nb.NbError) as e:
        pt.dispatch(scene, cam, env)
    assert e.value.status == 7


def test_equirect_environment_matches_oracle():
    desc = scenes.spheres_scene(width=48, height=48, spp=2, bounces=4)
    env_tex = scenes.sky_envmap(3, 256, 128)
    desc.env_texels = env_tex
    orc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    img, _, status, _ = gpu_render(desc, desc.spp)
    ref, _, _, _ = orc.render(desc.clip_to_world, desc.width, desc.height, nb.sobol_burley_table(), 1, desc.spp,
                              bounces=desc.bounces, env_texels=env_tex)
    assert status == 0
    assert np.mean(np.all(img == ref, axis=-1)) >= EXACT_FRAC
    assert rel_mse(img, ref) <= REL_MSE


def test_cube_environment_matches_oracle():
    """NB_ENV_CUBE (the reference's environment type): misses look the cube map up like the
    oracle - face by the major axis, bilinear inside the face."""
    desc = scenes.spheres_scene(width=48, height=48, spp=2, bounces=4)
    cube = scenes.cube_from_equirect(scenes.sky_envmap(3, 256, 128), 24)
    orc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    img, _, status, _ = gpu_render(desc, desc.spp, env=nb.EnvMap(cube=cube))
    ref, _, _, _ = orc.render(desc.clip_to_world, desc.width, desc.height, nb.sobol_burley_table(), 1, desc.spp,
                              bounces=desc.bounces, env_cube=cube)
    assert status == 0
    assert np.mean(np.all(img == ref, axis=-1)) >= EXACT_FRAC
    assert rel_mse(img, ref) <= REL_MSE
    plain_sky, _, _, _ = orc.render(desc.clip_to_world, desc.width, desc.height, nb.sobol_burley_table(), 1,
                                    desc.spp, bounces=desc.bounces, env=desc.env_color)
    assert not np.array_equal(plain_sky, ref)


def test_instanced_scene_crop_matches_oracle():
    desc = scenes.instanced_scene(n_instances=96, width=64, height=36, spp=2, bounces=8, env_size=(256, 128),
                                  scale=1 / 64)
    orc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    img, _, status, _ = gpu_render(desc, desc.spp)
    ref, _, _, _ = orc.render(desc.clip_to_world, desc.width, desc.height, nb.sobol_burley_table(), 1, desc.spp,
                              bounces=desc.bounces, env_texels=desc.env_texels)
    assert status == 0
    assert np.mean(np.all(img == ref, axis=-1)) >= EXACT_FRAC
    assert rel_mse(img, ref) <= REL_MSE


@pytest.mark.parametrize("size", [(37, 23), (5, 13), (64, 3), (8, 8)])
def test_image_sizes_off_the_8x8_tile_grid_match_oracle(size):
    """Rays are queued in 8x8 tiles with the columns and rows outside the last whole tile
    queued separately; every pixel of sizes off that grid (and narrower or lower than one
    tile) gets exactly its own samples."""
    w, h = size
    desc = scenes.spheres_scene(width=w, height=h, spp=3, bounces=4)
    orc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    img, _, status, _ = gpu_render(desc, desc.spp)
    ref, _, _, _ = orc.render(desc.clip_to_world, desc.width, desc.height, nb.sobol_burley_table(), 1, desc.spp,
                              bounces=desc.bounces, env=desc.env_color)
    assert status == 0
    assert (img[..., 3] == 1.0).all()
    assert np.mean(np.all(img == ref, axis=-1)) >= EXACT_FRAC
    assert rel_mse(img, ref) <= REL_MSE


@pytest.mark.parametrize("bounces", [0, 12])
def test_bounce_counts_outside_the_default_match_oracle(bounces):
    """bounces = 0 (primary hits only) and bounces = 12: past bounce 8 the per-bounce Sobol reads
    run beyond the fixed row stride of 17 into the next sample's row (pathtracing.wgsl:4,
    151-159; the reference GUI allows such counts, src/app.rs:132) - both sides reproduce it."""
    desc = scenes.spheres_scene(width=40, height=40, spp=3, bounces=bounces)
    orc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    img, _, status, _ = gpu_render(desc, desc.spp)
    ref, _, _, _ = orc.render(desc.clip_to_world, desc.width, desc.height, nb.sobol_burley_table(), 1, desc.spp,
                              bounces=desc.bounces, env=desc.env_color)
    assert status == 0
    assert np.mean(np.all(img == ref, axis=-1)) >= EXACT_FRAC
    assert rel_mse(img, ref) <= REL_MSE


def test_rr_from_bounce_3_matches_oracle():
    """The start-bounce Russian roulette variant (no roulette before bounce 3, the reference's
    schedule after) against the oracle running the same variant; it changes the image's noise
    but not what the image converges to."""
    desc = scenes.spheres_scene(width=40, height=40, spp=3, bounces=6)
    scene = nb.SceneBuffers.from_desc(desc)
    env = nb.EnvMap(desc.env_color)
    cam = nb.camera_struct(desc.world_to_clip, desc.clip_to_world)
    pt = nb.Pathtracer(desc.width, desc.height, nb.Globals(bounces=desc.bounces))
    pt.set_rr_start_bounce(3)
    pt.render(scene, cam, env, desc.spp)
    img = pt.download()
    assert pt.last_stats()[1] == 0
    orc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    ref, _, _, _ = orc.render(desc.clip_to_world, desc.width, desc.height, nb.sobol_burley_table(), 1, desc.spp,
                              bounces=desc.bounces, env=desc.env_color, rr_start=3)
    assert np.mean(np.all(img == ref, axis=-1)) >= EXACT_FRAC
    assert rel_mse(img, ref) <= REL_MSE
    plain, _, _, _ = gpu_render(desc, desc.spp)
    assert not np.array_equal(plain, img)


def test_benchmark_scene_full_frame_crop_matches_oracle():
    """Parity at the benchmark configuration's full size: the 4.9M-triangle, 1024-instance scene
    (terrain re-braided in the device TLAS) rendered at 1920x1080, 4 spp, 8 bounces; a centred
    96x64 crop of the GPU frame against the oracle rendering the same pixels."""
    desc = scenes.instanced_scene(width=1920, height=1080, spp=4)
    img, rays, status, _ = gpu_render(desc, desc.spp)
    assert status == 0 and np.isfinite(img).all() and (img[..., 3] == 1.0).all()
    orc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    w, h = 96, 64
    x0, y0 = (desc.width - w) // 2, (desc.height - h) // 2
    ref, _, _, _ = orc.render(desc.clip_to_world, desc.width, desc.height, nb.sobol_burley_table(), 1, desc.spp,
                              bounces=desc.bounces, env_texels=desc.env_texels, region=(x0, y0, w, h))
    crop = img[y0:y0 + h, x0:x0 + w]
    assert np.mean(np.all(crop == ref, axis=-1)) >= EXACT_FRAC
    assert rel_mse(crop, ref) <= REL_MSE


def test_sample_shards_merged_equal_one_render():
    """Sample sharding as the multi-GPU mode runs it (replicas.shard_samples /
    merge_running_means): three Pathtracers each render a contiguous range of Sobol rows,
    starting from sample counter start - 1; the merged running means equal one render of all
    rows up to float rounding."""
    from nbounce_gb300 import replicas
    desc = scenes.spheres_scene(width=48, height=40, spp=10, bounces=6)
    scene = nb.SceneBuffers.from_desc(desc)
    env = nb.EnvMap(desc.env_color)
    cam = nb.camera_struct(desc.world_to_clip, desc.clip_to_world)
    full = nb.Pathtracer(desc.width, desc.height, nb.Globals(bounces=desc.bounces))
    full.render(scene, cam, env, desc.spp)
    ref = full.download()
    means, lasts, counts = [], [], []
    for r in range(3):
        start, count = replicas.shard_samples(desc.spp, r, 3)
        pt = nb.Pathtracer(desc.width, desc.height, nb.Globals(bounces=desc.bounces))
        g = pt.globals
        g.sample = start - 1
        pt.globals = g
        pt.render(scene, cam, env, count)
        assert pt.last_stats()[1] == 0
        means.append(pt.download())
        lasts.append(start + count - 1)
        counts.append(count)
    merged = replicas.merge_running_means(means, lasts, counts)
    np.testing.assert_allclose(merged, ref, rtol=2e-5, atol=2e-6)
