"""nb_render_static: the render entry point that allocates nothing.

It exists for callers that cannot allocate device memory while they render (an engine that
owns all GPU memory through its own allocator, or a loop whose footprint must stay fixed);
its wavefront scratch lives in one static device array sized for 262,144 paths per wave.
Two calls in a row through the C ABI must reproduce, bit for bit, what the existing entry
point (nb_pathtracer_render) accumulates for the same samples, both when one wave holds all
of a call's samples and when the samples are split over several waves; a warm call must leave
the device's free memory unchanged.  This file is collected last so that a failure here
leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

import nbounce_gb300 as nb
from nbounce_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu


def _static(L, scene, env, cam, w, h, first, n, bounces, out):
    return L.nb_render_static(scene.handle, env.handle, C.byref(cam), w, h, first, n, bounces, C.c_float(4.0),
                              C.c_void_p(out.data_ptr()), None)


@pytest.mark.parametrize("width,height,calls", [
    (64, 48, ((1, 2), (3, 2))),          # 3,072 pixels: one wave holds every sample of a call
    (512, 300, ((1, 1), (2, 3))),        # 153,600 pixels: one sample per wave, three waves
])
def test_static_render_matches_pathtracer_over_two_calls(width, height, calls):
    torch = pytest.importorskip("torch")
    desc = scenes.spheres_scene(width=width, height=height, spp=4, bounces=6)
    scene = nb.SceneBuffers.from_desc(desc)
    env = nb.EnvMap(desc.env_color)
    cam = nb.camera_struct(desc.world_to_clip, desc.clip_to_world)
    out = torch.zeros((desc.height, desc.width, 4), dtype=torch.float32, device="cuda")
    pt = nb.Pathtracer(desc.width, desc.height, nb.Globals(bounces=desc.bounces))
    L = _lib.lib()
    for first, n in calls:
        st = _static(L, scene, env, cam, desc.width, desc.height, first, n, desc.bounces, out)
        assert st == 0, L.nb_last_error()
        pt.render(scene, cam, env, n)
        got = out.cpu().numpy()
        want = pt.download()
        assert np.array_equal(got, want), (first, n)


def test_static_render_allocates_no_device_memory():
    torch = pytest.importorskip("torch")
    desc = scenes.spheres_scene(width=96, height=64, spp=2, bounces=6)
    scene = nb.SceneBuffers.from_desc(desc)
    env = nb.EnvMap(desc.env_color)
    cam = nb.camera_struct(desc.world_to_clip, desc.clip_to_world)
    out = torch.zeros((desc.height, desc.width, 4), dtype=torch.float32, device="cuda")
    L = _lib.lib()
    assert _static(L, scene, env, cam, desc.width, desc.height, 1, 2, desc.bounces, out) == 0, L.nb_last_error()
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for first in (3, 5):
        assert _static(L, scene, env, cam, desc.width, desc.height, first, 2, desc.bounces, out) == 0, \
            L.nb_last_error()
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before


def test_static_render_rejects_images_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    desc = scenes.spheres_scene(width=16, height=16)
    scene = nb.SceneBuffers.from_desc(desc)
    env = nb.EnvMap(desc.env_color)
    cam = nb.camera_struct(desc.world_to_clip, desc.clip_to_world)
    out = torch.zeros((513, 512, 4), dtype=torch.float32, device="cuda")
    L = _lib.lib()
    st = _static(L, scene, env, cam, 512, 513, 1, 1, 4, out)
    assert st == _lib.NB_ERR_INVALID_ARG
    assert b"static scratch" in L.nb_last_error()
