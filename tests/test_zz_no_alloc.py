"""nb_render_static: the render entry point that allocates nothing.

It exists for callers that cannot allocate device memory while they render (an engine that
owns all GPU memory through its own allocator, or a loop whose footprint must stay fixed);
its wavefront scratch lives in one static device array sized for 262,144 paths per wave.
Two calls in a row through the C ABI must reproduce, bit for bit, what the existing entry
point (nb_pathtracer_render) accumulates for the same samples.  This file is collected last
so that a failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

import nbounce_gb300 as nb
from nbounce_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu


def test_static_render_matches_pathtracer_over_two_calls():
    torch = pytest.importorskip("torch")
    desc = scenes.spheres_scene(width=64, height=48, spp=4, bounces=6)
    scene = nb.SceneBuffers.from_desc(desc)
    env = nb.EnvMap(desc.env_color)
    cam = nb.camera_struct(desc.world_to_clip, desc.clip_to_world)
    out = torch.zeros((desc.height, desc.width, 4), dtype=torch.float32, device="cuda")
    pt = nb.Pathtracer(desc.width, desc.height, nb.Globals(bounces=desc.bounces))
    L = _lib.lib()
    for first, n in ((1, 2), (3, 2)):
        st = L.nb_render_static(scene.handle, env.handle, C.byref(cam), desc.width, desc.height, first, n,
                                desc.bounces, C.c_float(4.0), C.c_void_p(out.data_ptr()), None)
        assert st == 0, L.nb_last_error()
        pt.render(scene, cam, env, n)
        got = out.cpu().numpy()
        want = pt.download()
        assert np.array_equal(got, want), (first, n)


def test_static_render_rejects_images_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    desc = scenes.spheres_scene(width=16, height=16)
    scene = nb.SceneBuffers.from_desc(desc)
    env = nb.EnvMap(desc.env_color)
    cam = nb.camera_struct(desc.world_to_clip, desc.clip_to_world)
    out = torch.zeros((513, 512, 4), dtype=torch.float32, device="cuda")
    L = _lib.lib()
    st = L.nb_render_static(scene.handle, env.handle, C.byref(cam), 512, 513, 1, 1, 4, C.c_float(4.0),
                            C.c_void_p(out.data_ptr()), None)
    assert st == _lib.NB_ERR_INVALID_ARG
    assert b"static scratch" in L.nb_last_error()
