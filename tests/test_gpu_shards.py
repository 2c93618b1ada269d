"""The sharded-frame exchange on the device (bench.py --shard-frame): each rank renders a
contiguous range of Sobol rows and one NCCL all-reduce merges the running means of CUDA
tensors.  With the one GPU of a test box it runs as a one-rank NCCL group: the merged tensor
stays on the GPU, a shard of all rows merges to that render, and two shards of one frame
merge to one render of all rows up to float rounding (the reference's mean is a chain of mix()
steps, pathtracing.wgsl:258).  bench.py --shard-frame then times its steps with the merge in
them."""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

import nbounce_gb300 as nb
from nbounce_gb300 import replicas, scenes

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class _View:
    def __init__(self, ptr, shape):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": "<f4", "data": (int(ptr), False),
                                         "version": 3}


def test_one_rank_nccl_merge_on_the_device():
    torch = pytest.importorskip("torch")
    import torch.distributed as dist
    dist.init_process_group("nccl", init_method=f"tcp://127.0.0.1:{_port()}", rank=0, world_size=1,
                            device_id=torch.device("cuda", 0))
    try:
        desc = scenes.spheres_scene(width=48, height=40, spp=10, bounces=6)
        scene = nb.SceneBuffers.from_desc(desc)
        env = nb.EnvMap(desc.env_color)
        cam = nb.camera_struct(desc.world_to_clip, desc.clip_to_world)
        full = nb.Pathtracer(48, 40, nb.Globals(bounces=6))
        full.render(scene, cam, env, 10)
        ref = full.download()
        merged = {}
        for start, count in ((1, 10), (1, 3), (4, 7)):
            pt = nb.Pathtracer(48, 40, nb.Globals(bounces=6))
            g = pt.globals
            g.sample = start - 1
            pt.globals = g
            pt.render(scene, cam, env, count)
            ptr, w, h = pt.output_texture()
            image = torch.as_tensor(_View(ptr, (h, w, 4)), device="cuda")
            m = replicas.merge_running_means_distributed(image, start + count - 1, count)
            assert m.is_cuda and m.dtype == torch.float32 and bool((m[..., 3] == 1.0).all())
            merged[(start, count)] = m.cpu().numpy()
        np.testing.assert_allclose(merged[(1, 10)], ref, rtol=1e-6, atol=1e-7)  # one shard of all rows
        # two shards of one frame, each merged as one rank; combined as a two-rank all-reduce would
        both = (merged[(1, 3)][..., :3] * 3 + merged[(4, 7)][..., :3] * 7) / 10
        np.testing.assert_allclose(both, ref[..., :3], rtol=2e-5, atol=2e-6)
    finally:
        dist.destroy_process_group()


def test_bench_shard_frame_times_the_device_merge():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--shard-frame", "--width", "320",
                          "--height", "180", "--spp", "8", "--steps", "2", "--warmup", "3", "--no-serving",
                          "--no-cache", "--no-cpu-baseline"], capture_output=True, text=True, timeout=600,
                         env={**os.environ, "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(_port())})
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads([x for x in out.stdout.splitlines() if x.startswith("{")][-1])
    assert line["config"]["parallelism"] == "sample shards x1" and line["scaling"] == "strong"
    assert line["value"] > 0 and line["n_gpus"] == 1
