"""Host logic of bench.py that needs no GPU: the rank launcher behind --gpus N (two gloo ranks
started the way the benchmark starts its NCCL ranks), the workload description both arms
print, and the binary64 truth fixtures the relMSE figures are judged by."""
import json
import os
import sys
import textwrap

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from nbounce_gb300 import scenes  # noqa: E402


def test_launch_ranks_starts_n_ranks_and_rank0_prints(tmp_path, capfd):
    script = tmp_path / "ranks.py"
    script.write_text(textwrap.dedent("""
        import json, os, sys
        import torch, torch.distributed as dist
        dist.init_process_group("gloo")
        r, w = dist.get_rank(), dist.get_world_size()
        t = torch.tensor([float(r + 1)])
        dist.all_reduce(t)
        if r == 0:
            print(json.dumps({"world": w, "sum": float(t[0]), "argv": sys.argv[1:],
                              "master": os.environ["MASTER_ADDR"]}), flush=True)
        dist.destroy_process_group()
    """))
    rc = bench.launch_ranks(2, str(script), ["--steps", "1"])
    out = capfd.readouterr().out
    assert rc == 0
    line = json.loads([x for x in out.splitlines() if x.startswith("{")][-1])
    assert line == {"world": 2, "sum": 3.0, "argv": ["--steps", "1"], "master": "127.0.0.1"}


def test_both_arms_describe_the_same_workload():
    desc = scenes.spheres_scene(width=32, height=32)
    assert bench.workload_config(desc, 1) == bench.workload_config(desc, 1)
    assert bench.workload_config(desc, 2, shard=True)["parallelism"] == "sample shards x2"
    tiles = bench.cpu_sample_tiles(scenes.SceneDesc(None, None, [], [], width=1920, height=1080))
    assert len(tiles) == 24 and all(0 <= x and x + w <= 1920 and 0 <= y and y + h <= 1080 for x, y, w, h in tiles)


@pytest.mark.parametrize("name,tiles,size", [("spheres_256", 1, 256), ("instanced_1080p", 24, 32),
                                             ("instanced_cache", 24, 32)])
def test_truth_fixtures_are_binary64_16k_spp_of_this_generator(name, tiles, size):
    t = bench.load_truth(name)
    assert t is not None, name
    assert int(t["spp"]) == 16384 and int(t["precision"]) == 64
    assert t["rgb"].shape == (tiles, size, size, 3) and np.isfinite(t["rgb"]).all() and (t["rgb"] >= 0).all()
    assert int(t["fingerprint"][0]) > 0 and int(t["fingerprint"][1]) > 0
    if name == "spheres_256":
        desc = scenes.spheres_scene(width=256, height=256, spp=16, bounces=6)
        assert bench.truth_matches(desc, t)
        assert np.array_equal(np.asarray(t["clip_to_world"], np.float32), np.asarray(desc.clip_to_world, np.float32))
