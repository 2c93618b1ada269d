"""Multi-rank host logic on CPU with the gloo backend (world size 2).

Sample sharding: each rank renders its Sobol row range with the oracle, the ranks merge
their running means in one all-reduce, and the merged image matches the single-process
running mean of all rows.  Replica aggregation: total rays over the max time across ranks.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from nbounce_gb300 import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_shard_samples_partitions_rows():
    for spp in (1, 7, 64):
        for world in (1, 2, 3, 8):
            rows = []
            for r in range(world):
                s, c = replicas.shard_samples(spp, r, world)
                rows += list(range(s, s + c))
            assert rows == list(range(1, spp + 1))


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist

    from nbounce_gb300 import scenes
    from oracle import oracle as O

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    desc = scenes.spheres_scene(width=16, height=16)
    osc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    sob = O.sobol_table(1024, 17)
    start, count = replicas.shard_samples(8, rank, world)
    img, rays, _, _ = osc.render(desc.clip_to_world, 16, 16, sob, start, count, bounces=6, env=desc.env_color,
                                 threads=1)
    # a running mean over rows start..start+count-1 that starts from its own first sample
    merged = replicas.merge_running_means_distributed(img, start + count - 1, count)
    total_rays, t_max = replicas.aggregate_replicas(10.0 + rank, rays)
    if rank == 0:
        np.save(os.path.join(out_dir, "merged.npy"), merged)
        np.save(os.path.join(out_dir, "agg.npy"), np.array([total_rays, t_max]))
    dist.destroy_process_group()


def test_two_rank_sample_sharding_matches_single_process(tmp_path):
    from nbounce_gb300 import scenes
    from oracle import oracle as O

    mp.start_processes(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    merged = np.load(tmp_path / "merged.npy")
    desc = scenes.spheres_scene(width=16, height=16)
    osc = O.OracleScene(desc.vertices, desc.indices, desc.primitives(), dedup=True)
    full, rays, _, _ = osc.render(desc.clip_to_world, 16, 16, O.sobol_table(1024, 17), 1, 8, bounces=6,
                                  env=desc.env_color, threads=1)
    np.testing.assert_allclose(merged, full, rtol=1e-5, atol=1e-6)
    total_rays, t_max = np.load(tmp_path / "agg.npy")
    assert total_rays == rays and t_max == 11.0


def test_merge_running_means_numpy():
    a = np.random.default_rng(0).random((4, 4, 4)).astype(np.float32)
    b = np.random.default_rng(1).random((4, 4, 4)).astype(np.float32)
    # a covers rows 1..3 (mean = sum/3), b covers row 4 alone (mean = L4/4)
    m = replicas.merge_running_means([a, b], [3, 4], [3, 1])
    np.testing.assert_allclose(m[..., :3], (3 * a[..., :3] + 4 * b[..., :3]) / 4, rtol=1e-6)
    assert np.all(m[..., 3] == 1.0)
