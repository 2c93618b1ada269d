"""Host logic for running the pass on several ranks (one process per GPU).

Two modes:

* replicas (what bench.py --gpus N runs): every rank renders its own frame; throughput is
  the rays of all ranks over the slowest rank's time (``aggregate_replicas``); no collective.
* sample sharding (one frame over N ranks, bench.py --shard-frame): rank r sets its
  Pathtracer's sample counter to
  start - 1 and renders a contiguous range of Sobol rows (``shard_samples``).  Its running
  mean (mix with weight 1/k, pathtracing.wgsl:258) then holds sum(L) / last_row, so one
  exchange merges the ranks as sum_r(last_row_r * mean_r) / sum_r(count_r)
  (``merge_running_means``; ``merge_running_means_distributed`` is the one all-reduce, on the
  device for CUDA tensors).  The merge equals the single-rank running mean up to float
  rounding (not bit-exact: the reference's mean is a chain of mix() steps in sample order).
"""
import numpy as np


def shard_samples(spp, rank, world, first_sample=1):
    """Contiguous 1-based Sobol rows [start, start + count) for `rank` of `world`."""
    base, extra = divmod(spp, world)
    count = base + (1 if rank < extra else 0)
    start = first_sample + rank * base + min(rank, extra)
    return start, count


def merge_running_means(means, last_rows, counts):
    """Merge per-rank running means; rank r's mean covers `counts[r]` rows ending at
    `last_rows[r]` and started from zero (numpy, float64 accumulation)."""
    total = float(sum(counts))
    acc = np.zeros_like(np.asarray(means[0], np.float64))
    for m, last in zip(means, last_rows):
        acc += np.asarray(m, np.float64) * (last / total)
    out = acc.astype(np.float32)
    out[..., 3] = 1.0
    return out


def merge_running_means_distributed(mean, last_row, count, group=None):
    """The exchange step across ranks: all-reduce of last_row * mean and of count.

    `mean` is a numpy array (reduced on the host: gloo) or a torch tensor, which is reduced
    where it lives (a CUDA tensor stays on its GPU: NCCL) and returned as a float32 tensor
    there; the numpy form returns numpy."""
    import torch
    import torch.distributed as dist

    if isinstance(mean, torch.Tensor):
        t = mean.to(torch.float64) * float(last_row)
        n = torch.tensor([float(count)], dtype=torch.float64, device=mean.device)
        dist.all_reduce(t, group=group)
        dist.all_reduce(n, group=group)
        out = (t / n).to(torch.float32)
        out[..., 3] = 1.0
        return out
    t = torch.as_tensor(np.asarray(mean, np.float64) * last_row)
    n = torch.tensor([float(count)], dtype=torch.float64)
    dist.all_reduce(t, group=group)
    dist.all_reduce(n, group=group)
    out = (t / n).numpy().astype(np.float32)
    out[..., 3] = 1.0
    return out


def aggregate_replicas(local_ms, local_rays, group=None):
    """(total rays of all ranks, max time over ranks in ms) for replica throughput."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized():
        return float(local_rays), float(local_ms)
    v = torch.tensor([float(local_ms)], dtype=torch.float64)
    r = torch.tensor([float(local_rays)], dtype=torch.float64)
    dist.all_reduce(v, op=dist.ReduceOp.MAX, group=group)
    dist.all_reduce(r, group=group)
    return float(r.item()), float(v.item())
