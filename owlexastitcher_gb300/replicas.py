"""Multi-GPU runs of the render path: replicas.

Pixels, paths and frames are independent and the volume is read-only, so N
GPUs of one node render N independent frames with the volume replicated on
each; rank r renders with its own RNG streams (exa_lp_ext.frameID = r).
Nothing is exchanged on the data path: a step's time is the slowest rank's
(one MAX reduction after the timed region) and the job's throughput counts
the paths of every rank.  One process per GPU, launched by torchrun; any
process group backend works (NCCL on GPUs, gloo on CPU).
"""
import os

import torch
import torch.distributed as dist


def world_from_env():
    """(world size, rank, local rank) from torchrun's environment"""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def frame_id(rank, base=0):
    """RNG stream selector of a rank's frame"""
    return base + rank


def slowest_ms(ms, world, device="cpu"):
    """the step time of the job: the maximum over ranks"""
    if world <= 1:
        return float(ms)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_paths_per_s(world, paths_per_step, ms):
    """whole-job throughput: every rank's paths over the slowest rank's time"""
    return world * paths_per_step / (ms / 1e3)
