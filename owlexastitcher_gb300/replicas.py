"""Multi-GPU runs of the render path.

Pixels, paths and frames are independent and the volume is read-only, so
the volume is replicated on every GPU and nothing is exchanged while
rendering.  Two splits:
  replicas -- N GPUs render N independent frames; rank r renders with its
              own RNG streams (exa_lp_ext.frameID = r).  A step's time is the
              slowest rank's (one MAX reduction after the timed region) and
              the job's throughput counts the paths of every rank.
  bands    -- N GPUs render one frame, rank r the band of rows band_rows()
              gives it (exa_lp_ext.rowBegin / rowEnd: every pixel exactly as
              in the whole frame); gather_rows() assembles the frame on rank
              0 from the ranks' host copies of their rows.
One process per GPU, launched by torchrun; any process group backend works
(NCCL on GPUs, gloo on CPU).
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


def band_rows(rank, world, height):
    """rows [begin, end) of a height-row frame for rank `rank` of `world`:
    whole 8-row tile rows, split as evenly as they go"""
    tiles = (height + 7) // 8
    b = 8 * (rank * tiles // world)
    e = min(height, 8 * ((rank + 1) * tiles // world))
    return b, e


def gather_rows(rows, rank, world, height, width):
    """rank 0: the frame assembled from every rank's rows (a numpy array of
    (end - begin) * width records, its band_rows); other ranks: None"""
    import numpy as np
    if world <= 1:
        return rows
    parts = [None] * world if rank == 0 else None
    dist.gather_object(np.ascontiguousarray(rows), parts, dst=0)
    if rank != 0:
        return None
    out = np.empty((height * width,) + parts[0].shape[1:], parts[0].dtype)
    for r, p in enumerate(parts):
        b, e = band_rows(r, world, height)
        assert len(p) == (e - b) * width, "a rank's rows do not match its band"
        out[b * width:e * width] = p
    return out
