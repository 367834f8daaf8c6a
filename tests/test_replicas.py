"""The multi-GPU mode of the render path: replicas (independent frames per
rank, the job's step time the slowest rank's).  Exercised with two gloo
ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    from owlexastitcher_gb300 import replicas
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, local = replicas.world_from_env()
        ms = 10.0 + 2.5 * r                      # rank 1 is the slower one
        slow = replicas.slowest_ms(ms, w)
        out.put((r, w, local, replicas.frame_id(r), slow, replicas.job_paths_per_s(w, 1000, slow)))
    finally:
        dist.destroy_process_group()


def test_replicas_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [x[0] for x in res] == [0, 1] and all(x[1] == 2 for x in res)
    assert len({x[3] for x in res}) == 2               # each rank its own frame / RNG streams
    assert all(x[4] == 12.5 for x in res)              # the job waits for the slowest rank
    assert all(x[5] == pytest.approx(2 * 1000 / 12.5e-3) for x in res)


def test_single_process_needs_no_group():
    from owlexastitcher_gb300 import replicas
    assert replicas.slowest_ms(7.0, 1) == 7.0
    assert replicas.job_paths_per_s(1, 100, 10.0) == pytest.approx(1e4)
