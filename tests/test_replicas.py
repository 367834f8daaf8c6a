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


def test_band_rows_cover_the_frame():
    from owlexastitcher_gb300 import replicas
    for h in (1, 7, 8, 9, 100, 1024, 1080):
        for world in (1, 2, 3, 4, 8):
            bands = [replicas.band_rows(r, world, h) for r in range(world)]
            assert bands[0][0] == 0 and bands[-1][1] == h
            assert all(b[0] % 8 == 0 for b in bands)
            assert all(bands[i][1] == bands[i + 1][0] for i in range(world - 1))
            assert all(b[1] == h or b[1] % 8 == 0 for b in bands)


def _band_rank(rank, world, port, out):
    """renders this rank's band of a small frame with the oracle and gathers
    the frame on rank 0"""
    import sys
    import numpy as np
    import torch.distributed as dist
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    sys.path.insert(0, os.path.join(os.path.dirname(here), "oracle"))
    import pyoracle
    from conftest import dataset
    from helpers import OracleScene, host_lp, oracle_only_lp, ramp_tf
    from owlexastitcher_gb300 import replicas
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ds = dataset("tiny")
        f = pyoracle.Field(ds.vertices, ds.indices, ds.gridlets, ds.gridlet_scalars)
        lo, hi, vr = f.bounds()
        tf = ramp_tf()
        xf = (np.float32(vr[0]), np.float32(vr[1]))
        o = OracleScene(pyoracle, ds, (8, 8, 8), lo, hi, tf, xf)
        w, h = 24, 20
        lp = oracle_only_lp(lo, hi, (8, 8, 8), tf, xf, w, h, 0, 2)
        hl, hfb, hacc, _, _ = host_lp(lp, o, w, h)
        b, e = replicas.band_rows(rank, world, h)
        assert o.f.render(bytes(hl), w, h, b * w, e * w) == 0
        frame = replicas.gather_rows(hacc[b * w:e * w], rank, world, h, w)
        if rank == 0:
            full = np.zeros_like(hacc)
            hl2, _, full, _, _ = host_lp(lp, o, w, h)
            assert o.f.render(bytes(hl2), w, h) == 0
            out.put(frame.tobytes() == full.tobytes() and len(np.unique(full)) > 4)
    finally:
        dist.destroy_process_group()


def test_bands_two_gloo_ranks_equal_one_frame():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_band_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    ok = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert ok
