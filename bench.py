"""Benchmark: multi-scatter Woodcock path tracing of the medium AMR dataset
(4 levels, 128^3 root cells, ~51M cells, 256 Gaussians + noise) at
1024x1024, 16 spp, <= 8 bounces, albedo 0.8, HG g = 0.3, one directional
light, 128^3 majorant grid -- through the ExaStitch CUDA path.

A step renders one 1024x1024x16 frame (16.8M camera paths).  Prints one
JSON line (rank 0).  `--impl reference` times the CPU oracle's restatement
of the same integrator on the host cores instead (a bounded pixel sample per
step).  Multi-GPU runs (torchrun) render independent frames per rank
(replicas: no data-path collective), scaling = weak.

Beside the headline, the line carries: the walk kernel's roofline, field
sample rates, the end-to-end rate through the C ABI, the CPU baseline, SM
clocks, the majorant build of the workload's field (`majorant_build`: the
gridlet kernel's CUDA-event time and roofline), the learned field, the
batched frames and the small configuration (with its host timings).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "paths/s"
WIDTH, HEIGHT, SPP = 1024, 1024, 16
NUM_MCS = (128, 128, 128)
L2_BYTES = 129 * 1024 * 1024
DESCR = {"medium": "4 levels, 128^3 root, 256 Gaussians + noise",
         "cloud": "5 levels, 256^3 root, exp(3 fBm) cloud with 70% of root cells empty"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="medium", choices=["medium", "small", "tiny", "cloud"],
                    help="cloud: the large sparse cloud field (5 levels, 256^3 roots, ~394M cells) rendered at "
                         "1920x1080, 64 spp, <= 16 bounces, with the learned field (2^21 entries per level)")
    ap.add_argument("--width", type=int, default=None)
    ap.add_argument("--height", type=int, default=None)
    ap.add_argument("--spp", type=int, default=None)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-only", action="store_true", help="warm-up + 1 step, no extras (for ncu)")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-field (surrogate) measurements")
    ap.add_argument("--learned-steps", type=int, default=1600, help="surrogate training steps")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-frames measurements")
    ap.add_argument("--majorant-only", action="store_true",
                    help="only the majorant build on the workload's field (one untimed and 3 timed builds); prints "
                         "the majorant_build object (for ncu captures of the build kernels)")
    ap.add_argument("--split", default="replicas", choices=["replicas", "bands"],
                    help="multi-GPU: replicas (a frame per rank, weak scaling) or bands (one frame, a band of rows "
                         "per rank, gathered on rank 0; strong scaling)")
    a = ap.parse_args()
    big = a.config == "cloud"
    a.width = a.width or (1920 if big else WIDTH)
    a.height = a.height or (1080 if big else HEIGHT)
    a.spp = a.spp or (64 if big else SPP)
    a.bounces = 16 if big else 8
    if a.majorant_only:
        a.no_cpu_baseline = True
    if big:
        # the oracle's field for ~400M cells is too large for a bounded CPU
        # sample; the batched workload is defined on the small field
        a.no_cpu_baseline = True
        a.no_batched = True
    return a


def workload_config(a):
    return {
        "workload": f"{a.config} AMR ({DESCR.get(a.config, a.config)}), "
                    f"path tracing {a.width}x{a.height} {a.spp} spp",
        "dataset": a.config,
        "width": a.width, "height": a.height, "spp": a.spp,
        "max_bounces": a.bounces, "albedo": 0.8, "hg_g": 0.3, "light": "directional",
        "majorant_grid": list(NUM_MCS), "tf": "64-entry linear RGBA ramp",
        "l2": "flushed between timed steps (256 MiB write)",
    }


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic():
    p = os.path.join(ROOT, "profiles", "render_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def clocks_rejected(c, low=0.85):
    """whether a timed region's clock record fails the timing rules: a
    hardware or thermal slowdown, or SM clocks well below their maximum with
    no reason given (a clock lock left by another process); a power cap
    alone is kept"""
    if {"hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"} & set(c.get("reasons") or []):
        return True
    sm, mx = c.get("sm_mhz"), c.get("sm_max_mhz")
    return bool(sm and mx and sm < low * mx and not c.get("reasons"))


def make_scene(a, device):
    """The workload's dataset, made by the GPU generator; returns it and the
    generator record (wall seconds, per-stage seconds; the CPU generator's
    wall time beside it unless the CPU baselines are off)."""
    from owlexastitcher_gb300 import datagen
    t0 = time.time()
    ds = datagen.Dataset(a.config, device=device)
    gen = {"gpu_seconds": time.time() - t0, "gpu_stage_seconds": ds.stats["stageSeconds"], "cpu_seconds": None}
    if not a.no_cpu_baseline and not a.profile_only:
        t0 = time.time()
        cpu = datagen.Dataset(a.config)
        gen["cpu_seconds"] = time.time() - t0
        gen["cpu_stage_seconds"] = cpu.stats["stageSeconds"]
        gen["identical"] = all(getattr(cpu, k).tobytes() == getattr(ds, k).tobytes() for k in (
            "vertices", "indices", "gridlets", "gridlet_scalars", "amr_cells", "amr_scalars"))
        del cpu
    return ds, gen


def run_ours(a):
    import torch
    import torch.distributed as dist
    from helpers import orbit_camera, ramp_tf, setup_render
    from owlexastitcher_gb300 import exastitch as E

    from owlexastitcher_gb300 import replicas
    world, rank, local = replicas.world_from_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            dist.barrier()

    ds, gen = make_scene(a, local)
    if a.majorant_only:
        peak, peak_kind = load_peaks()
        print(json.dumps(majorant_build(ds, local, NUM_MCS, peak, peak_kind)))
        return
    ctx = E.Context(local)
    r = E.Renderer(ctx, E.ExaStitchModel.from_dataset(ctx, ds), NUM_MCS)
    lo, hi = r.model.cellBounds
    r.setColorMap(ramp_tf())
    r.resize(a.width, a.height)
    r.spp = a.spp
    cam = orbit_camera(lo, hi, a.width, a.height)
    setup_render(r.lp, cam, a.width, a.height, E.PATH_TRACING_INTEGRATOR, a.spp, "directional", True)
    r.lp.ext.maxBounces = a.bounces
    bands = a.split == "bands" and world > 1
    if bands:
        # one frame: this rank's band of rows
        r.lp.ext.rowBegin, r.lp.ext.rowEnd = replicas.band_rows(rank, world, a.height)
        band = (r.lp.ext.rowBegin, r.lp.ext.rowEnd)
    else:
        r.lp.ext.frameID = replicas.frame_id(rank)  # independent frames per rank
    paths_per_step = a.width * a.height * a.spp
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step():
        r.accumID = 0
        r.render()

    # warm-up
    for _ in range(a.warmup):
        step()
    torch.cuda.synchronize()
    ctx.sync()
    if a.profile_only:
        step()
        torch.cuda.synchronize()
        return

    def timed_steps():
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
        with ClockSampler(local) as clk:
            barrier()
            torch.cuda.synchronize()
            for i in range(a.steps):
                flush.fill_(float(i))
                starts[i].record(stream)
                step()
                ends[i].record(stream)
            torch.cuda.synchronize()
            barrier()
        ctx.sync()
        return [s.elapsed_time(e) for s, e in zip(starts, ends)], clk.summary()

    step_ms, clocks = timed_steps()
    # a timed region whose clocks any rank rejects is timed once more, and
    # the second record is reported
    remeasured = replicas.slowest_ms(float(clocks_rejected(clocks)), world, device="cuda") > 0
    if remeasured:
        step_ms, clocks = timed_steps()
    clocks["remeasured"] = remeasured
    render_stats = ctx.render_stats()
    # the last timed frame (accumID 0: the accumulation buffer holds its
    # per-pixel sums) for the CPU leg's bit-for-bit comparison
    timed_frame = (r.accum.cpu().numpy().reshape(-1, 4).copy(), r.fb.cpu().numpy().view(np.uint32).copy())
    ms = replicas.slowest_ms(sum(step_ms) / len(step_ms), world, device="cuda")
    # bands: the ranks share one frame's paths; replicas: every rank a frame
    value = replicas.job_paths_per_s(1 if bands else world, paths_per_step, ms)

    # counting launch (same frame): algorithmic work of one launch
    cnt = torch.zeros(16, dtype=torch.int64, device="cuda")
    r.lp.ext.stepCounters = cnt.data_ptr()
    step()
    torch.cuda.synchronize()
    r.lp.ext.stepCounters = None
    c = cnt.cpu().numpy()
    field_samples, g_samples, e_samples, dda_cells, paths = (int(x) for x in c[:5])
    work = dict(zip(["cache_misses", "table_queries", "gridlet_tests", "element_list_walks", "walks"],
                    (int(x) for x in c[5:10])))
    counts = np.count_nonzero(ds.indices >= 0, axis=1) if len(ds.indices) else np.array([8])
    avg_nv = float(counts.mean())
    alg_bytes = g_samples * 64 + e_samples * (32 + 16 * avg_nv) + dda_cells * 4
    peak, peak_kind = load_peaks()
    # dominant kernel: the wavefront walk kernel (all field samples and DDA
    # cells happen there); its time summed over the frame's launches
    walk_ms = render_stats["walkMs"] if render_stats["wavefront"] else ms
    achieved = alg_bytes / (walk_ms / 1e3) / 1e9
    tr = load_traffic()
    traffic = None
    if tr and tr.get("dataset") == a.config:
        traffic = tr["dram_bytes_per_launch"] * (paths_per_step / tr["paths_per_launch"])

    # end-to-end through the public API: render + read the RGBA8 frame back
    host_fb = torch.empty(a.width * a.height, dtype=torch.int32, pin_memory=True)
    e2e_t = []
    for i in range(max(3, a.steps)):
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step()
        host_fb.copy_(r.fb, non_blocking=True)
        torch.cuda.synchronize()
        if bands:  # rank 0 assembles the frame from the ranks' rows
            replicas.gather_rows(host_fb.numpy()[band[0] * a.width:band[1] * a.width], rank, world, a.height,
                                 a.width)
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = replicas.slowest_ms(statistics.median(e2e_t) * 1e3, world, device="cuda") / 1e3
    lp_bytes = E.C.sizeof(E.LaunchParams)

    # field point queries (1M uniform points in cellBounds), device and e2e
    rng = np.random.default_rng(42)
    P = rng.uniform(lo, hi, (1 << 20, 3)).astype(np.float32)
    pd = torch.from_numpy(P).cuda()
    out = torch.empty((1 << 20) * 3, dtype=torch.int32, device="cuda")
    for _ in range(3):
        r.sampler.sample_device(pd.data_ptr(), out.data_ptr(), len(P), cull=False)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    flush.fill_(1.0)
    ev0.record(stream)
    for _ in range(10):
        r.sampler.sample_device(pd.data_ptr(), out.data_ptr(), len(P), cull=False)
    ev1.record(stream)
    torch.cuda.synchronize()
    q_dev = 10 * len(P) / (ev0.elapsed_time(ev1) / 1e3)
    t0 = time.perf_counter()
    for _ in range(5):
        r.sampler.sample_host(P, cull=False)
    q_e2e = 5 * len(P) / (time.perf_counter() - t0)
    ctx.sync()

    majorants = None
    if rank == 0 and not a.profile_only:
        majorants = majorant_build(ds, local, NUM_MCS, peak, peak_kind)

    cpu = parity = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        cpu, parity = cpu_baseline(a, ds, r, a.cpu_seconds, timed_frame)

    small = None
    if rank == 0 and world == 1 and a.config != "cloud":
        small = run_small_config(a, local, flush, cpu=not a.no_cpu_baseline)

    batched = None
    if rank == 0 and not a.no_batched:
        batched = run_batched(a, local, flush)

    learned = None
    if rank == 0 and not a.no_learned:
        from owlexastitcher_gb300 import datagen
        if a.config == "cloud":
            # the large cloud: 2^21 table entries per level
            learned = {"workload_field": run_learned(a, local, ds, NUM_MCS, flush, log2T=21)}
        else:
            learned = {
                # the small config's field (3 levels, 32^3 root) with its 32^3 majorant grid
                "small_field": run_learned(a, local, datagen.Dataset("small"), (32, 32, 32), flush),
                # the same method on this workload's field and majorant grid
                "workload_field": run_learned(a, local, ds, NUM_MCS, flush),
            }

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "strong" if bands else "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded AMR Gaussians + value noise)",
            "config": workload_config(a) | {"multi_gpu": "bands: one frame, a band of rows per rank, gathered on "
                                                          "rank 0" if bands else "replicas: a frame per rank"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": "k_wf_walk (summed over the frame's launches)" if render_stats["wavefront"] else
                         "k_render_sample<PATH_TRACING>",
                         "kernel_ms_per_step": walk_ms,
                         "algorithmic_bytes_per_launch": alg_bytes},
            "field_samples": {"render_per_s": field_samples / (ms / 1e3), "per_step": field_samples,
                              "gridlet_per_step": g_samples, "element_per_step": e_samples,
                              "dda_cells_per_step": dda_cells,
                              "point_query_per_s": q_dev, "point_query_e2e_per_s": q_e2e,
                              "point_query_n": len(P), "work_per_step": work},
            "e2e": {"value": (1 if bands else world) * paths_per_step / e2e_s, "unit": "paths/s",
                    "h2d_bytes_per_step": lp_bytes, "d2h_bytes_per_step": a.width * a.height * 4},
            "cpu_baseline": cpu,
            "parity": parity,
            "clocks": clocks,
            # the library's count of its kernel launches per frame (camera, walk, events and
            # round-end kernels of each round, the resolve)
            "gpu_launches": a.steps * render_stats["kernelLaunches"],
            "render": render_stats,
            "majorant_build": majorants,
            "learned_field": learned,
            "batched_frames": batched,
            "small_config": small,
            "dataset": {k: ds.stats[k] for k in ("numAmrCells", "numGridlets", "numGridletScalars", "numPyramids",
                                                  "numWedges", "numHexes", "numTets")} | {
                "field_bytes": ds.field_bytes, "generator": gen},
            "step_ms": step_ms,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def majorant_build(ds, local, num_mcs, peak, peak_kind, reps=3):
    """Grid::build on the workload's field and majorant grid: the GPU times
    of the gridlet and element value-range kernels from the build's own CUDA
    events (median of `reps` builds after one untimed build; each build
    uploads the field first, so the scalars are not L2-resident), with the
    gridlet kernel's roofline.  Algorithmic bytes of that kernel: 4 B per
    corner scalar and 32 B per gridlet header read, 8 B per gridlet range
    and 8 B per macrocell range written."""
    from owlexastitcher_gb300 import exastitch as E
    ctx = E.Context(local)
    model = E.ExaStitchModel.from_dataset(ctx, ds)
    model.setNumGridCells(num_mcs)
    sampler = E.ExaStitchSampler(ctx)
    stats = []
    for _ in range(reps + 1):
        sampler.build(model)
        stats.append(ctx.build_stats())
    ctx.close()
    stats = stats[1:]
    g_ms = statistics.median(s["gridletMajorantMs"] for s in stats)
    n_mc = int(np.prod(num_mcs))
    alg = 4 * int(ds.stats["numGridletScalars"]) + 40 * int(ds.stats["numGridlets"]) + 8 * n_mc
    achieved = alg / (g_ms / 1e3) / 1e9
    return {"kernel": "k_gridlet_majorants_sep, then k_gridlet_majorants over the gridlets it leaves",
            "majorant_grid": list(num_mcs), "gpu_ms": g_ms,
            "elem_kernel_ms": statistics.median(s["elemMajorantMs"] for s in stats),
            "build_total_ms": statistics.median(s["totalMs"] for s in stats), "blocks": stats[0]["majorantBlocks"],
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind, "algorithmic_bytes_per_launch": alg}}


def run_learned(a, local, ds, num_mcs, flush, timed=3, log2T=19):
    """The learned field on one dataset: training, per-macrocell error
    bounds, memory, and the same path-traced frame rendered with the exact
    sampler and with the learned field (+ exact fallback), both through
    the public API, timed with CUDA events on the current stream."""
    import torch
    from helpers import orbit_camera, ramp_tf, setup_render
    from owlexastitcher_gb300 import exastitch as E
    ctx = E.Context(local)
    r = E.Renderer(ctx, E.ExaStitchModel.from_dataset(ctx, ds), num_mcs)
    lo, hi = r.model.cellBounds
    r.setColorMap(ramp_tf())
    r.resize(a.width, a.height)
    r.spp = a.spp
    setup_render(r.lp, orbit_camera(lo, hi, a.width, a.height), a.width, a.height, E.PATH_TRACING_INTEGRATOR,
                 a.spp, "directional", True)
    r.lp.ext.maxBounces = a.bounces
    stream = torch.cuda.current_stream()
    t0 = time.perf_counter()
    S = E.Surrogate(ctx, log2TableSize=log2T, baseResolution=16, growth=1.5, numSamples=1 << 24, batch=1 << 18,
                    importanceFraction=0.5, seed=1234)
    torch.cuda.synchronize()
    sample_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    loss = S.train(a.learned_steps)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    S.evaluate(0.02, 1 << 24)
    eval_s = time.perf_counter() - t0
    st = S.stats()
    res = {}
    imgs = {}
    for name, learned in (("exact", False), ("learned", True)):
        r.learned = learned
        for _ in range(2):
            r.accumID = 0
            r.render()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(timed)]
        for e0, e1 in ev:
            flush.fill_(2.0)
            r.accumID = 0
            e0.record(stream)
            r.render()
            e1.record(stream)
        torch.cuda.synchronize()
        ctx.sync()
        ms = sum(e0.elapsed_time(e1) for e0, e1 in ev) / timed
        imgs[name] = r.accum.cpu().numpy().reshape(-1, 4)[:, :3] / a.spp
        cnt = torch.zeros(16, dtype=torch.int64, device="cuda")
        r.lp.ext.stepCounters = cnt.data_ptr()
        r.accumID = 0
        r.render()
        torch.cuda.synchronize()
        r.lp.ext.stepCounters = None
        c = cnt.cpu().numpy()
        res[name] = {"paths_per_s": a.width * a.height * a.spp / (ms / 1e3), "ms_per_frame": ms,
                     "walk_ms": ctx.render_stats()["walkMs"],
                     "exact_field_samples": int(c[0]), "learned_samples": int(c[10]),
                     "majorant_violations": int(c[11])}
    r.learned = False
    conv = converged_rmse(a, r, lo, hi, S)
    # point queries: learned value vs exact sample at 1M uniform points
    rng = np.random.default_rng(42)
    P = rng.uniform(lo, hi, (1 << 20, 3)).astype(np.float32)
    pd = torch.from_numpy(P).cuda()
    vals = torch.empty(1 << 20, dtype=torch.float32, device="cuda")
    ex = torch.empty((1 << 20) * 3, dtype=torch.int32, device="cuda")
    q = {}
    for name, fn in (("exact", lambda: r.sampler.sample_device(pd.data_ptr(), ex.data_ptr(), len(P), cull=False)),
                     ("learned", lambda: S.sample_device(pd.data_ptr(), vals.data_ptr(), len(P)))):
        for _ in range(3):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush.fill_(3.0)
        e0.record(stream)
        for _ in range(10):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        q[name] = 10 * len(P) / (e0.elapsed_time(e1) / 1e3)
    ctx.sync()
    rmse = float(np.sqrt(np.mean((imgs["exact"] - imgs["learned"]) ** 2)))
    out = {
        "dataset": ds.config if hasattr(ds, "config") else None, "majorant_grid": list(num_mcs),
        "encoding": {"levels": 16, "features": 2, "table_entries_per_level": 1 << log2T, "base_resolution": 16,
                     "growth": 1.5},
        "mlp": "32-64-64-1 ReLU, BF16 weights, FP32 accumulate; training: tcgen05.mma (M = 128, accumulators in "
               "tensor memory); inference inside the walk: mma.sync m16n8k16",
        "training": {"pairs": 1 << 24, "importance_fraction": 0.5, "batch": 1 << 18, "steps": a.learned_steps,
                     "final_batch_mse": loss, "sample_seconds": sample_s, "train_seconds": train_s,
                     "pairs_per_s": a.learned_steps * (1 << 18) / train_s},
        "errors": {"tolerance": 0.02, "probe_points": st["probePoints"], "probe_rmse": st["rmse"],
                   "probe_max_error": st["maxError"], "eval_seconds": eval_s},
        "macrocells": {"total": st["numMacrocells"], "learned": st["numSurrogateMacrocells"],
                       "fraction_learned": st["numSurrogateMacrocells"] / max(st["numMacrocells"], 1)},
        "memory_bytes": {"learned_inference": st["inferenceBytes"], "exact_field": st["fieldBytes"],
                         "exact_fallback_needed": st["fallbackFieldBytes"],
                         "learned_plus_fallback_over_exact": (st["inferenceBytes"] + st["fallbackFieldBytes"]) /
                         max(st["fieldBytes"], 1)},
        "render": res,
        "paths_per_s_learned_over_exact": res["learned"]["paths_per_s"] / res["exact"]["paths_per_s"],
        "image_rmse_vs_exact_same_rng": rmse,
        "converged": conv,
        "point_queries_per_s": q,
    }
    ctx.close()
    return out


def converged_rmse(a, r, lo, hi, S, div=16, spp=256, frames=16, tolerances=(0.01, 0.005), default_tol=0.02):
    """The learned field's bias on a converged image: the frame's camera at
    1/div of its resolution, frames x spp samples per pixel accumulated
    progressively, rendered three times -- exact, exact with other random
    numbers (frameID 1), learned -- and the RMSE of each pair.  The two exact
    images differ by noise only, so their RMSE is the noise floor a bias has
    to show above.  Then the learned image again with the per-macrocell
    fallback at each tighter error tolerance (more macrocells on the exact
    sampler), and the evaluation back at the default tolerance."""
    from helpers import orbit_camera, setup_render
    from owlexastitcher_gb300 import exastitch as E
    w, h = max(a.width // div, 8), max(a.height // div, 8)
    saved = (r.fbSize, r.spp)
    r.resize(w, h)
    r.spp = spp
    setup_render(r.lp, orbit_camera(lo, hi, w, h), w, h, E.PATH_TRACING_INTEGRATOR, spp, "directional", True)
    r.lp.ext.maxBounces = a.bounces
    imgs = {}
    t0 = time.perf_counter()
    for name, learned, frame in (("exact", False, 0), ("exact_other_rng", False, 1), ("learned", True, 0)):
        r.learned = learned
        r.lp.ext.frameID = frame
        r.accumID = 0
        for _ in range(frames):
            r.render()
        r.ctx.sync()
        imgs[name] = r.accum.cpu().numpy().reshape(-1, 4)[:, :3] / (frames * spp)
    secs = time.perf_counter() - t0

    def e(x, y):
        return float(np.sqrt(np.mean((imgs[x] - imgs[y]) ** 2)))
    sweep = []
    for tol in tolerances:
        S.evaluate(tol, 1 << 24)
        st = S.stats()
        r.learned = True
        r.lp.ext.frameID = 0
        r.accumID = 0
        for _ in range(frames):
            r.render()
        r.ctx.sync()
        imgs["tol"] = r.accum.cpu().numpy().reshape(-1, 4)[:, :3] / (frames * spp)
        sweep.append({"tolerance": tol, "fraction_learned": st["numSurrogateMacrocells"] / max(st["numMacrocells"], 1),
                      "rmse_learned_vs_exact_other_rng": e("tol", "exact_other_rng")})
    S.evaluate(default_tol, 1 << 24)
    r.learned = False
    r.lp.ext.frameID = 0
    (fw, fh), r.spp = saved
    r.resize(fw, fh)
    setup_render(r.lp, orbit_camera(lo, hi, fw, fh), fw, fh, E.PATH_TRACING_INTEGRATOR, r.spp, "directional", True)
    r.lp.ext.maxBounces = a.bounces
    return {"width": w, "height": h, "spp": frames * spp, "seconds": secs, "tolerance": default_tol,
            "rmse_exact_vs_exact_other_rng": e("exact", "exact_other_rng"),
            "rmse_learned_vs_exact_other_rng": e("learned", "exact_other_rng"),
            "rmse_learned_vs_exact_same_rng": e("learned", "exact"),
            "tighter_tolerances": sweep}


def run_batched(a, local, flush):
    """256 frames of the small config's field (64 seeded orbit cameras x 4
    transfer functions, square sides drawn from 256..1024, 4 spp, path
    tracing) in one wavefront: autotuned and at the 32^3 grid, run as one
    CUDA graph, against the same frames rendered one exa_render call after
    another (grouped by transfer function)."""
    import ctypes as C
    import torch
    from helpers import orbit_camera, ramp_tf, random_tf, setup_render, step_tf, two_peak_tf
    from owlexastitcher_gb300 import datagen
    from owlexastitcher_gb300 import exastitch as E
    ds = datagen.Dataset("small")
    ctx = E.Context(local)
    model = E.ExaStitchModel.from_dataset(ctx, ds)
    model.setNumGridCells((32, 32, 32))
    sampler = E.ExaStitchSampler(ctx)
    sampler.build(model)
    lo, hi = model.cellBounds
    vr = model.valueRange
    xf = (np.float32(vr[0]), np.float32(vr[1]))
    tfs = [ramp_tf(), step_tf(), two_peak_tf(), random_tf()]
    sampler.computeMaxOpacities(tfs[0], xf)
    lp = E.new_launch_params()
    sampler.setLPs(lp)
    setup_render(lp, orbit_camera(lo, hi, 8, 8), 8, 8, E.PATH_TRACING_INTEGRATOR, 4, "directional", True)
    lp.ext.traceT = lp.ext.traceTr = None
    rng = np.random.default_rng(1234)
    spp = 4
    specs, bufs = [], []
    for cam_i in range(64):
        angle = 2 * np.pi * cam_i / 64 + rng.uniform(-0.05, 0.05)
        elev = rng.uniform(0.1, 0.6)
        for t in range(4):
            side = int(rng.choice([256, 512, 768, 1024]))
            cam = orbit_camera(lo, hi, side, side, angle=angle, elev=elev)
            fb = torch.zeros(side * side, dtype=torch.int32, device="cuda")
            bufs.append(fb)
            specs.append({"cam": cam, "width": side, "height": side, "spp": spp, "tf": t,
                          "frameID": cam_i * 4 + t, "fb": fb.data_ptr()})
    paths = sum(s_["width"] * s_["height"] * s_["spp"] for s_ in specs)
    stream = torch.cuda.current_stream()
    B = E.Batch(ctx)
    B.set_transfer_functions(tfs, [xf] * 4)
    frames = B.frames(specs)

    def timed(fn):
        # one run each: a batch is ~0.5G paths (tens of seconds); the first
        # graph launch of a shape includes its capture (milliseconds)
        flush.fill_(4.0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ctx.sync()
        return e0.elapsed_time(e1)

    # the model's 32^3 grid, tile width 16
    B.set_majorant_grid((32, 32, 32))
    B.set_tile_width(16)
    ms_fixed = timed(lambda: B.render(lp, frames, graph=True))
    st_fixed = ctx.render_stats()
    # autotuned (every 32nd frame at 1 spp for the trials)
    t0 = time.perf_counter()
    tune = B.autotune(lp, frames, sample_every=32)
    tune_s = time.perf_counter() - t0
    if tuple(tune["dims"]) == (32, 32, 32) and tune["tileWidth"] == 16:
        ms_tuned, st_tuned = ms_fixed, st_fixed
    else:
        ms_tuned = timed(lambda: B.render(lp, frames, graph=True))
        st_tuned = ctx.render_stats()

    # the same frames one exa_render call after another
    def sequential():
        for t in range(4):
            sampler.computeMaxOpacities(tfs[t], xf)
            sampler.setLPs(lp)
            for sp in specs:
                if sp["tf"] != t:
                    continue
                org, d00, du, dv = sp["cam"]
                lp.camera.org, lp.camera.dir_00, lp.camera.dir_du, lp.camera.dir_dv = (E._v3(org), E._v3(d00),
                                                                                       E._v3(du), E._v3(dv))
                lp.render.spp = sp["spp"]
                lp.ext.frameID = sp["frameID"]
                lp.accumID = 0
                lp.fbPointer, lp.accumBuffer = sp["fb"], None
                E._check(E.lib().exa_render(ctx.h, C.byref(lp), sp["width"], sp["height"]))
    ms_seq = timed(sequential)
    out = {
        "workload": "small field, 64 orbit cameras x 4 transfer functions = 256 frames, square sides drawn from "
                    "{256,512,768,1024}, 4 spp, path tracing <= 8 bounces",
        "frames": len(specs), "paths": paths,
        "batched_graph_autotuned": {"paths_per_s": paths / (ms_tuned / 1e3), "ms": ms_tuned,
                                    "majorant_grid": list(tune["dims"]), "tile_width": tune["tileWidth"],
                                    "rounds": st_tuned["rounds"], "autotune_seconds": tune_s,
                                    "trials": [{"grid": d[0], "tile_width": tw, "ms": m} for d, tw, m in
                                               tune["trials"]]},
        "batched_graph_grid32": {"paths_per_s": paths / (ms_fixed / 1e3), "ms": ms_fixed,
                                 "rounds": st_fixed["rounds"]},
        "sequential_exa_render_grid32": {"paths_per_s": paths / (ms_seq / 1e3), "ms": ms_seq},
        "speedup_batched_autotuned_over_sequential": ms_seq / ms_tuned,
    }
    ctx.close()
    return out


def run_small_config(a, local, flush, cpu=True):
    """The small configuration's own workloads: (i) 1M uniform points in the
    cell bounds -> field samples/s, (ii) 256x256 primary rays, 1 spp,
    single scatter (direct lighting), one directional light, 32^3 grid ->
    paths/s; plus the majorant build (value ranges + max opacities) at 32^3
    and 128^3.  CPU figures: the oracle on all host cores."""
    import ctypes as C
    import torch
    import pyoracle
    from helpers import host_lp, orbit_camera, ramp_tf, setup_render
    from owlexastitcher_gb300 import datagen
    from owlexastitcher_gb300 import exastitch as E
    ds = datagen.Dataset("small")
    stream = torch.cuda.current_stream()
    out = {"workload": "small field (3 levels, 32^3 root): 1M uniform points; 256x256 x 1 spp direct lighting"}
    builds = {}
    for dims in ((32, 32, 32), (128, 128, 128)):
        ctx = E.Context(local)
        model = E.ExaStitchModel.from_dataset(ctx, ds)
        model.setNumGridCells(dims)
        sampler = E.ExaStitchSampler(ctx)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sampler.build(model)
        vr = model.valueRange
        xf = (np.float32(vr[0]), np.float32(vr[1]))
        sampler.computeMaxOpacities(ramp_tf(), xf)
        ctx.sync()
        builds[f"{dims[0]}^3_gpu_ms"] = (time.perf_counter() - t0) * 1e3
        if dims == (32, 32, 32):
            keep = (ctx, model, sampler, xf)
        else:
            ctx.close()
    ctx, model, sampler, xf = keep
    lo, hi = model.cellBounds
    rng = np.random.default_rng(42)
    P = rng.uniform(lo, hi, (1 << 20, 3)).astype(np.float32)
    pd = torch.from_numpy(P).cuda()
    res = torch.empty((1 << 20) * 3, dtype=torch.int32, device="cuda")
    for _ in range(3):
        sampler.sample_device(pd.data_ptr(), res.data_ptr(), len(P), cull=False)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    flush.fill_(5.0)
    e0.record(stream)
    for _ in range(10):
        sampler.sample_device(pd.data_ptr(), res.data_ptr(), len(P), cull=False)
    e1.record(stream)
    torch.cuda.synchronize()
    out["points_per_s"] = 10 * len(P) / (e0.elapsed_time(e1) / 1e3)
    lp = E.new_launch_params()
    sampler.setLPs(lp)
    w = h = 256
    setup_render(lp, orbit_camera(lo, hi, w, h), w, h, E.DIRECT_LIGHT_INTEGRATOR, 1, "directional", False)
    fb = torch.zeros(w * h, dtype=torch.int32, device="cuda")
    acc = torch.zeros(w * h * 4, dtype=torch.float32, device="cuda")
    lp.fbPointer, lp.accumBuffer = fb.data_ptr(), acc.data_ptr()
    lp.ext.traceT = lp.ext.traceTr = None
    for _ in range(3):
        E._check(E.lib().exa_render(ctx.h, C.byref(lp), w, h))
    ms = []
    for _ in range(5):
        flush.fill_(6.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        E._check(E.lib().exa_render(ctx.h, C.byref(lp), w, h))
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    ctx.sync()
    out["render_256_1spp_dl"] = {"paths_per_s": w * h / (statistics.median(ms) / 1e3), "ms": statistics.median(ms)}
    out["majorant_build"] = builds
    if cpu:
        n = os.cpu_count()
        f = pyoracle.Field(ds.vertices, ds.indices, ds.gridlets, ds.gridlet_scalars)
        f.sample(P[:1000], cull=0, nthreads=n)
        t0 = time.perf_counter()
        f.sample(P, cull=0, nthreads=n)
        cpu_pts = len(P) / (time.perf_counter() - t0)
        t0 = time.perf_counter()
        f.sample(P[:1 << 17], cull=0, nthreads=1)
        cpu_pts1 = (1 << 17) / (time.perf_counter() - t0)
        t0 = time.perf_counter()
        f.majorants((32, 32, 32), lo, hi)
        maj32 = (time.perf_counter() - t0) * 1e3
        t0 = time.perf_counter()
        f.majorants((128, 128, 128), lo, hi)
        maj128 = (time.perf_counter() - t0) * 1e3
        # (ii) on the host: the oracle integrator renders the same frame (the
        # parity tests show it bit-identical), all threads and one thread
        _, ops = sampler.majorants((32, 32, 32))
        _, gops, eops = sampler.prim_majorants()
        o = _oracle_scene(a, ds, lp, ops, gops, eops, ramp_tf())
        hl, *_ = host_lp(lp, o, w, h)
        # 32-row bands: a 256-pixel row per call is too little work to spread over the cores
        dl_n, _, _ = _cpu_render_rate(o, hl, w, h, 1, 2.0, n, band_rows=32)
        dl_1, _, _ = _cpu_render_rate(o, hl, w, h, 1, 2.0, 1, band_rows=32)
        out["cpu"] = {"cores": n, "kind": "port", "points_per_s": cpu_pts, "points_per_s_1_core": cpu_pts1,
                      "render_256_1spp_dl_paths_per_s": dl_n, "render_256_1spp_dl_paths_per_s_1_core": dl_1,
                      "majorant_build_32^3_ms": maj32, "majorant_build_128^3_ms": maj128,
                      "note": "oracle/oracle.c point location (uniform-grid accel), integrator and majorant build"}
    ctx.close()
    out["amrcell_sampler"] = run_comparison_small(ds, local, P, flush, stream, "amrcell")
    out["exabrick_sampler"] = run_comparison_small(ds, local, P, flush, stream, "exabrick")
    return out


def run_comparison_small(ds, local, P, flush, stream, kind):
    """The same two workloads through a comparison sampler over the small
    field's AMR cells: "amrcell" (tent basis over the cells) or "exabrick"
    (bricks of x-runs of cells, region basis): points/s and 256^2 x 1 spp
    direct-lighting paths/s."""
    import ctypes as C
    import torch
    from helpers import orbit_camera, ramp_tf, setup_render
    from owlexastitcher_gb300 import datagen
    from owlexastitcher_gb300 import exastitch as E
    ctx = E.Context(local)
    if kind == "amrcell":
        model = E.AMRCellModel.from_dataset(ctx, ds)
        sampler = E.AMRCellSampler(ctx)
        out = {"cells": len(ds.amr_cells)}
    else:
        t0 = time.perf_counter()
        b, s = datagen.amr_to_bricks(ds.amr_cells, ds.amr_scalars)
        model = E.ExaBrickModel(ctx, b, s)
        sampler = E.ExaBrickSampler(ctx)
        out = {"bricks": len(b), "regions": len(model.abrs()[0]),
               "host_model_ms": (time.perf_counter() - t0) * 1e3}
    model.setNumGridCells((32, 32, 32))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sampler.build(model)
    vr = model.valueRange
    sampler.computeMaxOpacities(ramp_tf(), (np.float32(vr[0]), np.float32(vr[1])))
    ctx.sync()
    out["build_32^3_ms"] = (time.perf_counter() - t0) * 1e3
    pd = torch.from_numpy(P).cuda()
    res = torch.empty(len(P) * 3, dtype=torch.int32, device="cuda")
    for _ in range(3):
        sampler.sample_device(pd.data_ptr(), res.data_ptr(), len(P))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    flush.fill_(7.0)
    e0.record(stream)
    for _ in range(10):
        sampler.sample_device(pd.data_ptr(), res.data_ptr(), len(P))
    e1.record(stream)
    torch.cuda.synchronize()
    out["points_per_s"] = 10 * len(P) / (e0.elapsed_time(e1) / 1e3)
    lo, hi = model.cellBounds
    lp = E.new_launch_params()
    sampler.setLPs(lp)
    w = h = 256
    setup_render(lp, orbit_camera(lo, hi, w, h), w, h, E.DIRECT_LIGHT_INTEGRATOR, 1, "directional", False)
    fb = torch.zeros(w * h, dtype=torch.int32, device="cuda")
    acc = torch.zeros(w * h * 4, dtype=torch.float32, device="cuda")
    lp.fbPointer, lp.accumBuffer = fb.data_ptr(), acc.data_ptr()
    lp.ext.traceT = lp.ext.traceTr = None
    for _ in range(3):
        E._check(E.lib().exa_render(ctx.h, C.byref(lp), w, h))
    ms = []
    for _ in range(5):
        flush.fill_(8.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        E._check(E.lib().exa_render(ctx.h, C.byref(lp), w, h))
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    ctx.sync()
    out["render_256_1spp_dl"] = {"paths_per_s": w * h / (statistics.median(ms) / 1e3), "ms": statistics.median(ms)}
    ctx.close()
    return out


def _oracle_scene(a, ds, lp_src, max_ops, gops, eops, tf):
    import pyoracle
    from helpers import host_lp
    f = pyoracle.Field(ds.vertices, ds.indices, ds.gridlets, ds.gridlet_scalars)
    f.set_prim_opacities(gops if len(gops) else None, eops if len(eops) else None)

    class O:
        pass
    o = O()
    o.f, o.tf, o.max_ops = f, np.ascontiguousarray(tf, np.float32), np.ascontiguousarray(max_ops, np.float32)
    return o


def _cpu_render_rate(o, hl, w, h, spp, budget_s, nthreads, band_rows=1, rows_out=None):
    """Renders bands of `band_rows` rows spread over the frame until
    budget_s is used; returns (paths/s, pixels rendered, seconds).  The
    first rows of the bands rendered are appended to rows_out."""
    rows = h
    bands = 16
    total_px, total_s = 0, 0.0
    for b in range(bands * 64):
        y = (b * 37) % rows
        pb, pe = y * w, min(y + band_rows, rows) * w
        t0 = time.perf_counter()
        o.f.render(bytes(hl), w, h, pb, pe, nthreads)
        total_s += time.perf_counter() - t0
        total_px += pe - pb
        if rows_out is not None:
            rows_out.append(y)
        if total_s >= budget_s:
            break
    return total_px * spp / total_s, total_px, total_s


def _oracle_workload(ds, tf):
    """The workload's scene on the oracle, built from the dataset arrays
    alone: its own bounds, value range, majorant build and max opacities."""
    import pyoracle
    f = pyoracle.Field(ds.vertices, ds.indices, ds.gridlets, ds.gridlet_scalars)
    lo, hi, vr = f.bounds()
    xf = (np.float32(vr[0]), np.float32(vr[1]))
    t0 = time.perf_counter()
    ranges = f.majorants(NUM_MCS, lo, hi)
    build_s = time.perf_counter() - t0
    ops = pyoracle.max_opacities(ranges, tf, xf)
    gops = pyoracle.max_opacities(f.gridlet_value_ranges(), tf, xf) if len(ds.gridlets) else np.zeros(0, np.float32)
    eops = f.elem_max_opacities(tf, xf) if len(ds.indices) else np.zeros(0, np.float32)
    f.set_prim_opacities(gops if len(gops) else None, eops if len(eops) else None)

    class O:
        pass
    o = O()
    o.f, o.tf, o.max_ops = f, np.ascontiguousarray(tf, np.float32), np.ascontiguousarray(ops)
    o.ranges, o.lo, o.hi, o.xf, o.build_s = ranges, lo, hi, xf, build_s
    return o


def _same_floats(a, b):
    """bit-equal float arrays, except that +0 and -0 compare equal (the
    sign of a zero from competing min/max updates is order dependent in the
    reference too)"""
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    return bool(np.array_equal(a, b) and np.array_equal(np.isnan(a), np.isnan(b)))


def cpu_baseline(a, ds, r, budget_s, timed_frame):
    """The oracle integrator on the host cores, all threads (OpenMP), on
    rows of the benchmarked frame, with the oracle's own majorant build.
    Returns (cpu_baseline, parity): parity compares the oracle's majorant
    ranges and max opacities with the GPU build, and the oracle's rendered
    rows with the same rows of the last timed GPU frame, bit for bit."""
    from helpers import host_lp
    n = os.cpu_count()
    o = _oracle_workload(ds, r.colorMap)
    g_ranges, g_ops = r.sampler.majorants(NUM_MCS)
    glo, ghi = r.model.cellBounds
    hl, hfb, hacc, _, _ = host_lp(r.lp, o, a.width, a.height)
    rows = []
    rate, px, secs = _cpu_render_rate(o, hl, a.width, a.height, a.spp, budget_s, n, rows_out=rows)
    acc, fb = timed_frame
    sel = np.concatenate([np.arange(y * a.width, (y + 1) * a.width) for y in sorted(set(rows))])
    bad_px = int(np.count_nonzero((acc[sel] != hacc[sel]).any(axis=1) | (fb[sel] != hfb[sel])))
    parity = {
        "against": "oracle/oracle.c (own bounds, majorant build and max opacities from the dataset arrays)",
        "majorant_grid": list(NUM_MCS),
        "cell_bounds_equal": bool(np.array_equal(o.lo, glo) and np.array_equal(o.hi, ghi)),
        "majorant_ranges_bit_exact": _same_floats(o.ranges, g_ranges),
        "max_opacities_bit_exact": bool(o.max_ops.tobytes() == g_ops.tobytes()),
        "oracle_majorant_build_s": o.build_s,
        "frame": "the last timed frame (accumulation buffer sums and RGBA8 pixels)",
        "rows": len(set(rows)), "pixels": int(len(sel)), "mismatched_pixels": bad_px,
        "bit_exact": bool(acc[sel].tobytes() == hacc[sel].tobytes() and np.array_equal(fb[sel], hfb[sel])),
    }
    cpu = {"value": rate, "unit": "paths/s", "cores": n, "kind": "port",
           "sample": f"{px} pixels x {a.spp} spp (rows spread over the frame), {secs:.1f} s, oracle/oracle.c "
                     f"with OpenMP, majorants from the oracle's own build"}
    return cpu, parity


def run_reference(a):
    """--impl reference: the CPU restatement of the integrator (the reference's
    own path needs OptiX/OWL, which are not available)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if a.config == "cloud":
        print(json.dumps({"impl": "reference", "unavailable": "the CPU restatement's field structures for the "
                          "~400M-cell cloud exceed a bounded CPU sample; the reference arm is defined on medium"}))
        return
    import shutil
    import tempfile
    from helpers import host_lp, orbit_camera, ramp_tf, setup_render
    from owlexastitcher_gb300 import exastitch as E  # launch-parameter layout only; no library is loaded
    # the dataset's arrays come from the generator run as a separate process
    # (as the reference's amrMakeDualMesh tool writes files its renderer
    # loads): this process loads no library of the GPU path
    tmp = tempfile.mkdtemp(prefix="exa_ref_")
    try:
        path = os.path.join(tmp, a.config + ".npz")
        subprocess.check_call([sys.executable, "-m", "owlexastitcher_gb300.datagen", "--config", a.config, "--out",
                               path], cwd=ROOT)
        with np.load(path) as z:
            ds = type("Arrays", (), {k: z[k] for k in ("vertices", "indices", "gridlets", "gridlet_scalars")})
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    tf = ramp_tf()
    o = _oracle_workload(ds, tf)
    lo, hi, xf = o.lo, o.hi, o.xf
    lp = E.LaunchParams()
    lp.integrator = 0
    lp.render.dt = 1.0
    lp.transferFunc.opacityScale = 1.0
    lp.transferFunc.domain.lower, lp.transferFunc.domain.upper = float(xf[0]), float(xf[1])
    lp.transferFunc.numValues = len(tf)
    for A in (lp.voxelSpaceTransform, lp.lightSpaceTransform, lp.ext.voxelSpaceTransformInv):
        A.l.vx.x = A.l.vy.y = A.l.vz.z = 1.0
    lp.majorantGrid.dims = E.vec3i(*NUM_MCS)
    lp.majorantGrid.bounds = E._box(lo, hi)
    lp.worldSpaceBounds = E._box(lo, hi)
    lp.ext.cullTransparentPrims = 1
    cam = orbit_camera(lo, hi, a.width, a.height)
    setup_render(lp, cam, a.width, a.height, 0, a.spp, "directional", True)
    hl, *_ = host_lp(lp, o, a.width, a.height)
    n = os.cpu_count()
    per_step = max(1.0, a.cpu_seconds / max(1, a.steps + a.warmup))
    for _ in range(a.warmup):
        _cpu_render_rate(o, hl, a.width, a.height, a.spp, per_step * 0.3, n)
    rates, pxs, secs = [], 0, 0.0
    for _ in range(a.steps):
        rate, px, s = _cpu_render_rate(o, hl, a.width, a.height, a.spp, per_step, n)
        rates.append(rate)
        pxs += px
        secs += s
    value = pxs * a.spp / secs
    sample = (f"{pxs} pixels x {a.spp} spp over {a.steps} steps (rows spread over the frame), "
              f"oracle/oracle.c restatement with OpenMP; the reference's own path needs OptiX/OWL")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * secs / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded AMR Gaussians + value noise)",
        "config": workload_config(a),
        "cpu_baseline": {"value": value, "unit": "paths/s", "cores": n, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
