"""Batched frames (exa_render_batch): every frame of a batch equals exa_render
of that frame alone, bit for bit, whatever the job tile width and whether
the rounds run from a host loop or inside the CUDA graph -- including
transfer functions that make primitives transparent (culling) -- plus the
autotuner's trials."""
import ctypes as C

import numpy as np
import pytest

from conftest import dataset
from helpers import GpuScene, orbit_camera, ramp_tf, random_tf, setup_render, step_tf, two_peak_tf

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def scene(torch_cuda, native):
    ds = dataset("small")
    return ds, GpuScene(ds, (32, 32, 32))


TFS = [ramp_tf(), step_tf(), two_peak_tf(), random_tf()]
SIZES = [(16, 16), (40, 24), (33, 17), (24, 40), (8, 8), (47, 31)]


def _frames(g, torch, spps=(1, 2)):
    specs, bufs = [], []
    for i, (w, h) in enumerate(SIZES):
        cam = orbit_camera(g.lo, g.hi, w, h, angle=0.3 + 0.9 * i, elev=0.2 + 0.05 * i)
        fb = torch.zeros(w * h, dtype=torch.int32, device="cuda")
        acc = torch.zeros(w * h * 4, dtype=torch.float32, device="cuda")
        bufs.append((fb, acc))
        specs.append({"cam": cam, "width": w, "height": h, "spp": spps[i % 2], "tf": i % len(TFS),
                      "frameID": 7 * i, "fb": fb.data_ptr(), "accum": acc.data_ptr()})
    return specs, bufs


def _single(g, torch, lp_tpl, spec, accum=None):
    """exa_render of one frame with the same parameters"""
    from owlexastitcher_gb300 import exastitch as E
    w, h = spec["width"], spec["height"]
    g.sampler.computeMaxOpacities(TFS[spec["tf"]], g.xf)
    lp = E.LaunchParams.from_buffer_copy(bytes(lp_tpl))
    g.sampler.setLPs(lp)
    org, d00, du, dv = spec["cam"]
    lp.camera.org, lp.camera.dir_00, lp.camera.dir_du, lp.camera.dir_dv = E._v3(org), E._v3(d00), E._v3(du), E._v3(dv)
    lp.render.spp = spec["spp"]
    lp.ext.frameID = spec["frameID"]
    lp.accumID = spec.get("accumID", 0)
    fb = torch.zeros(w * h, dtype=torch.int32, device="cuda")
    acc = torch.zeros(w * h * 4, dtype=torch.float32, device="cuda") if accum is None else accum.clone()
    lp.fbPointer, lp.accumBuffer = fb.data_ptr(), acc.data_ptr()
    lp.ext.traceT = lp.ext.traceTr = None
    E._check(E.lib().exa_render(g.ctx.h, C.byref(lp), w, h))
    g.ctx.sync()
    return fb.cpu().numpy(), acc.cpu().numpy()


def _template(g, integrator):
    from owlexastitcher_gb300 import exastitch as E
    lp = setup_render(g.lp, orbit_camera(g.lo, g.hi, 8, 8), 8, 8, integrator, 1, "directional", integrator == 0,
                      g.lo, g.hi)
    tpl = E.LaunchParams.from_buffer_copy(bytes(lp))
    tpl.ext.traceT = tpl.ext.traceTr = None
    return tpl


def _restore(g):
    g.sampler.computeMaxOpacities(g.tf, g.xf)
    g.sampler.setLPs(g.lp)


@pytest.mark.parametrize("integrator,tile,graph", [(0, 16, True), (0, 8, False), (1, 32, True), (0, 32, False)])
def test_batch_equals_single_frames(scene, torch_cuda, integrator, tile, graph):
    torch = torch_cuda
    from owlexastitcher_gb300 import exastitch as E
    ds, g = scene
    tpl = _template(g, integrator)
    B = E.Batch(g.ctx)
    B.set_transfer_functions(TFS, [g.xf] * len(TFS))
    B.set_majorant_grid(g.num_mcs)
    B.set_tile_width(tile)
    specs, bufs = _frames(g, torch)
    B.render(tpl, B.frames(specs), graph=graph)
    g.ctx.sync()
    assert g.ctx.device_errors() == 0
    try:
        for spec, (fb, acc) in zip(specs, bufs):
            sfb, sacc = _single(g, torch, tpl, spec)
            assert np.array_equal(fb.cpu().numpy(), sfb)
            assert acc.cpu().numpy().tobytes() == sacc.tobytes()
    finally:
        _restore(g)


def test_batch_graph_replay_and_accumulation(scene, torch_cuda):
    """The cached graph replayed with accumID 1 gives the progressive result
    of exa_render."""
    torch = torch_cuda
    from owlexastitcher_gb300 import exastitch as E
    ds, g = scene
    tpl = _template(g, 0)
    B = E.Batch(g.ctx)
    B.set_transfer_functions(TFS, [g.xf] * len(TFS))
    B.set_majorant_grid(g.num_mcs)
    B.set_tile_width(16)
    specs, bufs = _frames(g, torch)
    B.render(tpl, B.frames(specs), graph=True)
    g.ctx.sync()
    first = [acc.clone() for _, acc in bufs]
    for sp in specs:
        sp["accumID"] = 1
    B.render(tpl, B.frames(specs), graph=True)
    g.ctx.sync()
    try:
        for spec, (fb, acc), acc0 in zip(specs, bufs, first):
            sfb, sacc = _single(g, torch, tpl, spec, accum=acc0)
            assert np.array_equal(fb.cpu().numpy(), sfb)
            assert acc.cpu().numpy().tobytes() == sacc.tobytes()
    finally:
        _restore(g)


def test_batch_autotune(scene, torch_cuda):
    torch = torch_cuda
    from owlexastitcher_gb300 import exastitch as E
    ds, g = scene
    tpl = _template(g, 0)
    B = E.Batch(g.ctx)
    B.set_transfer_functions(TFS, [g.xf] * len(TFS))
    specs, bufs = _frames(g, torch)
    res = B.autotune(tpl, B.frames(specs), sample_every=2)
    assert len(res["trials"]) == 12
    assert {t[0][0] for t in res["trials"]} == {32, 64, 128, 256}
    assert {t[1] for t in res["trials"]} == {8, 16, 32}
    assert all(t[2] > 0 for t in res["trials"])
    assert res["msBest"] == min(t[2] for t in res["trials"])
    # the tuned setting renders
    B.render(tpl, B.frames(specs), graph=True)
    g.ctx.sync()
    assert g.ctx.device_errors() == 0
