"""exa_render_noalloc: the allocation-free variant of exa_render for callers
that cannot allocate device memory in their frame loop.  Collected last
(test_zz_*) so that a stop-at-first-failure run has run everything else."""
import ctypes as C

import numpy as np
import pytest

from conftest import dataset
from helpers import GpuScene, orbit_camera, setup_render

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene(native):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch, GpuScene(dataset("tiny"), (8, 8, 8))


def _frames(torch, g, entry, w, h, spp, fb=None, acc=None):
    """Two progressive frames in a row through one entry point; returns the
    RGBA8 frame buffer and accumulation buffer after each call."""
    from owlexastitcher_gb300 import exastitch as E
    lp = setup_render(g.lp, orbit_camera(g.lo, g.hi, w, h), w, h, E.PATH_TRACING_INTEGRATOR, spp, "directional",
                      True)
    if fb is None:
        fb = torch.zeros(w * h, dtype=torch.int32, device="cuda")
        acc = torch.zeros(w * h * 4, dtype=torch.float32, device="cuda")
    lp.fbPointer, lp.accumBuffer = fb.data_ptr(), acc.data_ptr()
    lp.ext.traceT = lp.ext.traceTr = None
    out = []
    for frame in range(2):
        lp.accumID = frame
        E._check(getattr(E.lib(), entry)(g.ctx.h, C.byref(lp), w, h))
        g.ctx.sync()
        out.append((fb.cpu().numpy().copy(), acc.cpu().numpy().copy()))
    return out


def test_noalloc_matches_render(scene):
    torch, g = scene
    w, h, spp = 64, 48, 4
    ref = _frames(torch, g, "exa_render", w, h, spp)
    got = _frames(torch, g, "exa_render_noalloc", w, h, spp)
    for (rf, ra), (gf, ga) in zip(ref, got):
        assert np.array_equal(rf, gf)            # bit-exact, as in the other parity tests
        assert ra.tobytes() == ga.tobytes()
    assert len(np.unique(ref[1][0])) > 4


def test_noalloc_allocates_nothing(scene):
    """After the first call on the device (the set-up), further calls leave
    the device's free memory unchanged.  The frame buffers are allocated
    before the measurement."""
    torch, g = scene
    w, h = 100, 80
    fb = torch.zeros(w * h, dtype=torch.int32, device="cuda")
    acc = torch.zeros(w * h * 4, dtype=torch.float32, device="cuda")
    _frames(torch, g, "exa_render_noalloc", w, h, 2, fb, acc)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    _frames(torch, g, "exa_render_noalloc", w, h, 16, fb, acc)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_oversized_frame(scene):
    torch, g = scene
    from owlexastitcher_gb300 import exastitch as E
    lp = setup_render(g.lp, orbit_camera(g.lo, g.hi, 1024, 1024), 1024, 1024, E.PATH_TRACING_INTEGRATOR, 2,
                      "directional", True)
    rc = E.lib().exa_render_noalloc(g.ctx.h, C.byref(lp), 1024, 1024)
    assert rc == E.EXA_ERR_INVALID
    assert b"exceeds its static scratch" in E.lib().exa_last_error()


def test_noalloc_rejects_gridlet_shading_without_gridlets(scene):
    """The AMR-cell sampler has no gridlet cells to colour: both entry points
    refuse shade mode "gridlets" for it instead of painting every sample."""
    torch, _ = scene
    from owlexastitcher_gb300 import exastitch as E
    ds = dataset("tiny")
    ctx = E.Context(0)
    model = E.AMRCellModel.from_dataset(ctx, ds)
    model.setNumGridCells((8, 8, 8))
    sampler = E.AMRCellSampler(ctx)
    sampler.build(model)
    vr = model.valueRange
    from helpers import ramp_tf
    sampler.computeMaxOpacities(ramp_tf(), (np.float32(vr[0]), np.float32(vr[1])))
    lp = E.new_launch_params()
    sampler.setLPs(lp)
    lo, hi = model.cellBounds
    w = h = 16
    setup_render(lp, orbit_camera(lo, hi, w, h), w, h, E.DIRECT_LIGHT_INTEGRATOR, 1, "directional", False)
    fb = torch.zeros(w * h, dtype=torch.int32, device="cuda")
    lp.fbPointer, lp.accumBuffer = fb.data_ptr(), None
    lp.ext.traceT = lp.ext.traceTr = None
    lp.shadeMode = E.SHADE_MODE_GRIDLETS
    for entry in ("exa_render", "exa_render_noalloc"):
        assert getattr(E.lib(), entry)(ctx.h, C.byref(lp), w, h) == E.EXA_ERR_INVALID, entry
        assert b"shade mode default" in E.lib().exa_last_error()
    lp.shadeMode = E.SHADE_MODE_DEFAULT
    E._check(E.lib().exa_render_noalloc(ctx.h, C.byref(lp), w, h))
    ctx.sync()
    ctx.close()
