"""The failure paths: loop caps that end a walk and report it, and the
majorant build's bulk-copy wait.  Nothing here makes a GPU fault, trap or
hang: the caps are lowered to a few iterations (lp.ext.trackStepCap,
lp.ext.ddaCellCap), and the build's time-out is simulated after its copy
completed (exa_debug_set_flags).

A capped walk ends as the oracle's does (the same bits for the frame) and
raises its EXA_DEVERR bit; exa_sync then returns EXA_ERR_DEVICE_LIMIT, and
the next frame with the default caps renders cleanly.  A build whose copy
wait gave up returns EXA_ERR_CUDA; the next build succeeds."""
import ctypes as C

import numpy as np
import pytest

from conftest import dataset
from helpers import GpuScene, OracleScene, host_lp, orbit_camera, setup_render

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene(native, oracle):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ds = dataset("small")
    g = GpuScene(ds, (32, 32, 32))
    o = OracleScene(oracle, ds, (32, 32, 32), g.lo, g.hi, g.tf, g.xf)
    return torch, ds, g, o


def _frame(torch, g, o, w, h, track_cap=0, dda_cap=0):
    from owlexastitcher_gb300 import exastitch as E
    lp = setup_render(g.lp, orbit_camera(g.lo, g.hi, w, h), w, h, E.PATH_TRACING_INTEGRATOR, 2, "directional", True,
                      g.lo, g.hi)
    lp.ext.trackStepCap, lp.ext.ddaCellCap = track_cap, dda_cap
    fb = torch.zeros(w * h, dtype=torch.int32, device="cuda")
    acc = torch.zeros(w * h * 4, dtype=torch.float32, device="cuda")
    lp.accumID = 0
    lp.fbPointer, lp.accumBuffer = fb.data_ptr(), acc.data_ptr()
    lp.ext.traceT = lp.ext.traceTr = None
    try:
        E._check(E.lib().exa_render(g.ctx.h, C.byref(lp), w, h))
        rc = E.lib().exa_sync(g.ctx.h)
        msg = E.lib().exa_last_error()
        hl, hfb, hacc, _, _ = host_lp(lp, o, w, h)
        oerr = o.f.render(bytes(hl), w, h)
    finally:
        lp.ext.trackStepCap = lp.ext.ddaCellCap = 0
    same = acc.cpu().numpy().reshape(-1, 4).tobytes() == hacc.tobytes()
    return rc, msg, oerr, same


@pytest.mark.parametrize("cap,bit", [("track", 2), ("dda", 1)])
def test_lowered_cap_reported_then_clean(scene, cap, bit):
    torch, ds, g, o = scene
    from owlexastitcher_gb300 import exastitch as E
    kw = {"track_cap": 1} if cap == "track" else {"dda_cap": 2}
    rc, msg, oerr, same = _frame(torch, g, o, 40, 32, **kw)
    assert rc == E.EXA_ERR_DEVICE_LIMIT
    assert f"bits {bit})".encode() in msg
    assert oerr & bit          # the oracle hits the same cap
    assert same                # and ends the capped walks the same way
    # the next frame with the default caps is clean and bit-exact
    rc, msg, oerr, same = _frame(torch, g, o, 40, 32)
    assert rc == E.EXA_OK and oerr == 0 and same
    assert g.ctx.device_errors() == 0


def test_negative_cap_rejected(scene):
    torch, ds, g, o = scene
    from owlexastitcher_gb300 import exastitch as E
    lp = setup_render(g.lp, orbit_camera(g.lo, g.hi, 8, 8), 8, 8, 1, 1, "none", False)
    lp.ext.trackStepCap = -1
    try:
        assert E.lib().exa_render(g.ctx.h, C.byref(lp), 8, 8) == E.EXA_ERR_INVALID
        assert b"negative loop cap" in E.lib().exa_last_error()
    finally:
        lp.ext.trackStepCap = 0


def test_build_copy_wait_timeout_reported(scene, oracle):
    """The majorant build's bounded bulk-copy wait: a wait that gives up
    sets EXA_DEVERR_COPY_WAIT and exa_sampler_build returns EXA_ERR_CUDA."""
    torch, ds, g, o = scene
    from owlexastitcher_gb300 import exastitch as E
    ctx = E.Context(0)
    model = E.ExaStitchModel.from_dataset(ctx, ds)
    model.setNumGridCells((32, 32, 32))
    E._check(E.lib().exa_debug_set_flags(ctx.h, E.DEBUG_COPY_WAIT_TIMEOUT))
    assert E.lib().exa_sampler_build(ctx.h) == E.EXA_ERR_CUDA
    assert b"bulk copy into shared memory did not complete" in E.lib().exa_last_error()
    assert E.lib().exa_debug_set_flags(ctx.h, 2) == E.EXA_ERR_INVALID
    E._check(E.lib().exa_debug_set_flags(ctx.h, 0))
    sampler = E.ExaStitchSampler(ctx)
    sampler.build(model)
    ranges, _ = sampler.majorants((32, 32, 32))
    from test_gpu_parity import same_floats
    assert same_floats(ranges, o.ranges)
    assert ctx.device_errors() == 0
    ctx.close()


def test_majorant_grid_dims_checked(scene):
    """launch parameters whose majorant grid is not the built one (the DDA
    would index the max opacities past their end) are rejected by exa_render
    and exa_render_noalloc before any launch; the dims set by
    exa_sampler_set_lps render"""
    torch, ds, g, o = scene
    from owlexastitcher_gb300 import exastitch as E
    w = h = 16
    lp = setup_render(g.lp, orbit_camera(g.lo, g.hi, w, h), w, h, E.DIRECT_LIGHT_INTEGRATOR, 1, "directional", True,
                      g.lo, g.hi)
    fb = torch.zeros(w * h, dtype=torch.int32, device="cuda")
    lp.fbPointer, lp.accumBuffer = fb.data_ptr(), None
    lp.ext.traceT = lp.ext.traceTr = None
    dims = (lp.majorantGrid.dims.x, lp.majorantGrid.dims.y, lp.majorantGrid.dims.z)
    assert dims == (32, 32, 32)
    try:
        lp.majorantGrid.dims = E.vec3i(64, 32, 32)
        for fn in (E.lib().exa_render, E.lib().exa_render_noalloc):
            assert fn(g.ctx.h, C.byref(lp), w, h) == E.EXA_ERR_INVALID
            assert b"majorantGrid" in E.lib().exa_last_error()
    finally:
        lp.majorantGrid.dims = E.vec3i(*dims)
    E._check(E.lib().exa_render(g.ctx.h, C.byref(lp), w, h))
    g.ctx.sync()
    assert g.ctx.device_errors() == 0
