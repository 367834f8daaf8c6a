"""The linear transfer-function filter (EXA_TF_FILTER_LINEAR): the
reference's default texture lookup (deviceCode.cu:331-332 with the texture
of OWLRenderer.cpp:659-707: normalised coordinates, linear filtering, zero
border), restated in binary32.

CPU: known answers of the oracle's lookup (entry centres, midpoints, the
border fade, values outside the domain) and the bound property of the
linear-mode max opacities.  GPU: majorants, max opacities and frames of all
three integrators bit for bit against the oracle under the linear filter,
and a render whose launch parameters name the other filter is rejected."""
import ctypes as C

import numpy as np
import pytest

from helpers import GpuScene, OracleScene, host_lp, orbit_camera, ramp_tf, setup_render, two_peak_tf


def _lp(E, tf, domain, filt):
    lp = E.LaunchParams()
    lp.transferFunc.values = tf.ctypes.data
    lp.transferFunc.numValues = len(tf)
    lp.transferFunc.domain.lower, lp.transferFunc.domain.upper = domain
    lp.ext.tfFilter = filt
    return lp


def test_linear_lookup_known_answers(oracle):
    from owlexastitcher_gb300 import exastitch as E
    n = 8
    tf = np.zeros((n, 4), np.float32)
    tf[:, 3] = np.arange(n, dtype=np.float32) / 8  # alpha k/8 at entry k
    tf[:, 0] = 1.0
    lp = _lp(E, tf, (0.0, 1.0), E.TF_FILTER_LINEAR)
    # entry centres (k + 0.5) / n read entry k exactly
    centres = (np.arange(n, dtype=np.float32) + 0.5) / n
    out = oracle.lookup_tf(bytes(lp), centres)
    assert np.array_equal(out[:, 3], tf[:, 3])
    # midway between two centres: the mean of the two entries
    mids = np.arange(1, n, dtype=np.float32) / n
    out = oracle.lookup_tf(bytes(lp), mids)
    assert np.allclose(out[:, 3], (tf[:-1, 3] + tf[1:, 3]) / 2, atol=1e-7)
    # below the first centre the zero border fades in; past the ends it is 0
    out = oracle.lookup_tf(bytes(lp), np.array([0.0, -0.5 / n, -1.0, 1.0, 1.0 + 0.5 / n, 2.0, np.nan], np.float32))
    assert out[0, 0] == np.float32(0.5) and out[0, 3] == 0.0   # halfway to the border: half of entry 0 (alpha 0)
    assert np.all(out[1:3] == 0) and np.all(out[5:] == 0)
    assert out[3, 3] == np.float32(0.5 * tf[-1, 3])
    # the nearest filter clamps instead
    lpn = _lp(E, tf, (0.0, 1.0), E.TF_FILTER_NEAREST)
    out = oracle.lookup_tf(bytes(lpn), np.array([-1.0, 2.0, 0.49, np.nan], np.float32))
    assert out[0, 3] == tf[0, 3] and out[1, 3] == tf[-1, 3] and out[2, 3] == tf[3, 3]
    # NaN clamps to 1 as under std::min / fminf: the last entry
    assert np.array_equal(out[3], tf[-1])


@pytest.mark.parametrize("tf_fn", [ramp_tf, two_peak_tf])
def test_linear_max_opacities_bound_filtered_opacity(oracle, tf_fn):
    """For random value ranges, the linear-mode max opacity is at least the
    filtered opacity of every value in the range (the property that keeps
    delta tracking unbiased); the nearest-mode mapping of the reference does
    not have it under this filter."""
    from owlexastitcher_gb300 import exastitch as E
    tf = tf_fn()
    rng = np.random.default_rng(3)
    xf = (np.float32(-0.3), np.float32(1.7))
    lp = _lp(E, tf, xf, E.TF_FILTER_LINEAR)
    lo = rng.uniform(-0.6, 2.0, 400).astype(np.float32)
    hi = (lo + rng.exponential(0.05, 400)).astype(np.float32)
    ranges = np.stack([lo, hi], axis=1)
    ops_lin = oracle.max_opacities(ranges, tf, xf, E.TF_FILTER_LINEAR)
    ops_near = oracle.max_opacities(ranges, tf, xf, E.TF_FILTER_NEAREST)
    below_near = 0
    for i in range(len(ranges)):
        v = np.linspace(lo[i], hi[i], 64, dtype=np.float32)
        a = oracle.lookup_tf(bytes(lp), np.concatenate([v, ranges[i]]))[:, 3]
        assert a.max() <= ops_lin[i], i
        below_near += a.max() > ops_near[i]
    assert below_near > 0  # the reference's mapping misses an entry the filter reads for some ranges


@pytest.fixture(scope="module")
def lin_scene(native, oracle):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from conftest import dataset
    from owlexastitcher_gb300 import exastitch as E
    ds = dataset("small")
    g = GpuScene(ds, (32, 32, 32), tf=two_peak_tf())
    g.ctx.set_tf_filter(E.TF_FILTER_LINEAR)
    g.sampler.computeMaxOpacities(g.tf, g.xf)
    g.sampler.setLPs(g.lp)
    assert g.lp.ext.tfFilter == E.TF_FILTER_LINEAR
    o = OracleScene(oracle, ds, (32, 32, 32), g.lo, g.hi, g.tf, g.xf, tf_filter=E.TF_FILTER_LINEAR)
    return torch, ds, g, o


@pytest.mark.gpu
def test_linear_majorants_bit_exact(lin_scene, oracle):
    torch, ds, g, o = lin_scene
    ranges, ops = g.sampler.majorants(g.num_mcs)
    assert ops.tobytes() == o.max_ops.tobytes()
    gr, gop, eop = g.sampler.prim_majorants()
    assert gop.tobytes() == o.g_ops.tobytes() and eop.tobytes() == o.e_ops.tobytes()
    # the linear filter's spans differ from the nearest lookup's
    near = oracle.max_opacities(o.ranges, g.tf, g.xf, 0)
    assert np.any(ops != near)


@pytest.mark.gpu
@pytest.mark.parametrize("integrator,light,ext", [(0, "directional", True), (1, "point", False), (2, "none", False)])
def test_linear_render_bit_exact(lin_scene, integrator, light, ext):
    torch, ds, g, o = lin_scene
    from owlexastitcher_gb300 import exastitch as E
    w, h = 48, 40
    lp = setup_render(g.lp, orbit_camera(g.lo, g.hi, w, h), w, h, integrator, 2, light, ext, g.lo, g.hi)
    lp.render.dt = 0.5
    n = w * h
    fb = torch.zeros(n, dtype=torch.int32, device="cuda")
    acc = torch.zeros(n * 4, dtype=torch.float32, device="cuda")
    lp.accumID = 0
    lp.fbPointer, lp.accumBuffer = fb.data_ptr(), acc.data_ptr()
    lp.ext.traceT = lp.ext.traceTr = None
    E._check(E.lib().exa_render(g.ctx.h, C.byref(lp), w, h))
    g.ctx.sync()
    hl, hfb, hacc, _, _ = host_lp(lp, o, w, h)
    assert o.f.render(bytes(hl), w, h) == 0
    assert acc.cpu().numpy().reshape(-1, 4).tobytes() == hacc.tobytes()
    assert np.array_equal(fb.cpu().numpy().view(np.uint32), hfb)
    assert len(np.unique(hfb)) > 4
    lp.render.dt = 1.0


@pytest.mark.gpu
def test_filter_mismatch_rejected(lin_scene):
    torch, ds, g, o = lin_scene
    from owlexastitcher_gb300 import exastitch as E
    w = h = 16
    lp = setup_render(g.lp, orbit_camera(g.lo, g.hi, w, h), w, h, 1, 1, "none", False)
    fb = torch.zeros(w * h, dtype=torch.int32, device="cuda")
    lp.fbPointer, lp.accumBuffer = fb.data_ptr(), None
    lp.ext.tfFilter = E.TF_FILTER_NEAREST
    try:
        assert E.lib().exa_render(g.ctx.h, C.byref(lp), w, h) == E.EXA_ERR_INVALID
        assert b"tfFilter" in E.lib().exa_last_error()
    finally:
        lp.ext.tfFilter = E.TF_FILTER_LINEAR
    with pytest.raises(E.ExaError):
        g.ctx.set_tf_filter(7)
