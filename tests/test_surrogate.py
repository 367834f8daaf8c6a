"""The learned field (hash-grid encoding + MLP): oracle self-checks on the
CPU, and on the GPU the forward and gradients against the oracle, training,
per-macrocell error bounds, the fallback and rendering.

Tolerances: the encoding is restated bit for bit, but the tensor cores'
FP32 accumulation order is not specified, so a BF16 rounding of an
activation can land on the other side of a tie; the forward is compared at
1e-2 of the output scale (and 1e-4 at the median), the gradients as vectors
at 2e-2 relative L2 error.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import dataset
from helpers import GpuScene, OracleScene, host_lp, orbit_camera, ramp_tf, setup_render


# ------------------------------------------------------------------ CPU
def test_half_and_bf16_rounding(oracle):
    rng = np.random.default_rng(7)
    v = np.concatenate([rng.standard_normal(20000) * 10.0 ** rng.integers(-9, 5, 20000),
                        [0.0, -0.0, 65504.0, 65519.0, 6.1035156e-05, 5.9604645e-08, 1.0, 1.00048828125]]).astype(np.float32)
    L = oracle.lib()
    with np.errstate(over="ignore"):
        want_h = v.astype(np.float16).astype(np.float32)
    got_h = np.array([L.os_half(float(x)) for x in v], np.float32)
    assert got_h.tobytes() == want_h.tobytes()
    # bf16: round to nearest even on the upper 16 bits
    u = v.view(np.uint32).astype(np.uint64)
    want_b = (((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)).view(np.float32)
    got_b = np.array([L.os_bf16(float(x)) for x in v], np.float32)
    assert got_b.tobytes() == want_b.tobytes()


def test_resolution_schedule(oracle):
    g = oracle.sur_geom(19, 16, 1.5, [0, 0, 0], [128, 128, 128], 0.0, 1.0)
    res = list(g.res)
    assert res == [int(np.floor(16 * 1.5 ** l)) for l in range(16)]
    # dense where (res + 1)^3 fits 2^19 entries
    dense = [(r + 1) ** 3 <= (1 << 19) for r in res]
    assert [bool((g.denseMask >> l) & 1) for l in range(16)] == dense


def _random_params(rng, log2T, table_scale=0.5):
    w = np.concatenate([rng.uniform(-0.4, 0.4, 64 * 32), rng.uniform(-0.3, 0.3, 64 * 64),
                        rng.uniform(-0.3, 0.3, 64)]).astype(np.float32)
    t = rng.uniform(-table_scale, table_scale, 2 * 16 * (1 << log2T)).astype(np.float32)
    return w, t


def test_oracle_backward_matches_finite_differences(oracle):
    """The oracle's chain rule, with its roundings switched off, against
    central differences of its own forward."""
    L = oracle.lib()
    rng = np.random.default_rng(3)
    log2T = 10
    geom = oracle.sur_geom(log2T, 4, 1.5, [0, 0, 0], [1, 1, 1], 0.0, 1.0)
    w, t = _random_params(rng, log2T)
    pairs = np.concatenate([rng.uniform(0, 1, (24, 3)), rng.uniform(0, 1, (24, 1))], axis=1).astype(np.float32)
    L.os_set_exact(1)
    try:
        gw, gt, loss = oracle.sur_gradients(geom, w, t, pairs)

        def f(w_, t_):
            return oracle.sur_gradients(geom, w_, t_, pairs)[2]

        def fd_ok(vec, idx, grad, which):
            # central differences at three steps: a large step can carry a
            # ReLU input across zero, a small one drowns in rounding, so the
            # check passes when one of them agrees
            best = np.inf
            for h in (1e-2, 1e-3, 1e-4):
                p, m = vec.copy(), vec.copy()
                p[idx] += h
                m[idx] -= h
                h2 = float(p[idx]) - float(m[idx])
                fd = ((f(p, t) - f(m, t)) if which == "w" else (f(w, p) - f(w, m))) / h2
                best = min(best, abs(fd - grad))
            return best <= 2e-2 * abs(grad) + 2e-4 * np.abs(gw if which == "w" else gt).max()

        checked = 0
        for idx in rng.choice(len(w), 12, replace=False):
            assert fd_ok(w, idx, gw[idx], "w")
            checked += 1
        for idx in rng.choice(np.flatnonzero(gt), 12, replace=False):
            assert fd_ok(t, idx, gt[idx], "t")
            checked += 1
        assert checked == 24
    finally:
        L.os_set_exact(0)


# ------------------------------------------------------------------ GPU
gpu = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def small_scene(torch_cuda, native):
    ds = dataset("small")
    return ds, GpuScene(ds, (32, 32, 32))


def _surrogate(g, **kw):
    from owlexastitcher_gb300 import exastitch as E
    params = dict(log2TableSize=14, numSamples=1 << 18, batch=1 << 14, seed=11)
    params.update(kw)
    return E.Surrogate(g.ctx, **params)


@gpu
def test_geometry_matches_oracle(small_scene, oracle):
    ds, g = small_scene
    S = _surrogate(g)
    geo = oracle.sur_geom(14, 16, 1.5, g.lo, g.hi, g.vr[0], g.vr[1])
    a, b = S.geometry, geo
    assert a.log2TableSize == b.log2T and a.denseMask == b.denseMask
    assert list(a.res) == list(b.res)
    assert list(a.lo) == list(b.lo) and list(a.inv) == list(b.inv)
    assert (a.vmin, a.vrange) == (b.vmin, b.vrange)


@gpu
def test_forward_matches_oracle(small_scene, oracle, torch_cuda):
    torch = torch_cuda
    ds, g = small_scene
    S = _surrogate(g)
    rng = np.random.default_rng(5)
    w, t = _random_params(rng, 14)
    S.set_params(w, t)
    n = 8192
    pos = (g.lo + rng.uniform(-0.02, 1.02, (n, 3)) * (g.hi - g.lo)).astype(np.float32)
    pd = torch.from_numpy(pos).cuda()
    out = torch.zeros(n, dtype=torch.float32, device="cuda")
    S.sample_device(pd.data_ptr(), out.data_ptr(), n)
    g.ctx.sync()
    geo = oracle.sur_geom(14, 16, 1.5, g.lo, g.hi, g.vr[0], g.vr[1])
    want = geo.vmin + oracle.sur_forward(geo, w, t, pos) * geo.vrange
    got = out.cpu().numpy().astype(np.float64)
    err = np.abs(got - want)
    scale = max(np.abs(want - geo.vmin).max(), 1e-3)
    assert err.max() <= 1e-2 * scale
    assert np.median(err) <= 1e-4 * scale


@gpu
def test_gradients_match_oracle(small_scene, oracle):
    ds, g = small_scene
    S = _surrogate(g)
    rng = np.random.default_rng(9)
    w, t = _random_params(rng, 14, table_scale=0.2)
    S.set_params(w, t)
    n = 1000
    pos = (g.lo + rng.uniform(0, 1, (n, 3)) * (g.hi - g.lo)).astype(np.float32)
    val = (g.vr[0] + rng.uniform(0, 1, n) * (g.vr[1] - g.vr[0])).astype(np.float32)
    val[::17] = np.nan  # pairs without a sample take no part
    pairs = np.concatenate([pos, val[:, None]], axis=1)
    gw, gt, loss = S.gradients(pairs)
    geo = oracle.sur_geom(14, 16, 1.5, g.lo, g.hi, g.vr[0], g.vr[1])
    ow, ot, oloss = oracle.sur_gradients(geo, w, t, pairs)
    assert abs(loss - oloss) <= 1e-3 * oloss
    for a, b in ((gw[:2048], ow[:2048]), (gw[2048:6144], ow[2048:6144]), (gw[6144:], ow[6144:]), (gt, ot)):
        assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b)
    assert np.count_nonzero(gt) > 0


@gpu
def test_training_gains_over_untrained(small_scene):
    """What training buys: the probe error falls by far and many macrocells
    switch to the learned field (before training only cells whose values sit
    at the bottom of the range pass, where the untrained output is near 0)."""
    ds, g = small_scene
    S = _surrogate(g, log2TableSize=18, numSamples=1 << 22, batch=1 << 17)
    S.evaluate(0.02, 1 << 20)
    before = S.stats()
    loss0 = S.train(1)
    loss = S.train(1200)
    S.evaluate(0.02, 1 << 20)
    after = S.stats()
    assert loss < 0.1 * loss0
    assert after["rmse"] < 0.2 * before["rmse"]
    assert after["numSurrogateMacrocells"] > 0.5 * after["numMacrocells"]
    assert after["numSurrogateMacrocells"] > 10 * before["numSurrogateMacrocells"]
    mode, err, maj = S.macrocells(32 ** 3)
    ranges, ops = g.sampler.majorants(g.num_mcs)
    # widened majorants bound the exact ones; exact-mode cells keep theirs
    assert np.all(maj >= ops)
    assert np.array_equal(maj[mode == 0], ops[mode == 0])
    assert np.all(err[mode == 1] <= 0.02 * (g.vr[1] - g.vr[0]))
    assert after["inferenceBytes"] > 0 and after["fieldBytes"] > 0


@gpu
def test_zero_tolerance_render_equals_exact(small_scene, oracle, torch_cuda):
    """With tolerance 0 every macrocell keeps the exact sampler: the learned
    walk kernel must then give the exact path's image bit for bit."""
    torch = torch_cuda
    from owlexastitcher_gb300 import exastitch as E
    ds, g = small_scene
    S = _surrogate(g)
    S.train(20)
    S.evaluate(0.0, 1 << 18)
    assert S.stats()["numSurrogateMacrocells"] == 0
    w, h = 48, 40
    cam = orbit_camera(g.lo, g.hi, w, h)
    lp = setup_render(g.lp, cam, w, h, 0, 2, "directional", True, g.lo, g.hi)
    imgs = []
    for fn in (E.lib().exa_render, E.lib().exa_render_surrogate):
        fb = torch.zeros(w * h, dtype=torch.int32, device="cuda")
        acc = torch.zeros(w * h * 4, dtype=torch.float32, device="cuda")
        lp.accumID = 0
        lp.fbPointer, lp.accumBuffer = fb.data_ptr(), acc.data_ptr()
        lp.ext.traceT = lp.ext.traceTr = None
        E._check(fn(g.ctx.h, C.byref(lp), w, h))
        g.ctx.sync()
        imgs.append(acc.cpu().numpy())
    assert imgs[0].tobytes() == imgs[1].tobytes()


@gpu
def test_learned_render_converged_rmse(small_scene, oracle, torch_cuda):
    """The learned-field workload's integrator (path tracing, albedo 0.8,
    HG g = 0.3, <= 8 bounces, one directional light) on the small field:
    converged 32x32 images at 32768 spp against the FP64 path-tracing oracle
    at 32768 spp.  The exact sampler's image is within 0.005 RMSE of it
    (the noise floor of both), the learned field + exact fallback within
    0.01 (absolute).  Learned densities above their macrocell's widened
    majorant are limited to it (so tracking stays unbiased for the limited
    field); they are counted and must stay rare."""
    torch = torch_cuda
    from owlexastitcher_gb300 import exastitch as E
    ds, g = small_scene
    S = _surrogate(g, log2TableSize=18, numSamples=1 << 22, batch=1 << 17)
    S.train(1200)
    S.evaluate(0.02, 1 << 21)
    st = S.stats()
    assert st["numSurrogateMacrocells"] > 0
    w, h, spp, frames = 32, 32, 4096, 8
    cam = orbit_camera(g.lo, g.hi, w, h)
    lp = setup_render(g.lp, cam, w, h, E.PATH_TRACING_INTEGRATOR, spp, "directional", True, g.lo, g.hi)
    cnt = torch.zeros(16, dtype=torch.int64, device="cuda")

    def gpu_image(fn, counters=None):
        img = np.zeros((w * h, 3), np.float64)
        for fr in range(frames):  # independent RNG streams per frame
            fb = torch.zeros(w * h, dtype=torch.int32, device="cuda")
            acc = torch.zeros(w * h * 4, dtype=torch.float32, device="cuda")
            lp.accumID = 0
            lp.ext.frameID = fr
            lp.fbPointer, lp.accumBuffer = fb.data_ptr(), acc.data_ptr()
            lp.ext.traceT = lp.ext.traceTr = None
            lp.ext.stepCounters = counters
            E._check(fn(g.ctx.h, C.byref(lp), w, h))
            g.ctx.sync()
            lp.ext.stepCounters = None
            img += acc.cpu().numpy().reshape(-1, 4)[:, :3].astype(np.float64)
        return img / (spp * frames)

    exact = gpu_image(E.lib().exa_render)
    learned = gpu_image(E.lib().exa_render_surrogate, cnt.data_ptr())
    lp.ext.frameID = 0
    o = OracleScene(oracle, ds, g.num_mcs, g.lo, g.hi, g.tf, g.xf)
    hl = host_lp(lp, o, w, h)[0]
    hl.render.spp = spp * frames
    ref = o.f.render_f64(bytes(hl), w, h)
    c = cnt.cpu().numpy()
    n_learned, n_limited = int(c[10]), int(c[11])
    assert n_learned > 0
    assert n_limited <= 1e-3 * n_learned

    def rmse(a, b):
        return float(np.sqrt(np.mean((a - b) ** 2)))

    e_exact, e_learned = rmse(exact, ref), rmse(learned, ref)
    print(f"RMSE vs FP64: exact {e_exact:.5f}, learned {e_learned:.5f}; limited {n_limited} of {n_learned}")
    assert e_exact <= 0.005
    assert e_learned <= 0.01
