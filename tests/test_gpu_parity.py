"""Parity of the CUDA path with the oracle (bit-exact: the kernels and the
oracle evaluate the same IEEE binary32 operations in the same order).

Covers: majorant value ranges and max opacities (Grid.cu), per-primitive
ranges/opacities (sampler/ExaStitchSampler.cu), point sampling
(sampler/ExaStitchSampler.h sample()), and rendered frames of both
integrators (deviceCode.cu) including per-ray free-flight distance and
shadow transmittance.
"""
import numpy as np
import pytest

from conftest import dataset
from helpers import GpuScene, OracleScene, host_lp, orbit_camera, ramp_tf, setup_render, step_tf, two_peak_tf

pytestmark = pytest.mark.gpu

# (name, generator configuration, generator overrides, majorant grid); the
# unbalanced small field (no 2:1 balance) has tetrahedra in its dual mesh
CONFIGS = [("tiny", "tiny", {}, (8, 8, 8)), ("small", "small", {}, (32, 32, 32)),
           ("small_unbalanced", "small", {"balance": 0}, (32, 32, 32))]


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module", params=CONFIGS, ids=[c[0] for c in CONFIGS])
def scenes(request, torch_cuda, native, oracle):
    name, cfg, kw, dims = request.param
    ds = dataset(cfg, **kw)
    g = GpuScene(ds, dims)
    o = OracleScene(oracle, ds, dims, g.lo, g.hi, g.tf, g.xf)
    return ds, g, o


def same_floats(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    # +0 and -0 compare equal: the reference's CAS min/max keeps whichever
    # arrives first, so the sign of a zero is order dependent there
    return np.array_equal(a, b) and np.array_equal(np.isnan(a), np.isnan(b))


def test_majorant_ranges_bit_exact(scenes):
    ds, g, o = scenes
    ranges, ops = g.sampler.majorants(g.num_mcs)
    assert same_floats(ranges, o.ranges)
    assert (ranges[:, 0] <= ranges[:, 1]).sum() > 0
    assert ops.tobytes() == o.max_ops.tobytes()


def test_prim_ranges_and_opacities(scenes):
    ds, g, o = scenes
    gr, gop, eop = g.sampler.prim_majorants()
    assert same_floats(gr, o.g_ranges)
    assert gop.tobytes() == o.g_ops.tobytes()
    assert eop.tobytes() == o.e_ops.tobytes()


@pytest.mark.parametrize("tf_fn", [ramp_tf, step_tf, two_peak_tf])
def test_max_opacities_other_tfs(scenes, oracle, tf_fn):
    ds, g, o = scenes
    tf = tf_fn()
    xf = (np.float32(g.vr[0]), np.float32(0.5 * (g.vr[0] + g.vr[1])))
    g.sampler.computeMaxOpacities(tf, xf)
    _, ops = g.sampler.majorants(g.num_mcs)
    assert ops.tobytes() == oracle.max_opacities(o.ranges, tf, xf).tobytes()
    g.sampler.computeMaxOpacities(g.tf, g.xf)  # restore
    g.sampler.setLPs(g.lp)


def _check_samples(gs, os_):
    assert np.array_equal(gs["primID"], os_["primID"])
    assert np.array_equal(gs["cellID"], os_["cellID"])
    assert gs["value"].tobytes() == os_["value"].tobytes()


@pytest.mark.parametrize("cull", [False, True])
def test_sample_points_random(scenes, cull):
    ds, g, o = scenes
    rng = np.random.default_rng(42)
    ext = g.hi - g.lo
    P = rng.uniform(g.lo - 0.05 * ext, g.hi + 0.05 * ext, (20000, 3)).astype(np.float32)
    gs = g.sampler.sample_host(P, cull=cull)
    os_ = o.f.sample(P, cull=int(cull))
    _check_samples(gs, os_)
    assert (gs["primID"] >= 0).mean() > 0.5
    assert ((gs["primID"] >= 0) & (gs["cellID"] == -1)).sum() > 0  # elements hit too


def test_sample_points_on_faces_and_vertices(scenes):
    """Points exactly on gridlet faces / lattice vertices and on element
    vertices: several primitives contain them; both sides take the
    lowest-index one."""
    ds, g, o = scenes
    rng = np.random.default_rng(5)
    pts = []
    for gl in ds.gridlets[:: max(1, len(ds.gridlets) // 40)]:
        cw = 2.0 ** gl["level"]
        lo = (gl["lower"] + 0.5) * cw
        for _ in range(20):
            k = rng.integers(0, gl["dims"] + 1)
            p = lo + k * cw
            p[rng.integers(0, 3)] += rng.uniform(0, cw)
            pts.append(p)
        pts.append((gl["lower"] + gl["dims"] + 0.5) * cw)
    if len(ds.vertices):
        pts.extend(ds.vertices[rng.integers(0, len(ds.vertices), 500), :3])
    P = np.array(pts, np.float32)
    _check_samples(g.sampler.sample_host(P), o.f.sample(P))


def test_sample_points_edge_inputs(scenes):
    ds, g, o = scenes
    P = np.array([[np.nan, 1, 1], [np.inf, 0, 0], [-1e30, 5, 5], [1e30, 1e30, 1e30], g.lo, g.hi,
                  0.5 * (g.lo + g.hi)], np.float32)
    _check_samples(g.sampler.sample_host(P), o.f.sample(P))
    assert len(g.sampler.sample_host(np.zeros((0, 3), np.float32))) == 0


def test_sample_points_device_buffers(scenes, torch_cuda):
    torch = torch_cuda
    ds, g, o = scenes
    rng = np.random.default_rng(7)
    P = rng.uniform(g.lo, g.hi, (4096, 3)).astype(np.float32)
    pd = torch.from_numpy(P).cuda()
    out = torch.zeros(4096 * 3, dtype=torch.int32, device="cuda")
    g.sampler.sample_device(pd.data_ptr(), out.data_ptr(), 4096)
    torch.cuda.synchronize()
    from owlexastitcher_gb300.exastitch import SAMPLE_DTYPE
    gs = out.cpu().numpy().view(SAMPLE_DTYPE)
    _check_samples(gs, o.f.sample(P))


def _render_pair(g, o, torch, w, h, integrator, spp, light, ext, frames=1):
    cam = orbit_camera(g.lo, g.hi, w, h)
    lp = setup_render(g.lp, cam, w, h, integrator, spp, light, ext, g.lo, g.hi)
    n = w * h
    fb = torch.zeros(n, dtype=torch.int32, device="cuda")
    acc = torch.zeros(n * 4, dtype=torch.float32, device="cuda")
    tT = torch.zeros(n, dtype=torch.float32, device="cuda")
    tTr = torch.zeros(n, dtype=torch.float32, device="cuda")
    hacc = np.zeros((n, 4), np.float32)
    for f in range(frames):
        lp.accumID = f
        lp.fbPointer, lp.accumBuffer = fb.data_ptr(), acc.data_ptr()
        lp.ext.traceT, lp.ext.traceTr = tT.data_ptr(), tTr.data_ptr()
        from owlexastitcher_gb300 import exastitch as E
        E._check(E.lib().exa_render(g.ctx.h, E.C.byref(lp), w, h))
        hl, hfb, hacc, htT, htTr = host_lp(lp, o, w, h, accum=hacc)
        assert o.f.render(bytes(hl), w, h) == 0
    g.ctx.sync()
    return (fb.cpu().numpy().view(np.uint32), acc.cpu().numpy().reshape(-1, 4), tT.cpu().numpy(), tTr.cpu().numpy(),
            hfb, hacc, htT, htTr)


@pytest.mark.parametrize("integrator,spp,light,ext", [
    (1, 1, "directional", False),   # single scatter, the small config's primary-ray workload
    (1, 2, "point", False),
    (0, 2, "point", False),         # path tracer, reference defaults
    (0, 2, "directional", True),    # path tracer, albedo 0.8 / HG 0.3 / 8 bounces
    (0, 1, "none", False),          # ambient (no light)
])
@pytest.mark.parametrize("path", ["wavefront", "single_launch", "auto"])
def test_render_bit_exact(scenes, torch_cuda, integrator, spp, light, ext, path):
    """Both renderers of exa_render (and the automatic choice, which takes
    the single launch for a frame this small) against the oracle."""
    ds, g, o = scenes
    from owlexastitcher_gb300 import exastitch as E
    w, h = 48, 40
    g.ctx.set_render_path({"wavefront": E.RENDER_PATH_WAVEFRONT, "single_launch": E.RENDER_PATH_SINGLE_LAUNCH,
                           "auto": E.RENDER_PATH_AUTO}[path])
    try:
        fb, acc, tT, tTr, hfb, hacc, htT, htTr = _render_pair(g, o, torch_cuda, w, h, integrator, spp, light, ext)
        st = g.ctx.render_stats()
    finally:
        g.ctx.set_render_path(E.RENDER_PATH_WAVEFRONT)
    assert st["wavefront"] == (1 if path == "wavefront" else 0)
    assert np.array_equal(fb, hfb)
    assert acc.tobytes() == hacc.tobytes()
    assert tT.tobytes() == htT.tobytes()      # per-ray free-flight distance
    assert tTr.tobytes() == htTr.tobytes()    # per-ray shadow transmittance
    assert (tT > 0).sum() > 0                 # some rays interact
    assert len(np.unique(fb)) > 4


def test_progressive_accumulation(scenes, torch_cuda):
    ds, g, o = scenes
    fb, acc, tT, tTr, hfb, hacc, htT, htTr = _render_pair(g, o, torch_cuda, 32, 24, 0, 1, "directional", True,
                                                          frames=3)
    assert np.array_equal(fb, hfb)
    assert acc.tobytes() == hacc.tobytes()


def test_gridlet_shade_mode(scenes, torch_cuda):
    ds, g, o = scenes
    g.lp.shadeMode = 1
    try:
        fb, acc, tT, tTr, hfb, hacc, htT, htTr = _render_pair(g, o, torch_cuda, 32, 32, 1, 1, "directional", False)
    finally:
        g.lp.shadeMode = 0
    assert np.array_equal(fb, hfb)


def test_render_axis_parallel_rays(scenes, torch_cuda):
    """A directional light along (0.4, 0.8, 0): every shadow ray's z
    component is exactly 0, so the DDA never crosses a z plane.  Bit-exact
    with the oracle and no device iteration cap raised.  (Camera rays cannot
    test this: generateRay lifts components below 1e-5.)"""
    ds, g, o = scenes
    from owlexastitcher_gb300 import exastitch as E
    w, h = 40, 32
    cam = orbit_camera(g.lo, g.hi, w, h)
    lp = setup_render(g.lp, cam, w, h, 0, 2, "directional", True, g.lo, g.hi)
    lp.lights[0].pos = E._v3([0.4, 0.8, 0.0])
    n = w * h
    fb = torch_cuda.zeros(n, dtype=torch_cuda.int32, device="cuda")
    acc = torch_cuda.zeros(n * 4, dtype=torch_cuda.float32, device="cuda")
    lp.accumID = 0
    lp.fbPointer, lp.accumBuffer = fb.data_ptr(), acc.data_ptr()
    lp.ext.traceT = lp.ext.traceTr = None
    try:
        E._check(E.lib().exa_render(g.ctx.h, E.C.byref(lp), w, h))
        g.ctx.sync()
        assert g.ctx.device_errors() == 0
        hl, hfb, hacc, htT, htTr = host_lp(lp, o, w, h)
        assert o.f.render(bytes(hl), w, h) == 0
        assert acc.cpu().numpy().reshape(-1, 4).tobytes() == hacc.tobytes()
    finally:
        lp.lights[0].pos = E._v3([0.4, 0.8, 0.45])


@pytest.mark.parametrize("light,dt", [("none", 0.5), ("point", 0.25), ("directional", 1.0)])
def test_render_ray_marching_bit_exact(scenes, torch_cuda, light, dt):
    """The ray-marching integrator (RAY_MARCHING_INTEGRATOR, deviceCode.cu:
    348-398, 1213-1260): compositing at spacing render.dt from a jittered
    first sample, early exit at opacity 0.99."""
    ds, g, o = scenes
    w, h = 40, 32
    cam = orbit_camera(g.lo, g.hi, w, h)
    lp = setup_render(g.lp, cam, w, h, 2, 2, light, False, g.lo, g.hi)
    lp.render.dt = dt
    try:
        fb, acc, tT, tTr, hfb, hacc, htT, htTr = _render_pair(g, o, torch_cuda, w, h, 2, 2, light, False)
    finally:
        g.lp.render.dt = 1.0
    assert np.array_equal(fb, hfb)
    assert acc.tobytes() == hacc.tobytes()
    assert len(np.unique(fb)) > 4


@pytest.mark.parametrize("integrator,flip", [(0, False), (0, True), (1, False), (2, True)])
def test_render_clip_plane_bit_exact(scenes, torch_cuda, integrator, flip):
    """A clip plane through the volume's centre (deviceCode.cu:53-60 and the
    integrators' clipping after the box test), for both orientations."""
    ds, g, o = scenes
    w, h = 40, 32
    c = 0.5 * (g.lo + g.hi)
    n = np.array([0.6, 0.1, 0.8], np.float32)
    n /= np.linalg.norm(n)
    if flip:
        n = -n
    g.lp.clipPlanes[0].enabled = 1
    g.lp.clipPlanes[0].N = tuple_to_v3(n)
    g.lp.clipPlanes[0].d = float(np.dot(n, c))
    try:
        fb, acc, tT, tTr, hfb, hacc, htT, htTr = _render_pair(g, o, torch_cuda, w, h, integrator, 2, "point",
                                                              integrator == 0)
    finally:
        g.lp.clipPlanes[0].enabled = 0
    assert np.array_equal(fb, hfb)
    assert acc.tobytes() == hacc.tobytes()
    assert len(np.unique(fb)) > 4


def tuple_to_v3(v):
    from owlexastitcher_gb300 import exastitch as E
    return E._v3(v)


def mesh_scene(lo, hi, rings=10, segs=16):
    """A UV sphere inside the volume and a ground quad that reaches past its
    bounds (so it extends the world bounds): float3 vertices, int3 triangles."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    ext = hi - lo
    c = lo + ext * np.array([0.55, 0.45, 0.5])
    r = 0.22 * ext.min()
    verts, tris = [], []
    for i in range(rings + 1):
        th = np.pi * i / rings
        for j in range(segs):
            ph = 2 * np.pi * j / segs
            verts.append(c + r * np.array([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)]))
    for i in range(rings):
        for j in range(segs):
            a, b = i * segs + j, i * segs + (j + 1) % segs
            tris += [(a, a + segs, b), (b, a + segs, b + segs)]
    z = lo[2] + 0.2 * ext[2]
    base = len(verts)
    verts += [(lo[0] - 0.3 * ext[0], lo[1] - 0.3 * ext[1], z), (hi[0] + 0.3 * ext[0], lo[1] - 0.3 * ext[1], z),
              (hi[0] + 0.3 * ext[0], hi[1] + 0.3 * ext[1], z), (lo[0] - 0.3 * ext[0], hi[1] + 0.3 * ext[1], z)]
    tris += [(base, base + 1, base + 2), (base, base + 2, base + 3)]
    return np.array(verts, np.float32), np.array(tris, np.int32)


@pytest.mark.parametrize("integrator,spp,light,ext", [
    (0, 2, "point", True),         # path tracer: Lambertian bounces off the surfaces
    (0, 1, "none", False),         # path tracer, ambient light
    (1, 2, "directional", False),  # direct light: shadow rays that end on a surface
    (1, 1, "none", False),         # direct light without lights: headlight shading
    (2, 2, "point", False),        # ray marcher: the surface ends the march
])
def test_render_mesh_bit_exact(scenes, torch_cuda, integrator, spp, light, ext):
    """Surface meshes (MeshGeomCH and the integrators' mesh tests,
    deviceCode.cu:295-318, 897-925, 1032-1087, 1165-1198, 1243-1251): the
    BVH closest hit on the GPU against the oracle's brute force."""
    ds, g, o = scenes
    from owlexastitcher_gb300 import exastitch as E
    v, t = mesh_scene(g.lo, g.hi)
    E.set_mesh(g.ctx, v, t)
    g.sampler.setLPs(g.lp)
    o.f.set_mesh(v, t)
    mlo, mhi = E.mesh_bounds(g.ctx)
    assert np.array_equal(mlo, v[t.ravel()].min(0)) and np.array_equal(mhi, v[t.ravel()].max(0))
    wb = g.lp.worldSpaceBounds
    assert wb.lower.x == min(mlo[0], g.model.getBounds()[0][0]) and wb.lower.z == min(mlo[2], g.lo[2])
    assert g.lp.meshBVH != 0
    try:
        w, h = 40, 32
        fb, acc, tT, tTr, hfb, hacc, htT, htTr = _render_pair(g, o, torch_cuda, w, h, integrator, spp, light, ext)
        assert g.ctx.device_errors() == 0
    finally:
        E.set_mesh(g.ctx, np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32))
        g.sampler.setLPs(g.lp)
        o.f.set_mesh(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32))
    assert g.lp.meshBVH == 0
    assert np.array_equal(fb, hfb)
    assert acc.tobytes() == hacc.tobytes()
    assert tT.tobytes() == htT.tobytes()
    assert tTr.tobytes() == htTr.tobytes()
    assert len(np.unique(fb)) > 4


def test_mesh_rejected_where_unsupported(scenes, torch_cuda):
    """lp.meshBVH must be this context's mesh; the batched and no-allocation
    entry points reject meshes."""
    ds, g, o = scenes
    from owlexastitcher_gb300 import exastitch as E
    w, h = 16, 16
    cam = orbit_camera(g.lo, g.hi, w, h)
    lp = setup_render(g.lp, cam, w, h, 1, 1, "none", False, g.lo, g.hi)
    fb = torch_cuda.zeros(w * h, dtype=torch_cuda.int32, device="cuda")
    acc = torch_cuda.zeros(w * h * 4, dtype=torch_cuda.float32, device="cuda")
    lp.fbPointer, lp.accumBuffer = fb.data_ptr(), acc.data_ptr()
    lp.ext.traceT = lp.ext.traceTr = None
    lp.meshBVH = 16  # not a mesh of this context
    try:
        assert E.lib().exa_render(g.ctx.h, E.C.byref(lp), w, h) == E.EXA_ERR_INVALID
        assert b"meshBVH" in E.lib().exa_last_error()
        v, t = mesh_scene(g.lo, g.hi, 4, 6)
        E.set_mesh(g.ctx, v, t)
        g.sampler.setLPs(lp)
        assert E.lib().exa_render_noalloc(g.ctx.h, E.C.byref(lp), w, h) == E.EXA_ERR_INVALID
        with pytest.raises(E.ExaError, match="broken triangle model"):
            E.set_mesh(g.ctx, v, t + len(v))
    finally:
        E.set_mesh(g.ctx, np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32))
        g.sampler.setLPs(g.lp)
    assert g.lp.meshBVH == 0


@pytest.mark.parametrize("feature,integrator", [
    ("subimage", 0), ("subimage", 1), ("subimage", 2),
    ("selecting", 1),
    ("teaser", 0), ("teaser", 1),
    ("heatmap", 0), ("heatmap", 1), ("heatmap", 2),
])
def test_render_features_bit_exact(scenes, torch_cuda, feature, integrator):
    """The sub-image window and its selection border (deviceCode.cu:114-142,
    1286-1294, 1337-1342), the Teaser shade mode (:652-695) and the heat map
    (:155-177, 1323-1327; here the pixel's walk DDA cells or march positions
    stand in for its clock cycles)."""
    ds, g, o = scenes
    lp = g.lp
    if feature == "subimage":
        lp.subImage.active = 1
        lp.subImage.value.lower.x, lp.subImage.value.lower.y = 0.25, 0.3
        lp.subImage.value.upper.x, lp.subImage.value.upper.y = 0.7, 0.85
    elif feature == "selecting":
        lp.subImage.selecting = 1
        lp.subImage.selection.lower.x, lp.subImage.selection.lower.y = 0.2, 0.25
        lp.subImage.selection.upper.x, lp.subImage.selection.upper.y = 0.8, 0.6
    elif feature == "teaser":
        lp.shadeMode = 2
    else:
        lp.render.heatMapEnabled = 1
        lp.render.heatMapScale = 0.02
    lp.render.dt = 0.5
    try:
        fb, acc, tT, tTr, hfb, hacc, htT, htTr = _render_pair(g, o, torch_cuda, 40, 32, integrator, 2, "point",
                                                              integrator == 0, frames=2)
    finally:
        lp.subImage.active = lp.subImage.selecting = 0
        lp.shadeMode = 0
        lp.render.heatMapEnabled = 0
        lp.render.dt = 1.0
    assert np.array_equal(fb, hfb)
    assert acc.tobytes() == hacc.tobytes()
    assert tT.tobytes() == htT.tobytes()
    assert len(np.unique(fb)) > 4


@pytest.mark.parametrize("integrator", [0, 1])
def test_row_bands_equal_whole_frame(scenes, torch_cuda, integrator):
    """exa_lp_ext.rowBegin / rowEnd (a frame split across GPUs): each band's
    pixels equal the whole frame's bit for bit, the other rows untouched;
    bands are rejected where they are not supported."""
    torch = torch_cuda
    ds, g, o = scenes
    from owlexastitcher_gb300 import exastitch as E
    w, h = 40, 30
    lp = setup_render(g.lp, orbit_camera(g.lo, g.hi, w, h), w, h, integrator, 2, "point", integrator == 0, g.lo, g.hi)
    lp.ext.traceT = lp.ext.traceTr = None
    lp.accumID = 0

    def render(rows):
        fb = torch.full((w * h,), 7, dtype=torch.int32, device="cuda")
        acc = torch.full((w * h * 4,), -1.0, dtype=torch.float32, device="cuda")
        lp.fbPointer, lp.accumBuffer = fb.data_ptr(), acc.data_ptr()
        lp.ext.rowBegin, lp.ext.rowEnd = rows
        try:
            E._check(E.lib().exa_render(g.ctx.h, E.C.byref(lp), w, h))
            g.ctx.sync()
        finally:
            lp.ext.rowBegin = lp.ext.rowEnd = 0
        return fb.cpu().numpy(), acc.cpu().numpy().reshape(-1, 4)

    fb, acc = render((0, 0))
    for b, e in ((0, 8), (8, 24), (24, 30)):
        bfb, bacc = render((b, e))
        assert np.array_equal(bfb[b * w:e * w], fb[b * w:e * w])
        assert bacc[b * w:e * w].tobytes() == acc[b * w:e * w].tobytes()
        assert np.all(bfb[:b * w] == 7) and np.all(bfb[e * w:] == 7)
        assert np.all(bacc[:b * w] == -1.0) and np.all(bacc[e * w:] == -1.0)
    for bad in ((4, 16), (8, 8), (0, 31), (16, 20)):
        lp.ext.rowBegin, lp.ext.rowEnd = bad
        try:
            assert E.lib().exa_render(g.ctx.h, E.C.byref(lp), w, h) == E.EXA_ERR_INVALID, bad
        finally:
            lp.ext.rowBegin = lp.ext.rowEnd = 0


def test_progressive_checkpoint_resume(scenes, torch_cuda, tmp_path):
    """Renderer.checkpoint / restore: a progressive render saved after two
    frames and continued in a new context equals four frames in one go, bit
    for bit (the accumulation buffer and accumID are its whole state)."""
    torch = torch_cuda
    ds, g, o = scenes
    from owlexastitcher_gb300 import exastitch as E
    w, h = 32, 24

    def renderer():
        ctx = E.Context(0)
        r = E.Renderer(ctx, E.ExaStitchModel.from_dataset(ctx, ds), g.num_mcs)
        r.setColorMap(g.tf)
        r.resize(w, h)
        r.spp = 2
        lo, hi = r.model.cellBounds
        setup_render(r.lp, orbit_camera(lo, hi, w, h), w, h, E.PATH_TRACING_INTEGRATOR, 2, "directional", True)
        r.lp.ext.traceT = r.lp.ext.traceTr = None
        return ctx, r

    ctx, full = renderer()
    for _ in range(4):
        full.render()
    ctx.sync()
    want_acc, want_fb = full.accum.cpu().numpy(), full.fb.cpu().numpy()
    ctx.close()
    ctx, part = renderer()
    for _ in range(2):
        part.render()
    ctx.sync()
    part.checkpoint(tmp_path / "progress.npz")
    ctx.close()
    ctx, resumed = renderer()
    resumed.restore(tmp_path / "progress.npz")
    assert resumed.accumID == 2
    for _ in range(2):
        resumed.render()
    ctx.sync()
    assert resumed.accum.cpu().numpy().tobytes() == want_acc.tobytes()
    assert np.array_equal(resumed.fb.cpu().numpy(), want_fb)
    ctx.close()
