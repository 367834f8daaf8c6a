"""Known-answer tests of the oracle's interpolation and tracking: linear
fields are reproduced by every cell type, and Woodcock tracking through a
homogeneous medium scatters with probability 1 - exp(-sigma*d)."""
import ctypes as C

import numpy as np
import pytest

from golden.make_golden import SHAPES


def lin(p):
    return 0.3 + 0.2 * p[..., 0] - 0.1 * p[..., 1] + 0.05 * p[..., 2]


@pytest.mark.parametrize("nv", [4, 5, 6, 8])
def test_linear_field_elements(oracle, nv):
    """Tets are exact to rounding; pyramids/wedges/hexes to the Newton
    convergence tolerance of UElems.h (|delta| < 1e-4 in parametric space),
    and Newton may give up on a point inside (the reference's behaviour)."""
    rng = np.random.default_rng(nv)
    misses = 0
    for _ in range(300):
        V = np.zeros((nv, 4), np.float32)
        V[:, :3] = (SHAPES[nv] + rng.normal(0, 0.03, SHAPES[nv].shape)) * 2.0 + 10
        V[:, 3] = lin(V[:, :3])
        w = rng.dirichlet(np.ones(nv))
        P = (w[:, None] * V[:, :3]).sum(0).astype(np.float32)   # inside the element
        h, v = oracle.intersect_elem(P, V)
        if not h:
            misses += 1
            continue
        assert abs(v - lin(P)) < (1e-6 if nv == 4 else 1e-4)
    assert misses <= (0 if nv == 4 else 3)


def test_linear_field_gridlet(oracle):
    g = np.zeros(1, oracle.GRIDLET_DTYPE)
    g["lower"], g["level"], g["dims"], g["begin"] = (3, 4, 5), 1, (4, 3, 2), 0
    idx = np.stack(np.meshgrid(np.arange(5), np.arange(4), np.arange(3), indexing="ij"), -1)
    pos = ((idx + g["lower"][0]) + 0.5) * 2.0
    sc = lin(pos).transpose(2, 1, 0).reshape(-1).astype(np.float32)  # x fastest
    rng = np.random.default_rng(3)
    lo, hi = (g["lower"][0] + 0.5) * 2, (g["lower"][0] + g["dims"][0] + 0.5) * 2
    for P in rng.uniform(lo, hi, (300, 3)).astype(np.float32):
        h, v, c = oracle.intersect_gridlet(P, g[0], sc)
        assert h and abs(v - lin(P)) < 2e-6


def test_homogeneous_medium_scatter_probability(oracle, native):
    """One 8^3 gridlet of constant value; alpha = 0.05 everywhere; rays
    along +x across the full 8-unit slab: P(scatter) = 1 - exp(-0.05*8)."""
    from helpers import host_lp
    from owlexastitcher_gb300 import exastitch as E
    g = np.zeros(1, oracle.GRIDLET_DTYPE)
    g["lower"], g["level"], g["dims"], g["begin"] = (0, 0, 0), 0, (8, 8, 8), 0
    sc = np.full(9 ** 3, 0.5, np.float32)
    f = oracle.Field(np.zeros((0, 4), np.float32), np.zeros((0, 8), np.int32), g, sc)
    lo, hi, _ = f.bounds()
    tf = np.tile(np.float32([[1, 1, 1, 0.05]]), (16, 1))
    ranges = f.majorants((4, 4, 4), lo, hi)
    ops = oracle.max_opacities(ranges, tf, (0.0, 1.0))
    W, H = 64, 64
    lp = E.LaunchParams()
    E.lib().exa_launch_params_init(C.byref(lp))
    lp.integrator = 1
    lp.render.spp = 1
    lp.transferFunc.domain.lower, lp.transferFunc.domain.upper = 0.0, 1.0
    lp.transferFunc.numValues = 16
    lp.majorantGrid.dims = E.vec3i(4, 4, 4)
    lp.majorantGrid.bounds = E._box(lo, hi)
    lp.worldSpaceBounds = E._box(lo, hi)
    lp.ext.cullTransparentPrims = 0
    # orthographic-like: rays start left of the slab, direction +x, one per pixel row/col
    lp.camera.org = E._v3([-50.0, 4.5, 4.5])
    lp.camera.dir_00 = E._v3([1.0, -1e-3 * W / 2, -1e-3 * H / 2])
    lp.camera.dir_du = E._v3([0.0, 1e-3, 0.0])
    lp.camera.dir_dv = E._v3([0.0, 0.0, 1e-3])

    class O:
        pass
    o = O()
    o.f, o.tf, o.max_ops = f, tf, ops
    tot, n = 0, 0
    for frame in range(20):
        lp.accumID = frame
        hl, fb, acc, tT, tTr = host_lp(lp, o, W, H)
        f.render(bytes(hl), W, H)
        tot += (tT >= 0).sum()
        n += len(tT)
    p = tot / n
    expect = 1 - np.exp(-0.05 * (hi[0] - lo[0]))
    assert abs(p - expect) < 4 * np.sqrt(expect * (1 - expect) / n)


@pytest.mark.parametrize("zero_axes", [(2,), (1,), (0, 2)])
def test_dda_axis_parallel_ray(oracle, zero_axes):
    """A ray with direction components of exactly 0 never crosses that axis's
    planes: the walk ends at the grid's far side with those cell indices
    fixed, and visits at most one cell per crossing."""
    dims = (16, 12, 10)
    lo, hi = np.zeros(3, np.float32), np.array([16, 12, 10], np.float32)
    d = np.array([0.6, -0.5, 0.62], np.float32)
    for a in zero_axes:
        d[a] = 0.0
    d /= np.linalg.norm(d)
    for org in (np.array([7.3, 5.1, 4.4], np.float32), np.array([7.0, 6.0, 5.0], np.float32)):
        ids, t0, t1 = oracle.dda3(org, d, 0.0, 1e3, dims, lo, hi)
        assert 0 < len(ids) <= sum(dims)
        cells = np.stack([ids % dims[0], (ids // dims[0]) % dims[1], ids // (dims[0] * dims[1])], axis=1)
        start = [min(int(org[a]), dims[a] - 1) for a in range(3)]
        for a in zero_axes:
            assert np.all(cells[:, a] == start[a])
        assert np.all(np.isfinite(t0)) and np.all(np.isfinite(t1)) and np.all(t1 >= t0)


def test_mesh_headlight_shading(oracle, native):
    """A transparent volume and one quad across every ray at x = 4, facing
    the camera: the direct-light integrator without lights shades a surface
    hit by kd * max(0, -dir . Ng) (deviceCode.cu:1182-1198), kd = 0.8."""
    from helpers import host_lp
    from owlexastitcher_gb300 import exastitch as E
    g = np.zeros(1, oracle.GRIDLET_DTYPE)
    g["lower"], g["level"], g["dims"], g["begin"] = (0, 0, 0), 0, (8, 8, 8), 0
    f = oracle.Field(np.zeros((0, 4), np.float32), np.zeros((0, 8), np.int32), g, np.full(9 ** 3, 0.5, np.float32))
    lo, hi, _ = f.bounds()
    quad = np.float32([[4, -10, -10], [4, 20, -10], [4, 20, 20], [4, -10, 20]])
    f.set_mesh(quad, np.int32([[0, 2, 1], [0, 3, 2]]))   # winding: Ng = -x, towards the camera
    tf = np.tile(np.float32([[1, 1, 1, 0.0]]), (16, 1))
    ranges = f.majorants((4, 4, 4), lo, hi)
    ops = oracle.max_opacities(ranges, tf, (0.0, 1.0))
    W, H = 32, 32
    lp = E.LaunchParams()
    E.lib().exa_launch_params_init(C.byref(lp))
    lp.integrator = 1
    lp.render.spp = 1
    lp.meshBVH = 1   # any non-zero handle: the oracle traces its own mesh
    lp.transferFunc.domain.lower, lp.transferFunc.domain.upper = 0.0, 1.0
    lp.transferFunc.numValues = 16
    lp.majorantGrid.dims = E.vec3i(4, 4, 4)
    lp.majorantGrid.bounds = E._box(lo, hi)
    lp.worldSpaceBounds = E._box(lo, hi)
    lp.camera.org = E._v3([-50.0, 4.5, 4.5])
    sp = 0.05   # rays spread over y, z in 4.5 +- 0.8 at x = 0.5: all cross the volume
    lp.camera.dir_00 = E._v3([1.0, -sp * W / 2 / 50, -sp * H / 2 / 50])
    lp.camera.dir_du = E._v3([0.0, sp / 50, 0.0])
    lp.camera.dir_dv = E._v3([0.0, 0.0, sp / 50])

    class O:
        pass
    o = O()
    o.f, o.tf, o.max_ops = f, tf, ops
    hl, fb, acc, tT, tTr = host_lp(lp, o, W, H)
    f.render(bytes(hl), W, H)
    # cos = d.x / |d| for the jittered d = dir_00 + (px + rx) du + (py + ry) dv,
    # rx, ry in [0, 1): each pixel lies between the values at its corners
    px, py = np.meshgrid(np.arange(W), np.arange(H))
    corner = []
    for rx, ry in ((0.0, 0.0), (1.0, 0.0), (0.0, 1.0), (1.0, 1.0)):
        dy = (-W / 2 + px + rx) * sp / 50
        dz = (-H / 2 + py + ry) * sp / 50
        corner.append((0.8 / np.sqrt(1 + dy * dy + dz * dz)).ravel())
    lo_c = np.min(corner, 0) - 1e-6
    hi_c = np.max(corner, 0) + 1e-6
    col = acc[:, 0]
    assert np.all((col >= lo_c) & (col <= hi_c))
    assert np.array_equal(acc[:, 0], acc[:, 1]) and np.array_equal(acc[:, 0], acc[:, 2])
    assert np.all(acc[:, 3] == 1.0)


def test_f64_path_tracer_agrees_with_f32(oracle):
    """The binary64 path tracer (the converged reference of the learned
    field's image checks) against the FP32 restatement of
    pathTracingIntegrate at the same sample count, with independent random
    numbers: image means within 1 %, and the RMSE at the level of the noise
    (two FP32 images of other random streams differ by as much)."""
    from conftest import dataset
    from helpers import OracleScene, host_lp, oracle_only_lp, ramp_tf
    ds = dataset("small")
    f = oracle.Field(ds.vertices, ds.indices, ds.gridlets, ds.gridlet_scalars)
    lo, hi, vr = f.bounds()
    tf = ramp_tf()
    xf = (np.float32(vr[0]), np.float32(vr[1]))
    o = OracleScene(oracle, ds, (32, 32, 32), lo, hi, tf, xf)
    w = h = 12
    spp = 2048
    lp = oracle_only_lp(lo, hi, (32, 32, 32), tf, xf, w, h, 0, spp)
    hl, _, hacc, _, _ = host_lp(lp, o, w, h)
    assert o.f.render(bytes(hl), w, h) == 0
    a = hacc[:, :3].astype(np.float64) / spp
    hl.ext.frameID = 5
    hacc[:] = 0
    assert o.f.render(bytes(hl), w, h) == 0
    b = hacc[:, :3].astype(np.float64) / spp
    ref = o.f.render_f64(bytes(hl), w, h)
    noise = np.sqrt(np.mean((a - b) ** 2))
    assert 0 < noise < 0.05
    assert np.sqrt(np.mean((a - ref) ** 2)) < 1.5 * noise
    assert abs(a.mean() - ref.mean()) < 0.01 * ref.mean()
    assert ref.mean() > 0.1


def test_progressive_render_resumes_bit_exact(oracle, tmp_path):
    """The accumulation buffer and the next accumID are the whole state of a
    progressive render (deviceCode.cu:1329-1332): frames 0..3 in one go equal
    frames 0..1, a save of the buffer to a file, and frames 2..3 from the
    loaded copy, bit for bit."""
    from conftest import dataset
    from helpers import OracleScene, host_lp, oracle_only_lp, ramp_tf
    ds = dataset("tiny")
    f = oracle.Field(ds.vertices, ds.indices, ds.gridlets, ds.gridlet_scalars)
    lo, hi, vr = f.bounds()
    tf = ramp_tf()
    xf = (np.float32(vr[0]), np.float32(vr[1]))
    o = OracleScene(oracle, ds, (8, 8, 8), lo, hi, tf, xf)
    w, h = 16, 12

    def frames(acc, ids):
        lp = oracle_only_lp(lo, hi, (8, 8, 8), tf, xf, w, h, 0, 2)
        for a in ids:
            lp.accumID = a
            hl, fb, _, _, _ = host_lp(lp, o, w, h, accum=acc)
            assert o.f.render(bytes(hl), w, h) == 0
        return acc, fb

    full, fb_full = frames(np.zeros((w * h, 4), np.float32), range(4))
    part, _ = frames(np.zeros((w * h, 4), np.float32), range(2))
    np.save(tmp_path / "accum.npy", part)
    resumed, fb_res = frames(np.load(tmp_path / "accum.npy"), range(2, 4))
    assert resumed.tobytes() == full.tobytes() and np.array_equal(fb_res, fb_full)
    assert len(np.unique(fb_full)) > 4
