"""Stitching elements on the CUDA path against the golden vectors that the
reference's own headers produced (tests/golden/elements.npz, made by
tests/golden/make_golden.py from Plane.h:57-99 intersectTet with its
`fa > 1` tests at :89,92,95, and UElems.h intersectPyrEXT / intersectWedgeEXT /
intersectHexEXT).

Each element type's 400 golden elements form one element-only model; every
golden point is sampled through exa_sample_points_host.  Where the point lies
in no other element of the model (the oracle's list of every containing
primitive decides), the GPU's answer must be the golden one: the hit flag,
the element id and the value's bits.  A quarter of the points sit on a
vertex or an edge midpoint (boundary cases of the inside tests).

Degenerate elements (flattened, collapsed, twisted) sample as the oracle,
whose answers on them equal the reference headers' (test_oracle_ref.py), and
frames over overlapping collapsed tets, whose samples carry NaN values, render
bit for bit as the oracle under both transfer-function filters."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def element_model(V):
    """vertices (x, y, z, value) and 8-wide -1 padded index rows of n
    elements with nv vertices each"""
    n, nv, _ = V.shape
    verts = np.ascontiguousarray(V.reshape(-1, 4), np.float32)
    idx = -np.ones((n, 8), np.int32)
    idx[:, :nv] = np.arange(n * nv, dtype=np.int32).reshape(n, nv)
    return verts, idx


def degenerate_elements(rng, nv, n):
    """n elements with nv vertices, by turns flattened along an axis (to
    1e-4..1e-2 of their size), perturbed with two vertices then collapsed
    (a tet becomes a triangle whose inside test passes off its plane with NaN
    weights, as Plane.h's does), strongly twisted,
    or mildly perturbed, each in its own cell of a 40-unit lattice (so no two
    overlap), and per element three points: one uniform over its bounds
    widened by 5 %, its vertex mean and one of its vertices"""
    from golden.make_golden import SHAPES
    base = SHAPES[nv]
    V = np.zeros((n, nv, 4), np.float32)
    P = np.zeros((n, 3, 3), np.float32)
    for i in range(n):
        B = base.copy()
        kind = i % 4
        if kind == 0:
            B[:, rng.integers(0, 3)] *= rng.uniform(1e-4, 1e-2)
        elif kind == 1:  # in a general orientation, so that its box is not flat
            B = B + rng.normal(0, 0.3, B.shape)
            a, b = rng.choice(nv, 2, replace=False)
            B[b] = B[a]
        elif kind == 2:
            B = B + rng.normal(0, 0.4, B.shape)
        else:
            B = B + rng.normal(0, 0.08, B.shape)
        cell = np.array([i % 16, (i // 16) % 16, i // 256], np.float32) * 40
        V[i, :, :3] = B * rng.uniform(0.5, 8) + cell
        V[i, :, 3] = rng.uniform(-1, 1, nv)
        lo, hi = V[i, :, :3].min(0), V[i, :, :3].max(0)
        P[i, 0] = rng.uniform(lo - 0.05 * (hi - lo), hi + 0.05 * (hi - lo))
        P[i, 1] = V[i, :, :3].mean(0)
        P[i, 2] = V[i, rng.integers(0, nv), :3]
    return V, P


@pytest.mark.gpu
@pytest.mark.parametrize("nv", [4, 5, 6, 8], ids=["tet", "pyramid", "wedge", "hex"])
def test_degenerate_elements_on_gpu(cuda, native, oracle, nv):
    """flattened, collapsed and twisted elements (where the Newton inversion
    may stop at its iteration cap) sample bit for bit as the oracle, which
    equals the reference's headers on them (test_oracle_ref.py)"""
    from owlexastitcher_gb300 import exastitch as E
    V, P = degenerate_elements(np.random.default_rng(31), nv, 1024)
    P = P.reshape(-1, 3)
    verts, idx = element_model(V)
    ctx = E.Context(0)
    model = E.ExaStitchModel(ctx, verts, idx, np.zeros(0, E.GRIDLET_DTYPE), np.zeros(0, np.float32))
    model.setNumGridCells((16, 16, 8))
    sampler = E.ExaStitchSampler(ctx)
    sampler.build(model)
    got = sampler.sample_host(P)
    assert ctx.device_errors() == 0
    ctx.close()
    want = oracle.Field(verts, idx, np.zeros(0, oracle.GRIDLET_DTYPE), np.zeros(0, np.float32)).sample(P)
    assert np.array_equal(got["primID"], want["primID"]) and np.array_equal(got["cellID"], want["cellID"])
    # tets with two collapsed vertices hit with NaN values (as Plane.h's test
    # does); a NaN's bits are the host's or the GPU's default NaN, so NaNs
    # compare as NaN and every other value bit for bit
    nan = np.isnan(want["value"])
    assert np.array_equal(np.isnan(got["value"]), nan)
    assert got["value"][~nan].tobytes() == want["value"][~nan].tobytes()
    hit = want["primID"] >= 0
    assert hit.sum() > 200 and np.all(want["primID"][hit] == np.nonzero(hit)[0] // 3)
    assert (nan & hit).any() == (nv == 4)


def collapsed_scene(rng, side=4, spacing=6.0, size=10.0):
    """side^3 overlapping tets of about `size` on a lattice of `spacing`,
    every other one perturbed and then collapsed to a triangle: about half
    of the hits in the scene's box carry NaN values"""
    from golden.make_golden import SHAPES
    n = side ** 3
    V = np.zeros((n, 4, 4), np.float32)
    for i in range(n):
        B = SHAPES[4] + rng.normal(0, 0.3, (4, 3))
        if i % 2 == 0:
            a, b = rng.choice(4, 2, replace=False)
            B[b] = B[a]
        cell = np.array([i % side, (i // side) % side, i // side ** 2], np.float32) * spacing
        V[i, :, :3] = B * size + cell
        V[i, :, 3] = rng.uniform(-1, 1, 4)
    return V


@pytest.mark.gpu
@pytest.mark.parametrize("tf_filter", [0, 1], ids=["nearest", "linear"])
@pytest.mark.parametrize("integrator,light,ext", [(0, "directional", True), (1, "point", False), (2, "none", False)])
def test_collapsed_tets_render_bit_exact(cuda, native, oracle, tf_filter, integrator, light, ext):
    """frames over overlapping tets, half of them collapsed: their samples
    carry NaN values, which the nearest transfer-function lookup clamps to
    its last entry and the linear one maps to the zero border; the domain
    ends past the largest value, so under the nearest filter only NaN samples
    take the last entry (the oracle's frame changes with it); all three
    integrators render bit for bit as the oracle"""
    import ctypes as C
    import types

    from helpers import GpuScene, OracleScene, host_lp, orbit_camera, ramp_tf, setup_render
    from owlexastitcher_gb300 import exastitch as E
    verts, idx = element_model(collapsed_scene(np.random.default_rng(5)))
    ds = types.SimpleNamespace(vertices=verts, indices=idx, gridlets=np.zeros(0, E.GRIDLET_DTYPE),
                               gridlet_scalars=np.zeros(0, np.float32))
    dims = (8, 8, 8)
    g = GpuScene(ds, dims, tf=ramp_tf())
    vmin, vmax = g.xf
    g.xf = (vmin, np.float32(vmax + (vmax - vmin) / 8))
    if tf_filter:
        g.ctx.set_tf_filter(E.TF_FILTER_LINEAR)
    g.sampler.computeMaxOpacities(g.tf, g.xf)
    g.sampler.setLPs(g.lp)
    o = OracleScene(oracle, ds, dims, g.lo, g.hi, g.tf, g.xf, tf_filter=tf_filter)
    w, h = 48, 32
    lp = setup_render(g.lp, orbit_camera(g.lo, g.hi, w, h), w, h, integrator, 2, light, ext, g.lo, g.hi)
    n = w * h
    fb = cuda.zeros(n, dtype=cuda.int32, device="cuda")
    acc = cuda.zeros(n * 4, dtype=cuda.float32, device="cuda")
    lp.accumID = 0
    lp.fbPointer, lp.accumBuffer = fb.data_ptr(), acc.data_ptr()
    lp.ext.traceT = lp.ext.traceTr = None
    E._check(E.lib().exa_render(g.ctx.h, C.byref(lp), w, h))
    g.ctx.sync()
    assert g.ctx.device_errors() == 0
    hl, hfb, hacc, _, _ = host_lp(lp, o, w, h)
    assert o.f.render(bytes(hl), w, h) == 0
    assert acc.cpu().numpy().reshape(-1, 4).tobytes() == hacc.tobytes()
    assert np.array_equal(fb.cpu().numpy().view(np.uint32), hfb)
    assert len(np.unique(hfb)) > 100
    if tf_filter == 0:
        tf0 = g.tf.copy()
        tf0[-1] = 0.0
        o0 = OracleScene(oracle, ds, dims, g.lo, g.hi, tf0, g.xf)
        hl0, _, hacc0, _, _ = host_lp(lp, o0, w, h)
        assert o0.f.render(bytes(hl0), w, h) == 0
        assert np.count_nonzero(np.any(hacc0 != hacc, axis=1)) > 50
    g.ctx.close()


@pytest.mark.gpu
def test_rows_without_an_element_type(cuda, native, oracle):
    """index rows of 0, 1, 2, 3 and 7 vertices name no element type
    (programs/ExaStitchSampler.cu:145-148 tests 4, 5, 6 and 8 only): they
    overlap a hex and are never hit, and the points sample bit for bit as
    the oracle; a row with a vertex after its -1 padding is rejected"""
    from owlexastitcher_gb300 import exastitch as E
    hexv = np.array([[0, 0, 0], [4, 0, 0], [4, 4, 0], [0, 4, 0], [0, 0, 4], [4, 0, 4], [4, 4, 4], [0, 4, 4]],
                    np.float32)
    rng = np.random.default_rng(8)
    extra = rng.uniform(-1, 5, (24, 3)).astype(np.float32)
    verts = np.zeros((8 + len(extra), 4), np.float32)
    verts[:8, :3], verts[8:, :3] = hexv, extra
    verts[:, 3] = rng.uniform(-1, 1, len(verts))
    idx = -np.ones((6, 8), np.int32)
    for r, count in enumerate((0, 1, 2, 3, 7)):  # the short rows come first: lower indices
        idx[r, :count] = 8 + rng.choice(len(extra), count, replace=False)
    idx[5] = np.arange(8)
    P = rng.uniform(-0.5, 4.5, (20000, 3)).astype(np.float32)
    ctx = E.Context(0)
    model = E.ExaStitchModel(ctx, verts, idx, np.zeros(0, E.GRIDLET_DTYPE), np.zeros(0, np.float32))
    model.setNumGridCells((4, 4, 4))
    sampler = E.ExaStitchSampler(ctx)
    sampler.build(model)
    got = sampler.sample_host(P)
    assert ctx.device_errors() == 0
    want = oracle.Field(verts, idx, np.zeros(0, oracle.GRIDLET_DTYPE), np.zeros(0, np.float32)).sample(P)
    assert got.tobytes() == want.tobytes()
    hit = got["primID"] >= 0
    assert hit.mean() > 0.4 and np.all(got["primID"][hit] == 5)
    gap = idx.copy()
    gap[5, 3] = -1  # a hex row with a hole
    with pytest.raises(E.ExaError):
        E.ExaStitchModel(ctx, verts, gap, np.zeros(0, E.GRIDLET_DTYPE), np.zeros(0, np.float32))
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("nv", [4, 5, 6, 8], ids=["tet", "pyramid", "wedge", "hex"])
def test_elements_golden_on_gpu(cuda, native, oracle, nv):
    from owlexastitcher_gb300 import exastitch as E
    g = np.load(os.path.join(GOLD, "elements.npz"))
    V, P, hit, val = g[f"V_{nv}"], g[f"P_{nv}"], g[f"hit_{nv}"], g[f"val_{nv}"]
    verts, idx = element_model(V)
    ctx = E.Context(0)
    model = E.ExaStitchModel(ctx, verts, idx, np.zeros(0, E.GRIDLET_DTYPE), np.zeros(0, np.float32))
    model.setNumGridCells((8, 8, 8))
    sampler = E.ExaStitchSampler(ctx)
    sampler.build(model)
    got = sampler.sample_host(P)
    assert ctx.device_errors() == 0
    f = oracle.Field(verts, idx, np.zeros(0, oracle.GRIDLET_DTYPE), np.zeros(0, np.float32))
    checked = hits = 0
    for i in range(len(P)):
        others = [pid for kind, pid, _ in f.sample_all(P[i]) if pid != i]
        if others:
            continue  # another golden element contains the point as well
        checked += 1
        if hit[i]:
            hits += 1
            assert got["primID"][i] == i and got["cellID"][i] == -1, i
            assert got["value"][i:i + 1].tobytes() == val[i:i + 1].tobytes(), (i, got["value"][i], val[i])
        else:
            assert got["primID"][i] < 0, i
    assert checked >= 0.95 * len(P)
    assert hits > 20
    ctx.close()


@pytest.mark.gpu
def test_tets_in_unbalanced_dataset_sampled(cuda, native, oracle):
    """The unbalanced small dataset's dual mesh holds tetrahedra: points at
    their centroids (and at their vertices) sample bit-exact with the oracle
    and mostly report a tet."""
    from conftest import dataset
    from owlexastitcher_gb300 import exastitch as E
    ds = dataset("small", balance=0)
    nvs = np.count_nonzero(ds.indices >= 0, axis=1)
    tets = np.nonzero(nvs == 4)[0]
    assert len(tets) > 1000
    corners = ds.vertices[ds.indices[tets, :4]][:, :, :3]
    P = np.concatenate([corners.mean(axis=1), corners[:, 0]]).astype(np.float32)
    ctx = E.Context(0)
    model = E.ExaStitchModel.from_dataset(ctx, ds)
    model.setNumGridCells((32, 32, 32))
    sampler = E.ExaStitchSampler(ctx)
    sampler.build(model)
    got = sampler.sample_host(P)
    want = oracle.Field(ds.vertices, ds.indices, ds.gridlets, ds.gridlet_scalars).sample(P)
    assert np.array_equal(got["primID"], want["primID"]) and np.array_equal(got["cellID"], want["cellID"])
    assert got["value"].tobytes() == want["value"].tobytes()
    centroid = got[: len(tets)]
    is_tet = (centroid["cellID"] == -1) & (centroid["primID"] >= 0)
    is_tet[is_tet] = nvs[centroid["primID"][is_tet]] == 4
    assert is_tet.mean() > 0.5
    ctx.close()


def test_element_box_bounds_the_tolerance(oracle):
    """The hex test accepts points up to 1e-6 outside the element in its
    parametric coordinates (UElems.h), so it reports a hit just above the
    top face; the element's bounding box (its bounds program,
    programs/ExaStitchSampler.cu:73-92) does not hold that point, so OptiX
    never calls the test there.  The oracle's sampler keeps that rule."""
    V = np.array([[0, 0, 0, 1], [1, 0, 0, 2], [1, 1, 0, 3], [0, 1, 0, 4], [0, 0, 1, 5], [1, 0, 1, 6], [1, 1, 1, 7],
                  [0, 1, 1, 8]], np.float32)
    P = np.array([[0.5, 0.5, 1 + 5e-7], [0.5, 0.5, 1.0], [0.25, 0.5, 0.75]], np.float32)
    assert P[0, 2] > 1 and oracle.intersect_elem(P[0], V)[0]  # the tolerance accepts it
    verts, idx = element_model(V[None])
    f = oracle.Field(verts, idx, np.zeros(0, oracle.GRIDLET_DTYPE), np.zeros(0, np.float32))
    s = f.sample(P)
    assert list(s["primID"]) == [-1, 0, 0]
    assert [k for k, _, _ in f.sample_all(P[0])] == []


@pytest.mark.gpu
def test_element_box_bounds_the_tolerance_gpu(cuda, native, oracle):
    from owlexastitcher_gb300 import exastitch as E
    V = np.array([[0, 0, 0, 1], [1, 0, 0, 2], [1, 1, 0, 3], [0, 1, 0, 4], [0, 0, 1, 5], [1, 0, 1, 6], [1, 1, 1, 7],
                  [0, 1, 1, 8]], np.float32)
    P = np.array([[0.5, 0.5, 1 + 5e-7], [0.5, 0.5, 1.0], [0.25, 0.5, 0.75]], np.float32)
    verts, idx = element_model(V[None])
    ctx = E.Context(0)
    model = E.ExaStitchModel(ctx, verts, idx, np.zeros(0, E.GRIDLET_DTYPE), np.zeros(0, np.float32))
    model.setNumGridCells((2, 2, 2))
    sampler = E.ExaStitchSampler(ctx)
    sampler.build(model)
    got = sampler.sample_host(P)
    want = oracle.Field(verts, idx, np.zeros(0, oracle.GRIDLET_DTYPE), np.zeros(0, np.float32)).sample(P)
    assert list(got["primID"]) == [-1, 0, 0]
    assert got.tobytes() == want.tobytes()
    ctx.close()
