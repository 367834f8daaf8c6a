"""Majorant build edge cases (Grid.cu:134-246 with the gridlet value ranges
of sampler/ExaStitchSampler.cu:52-142) against the oracle, bit-exact, on
hand-made gridlet sets that reach every staging case of the build kernel:
full 8^3 bricks, bricks larger than a staging buffer, bricks that start off
a 16-byte boundary, a last brick that ends past the last 16-byte boundary of
the scalar buffer (the rest is loaded without the bulk copy), one that lies
entirely past it, gridlets without cells along an axis, NaN corners, signed
zeros, and macrocell windows above the shared-memory window size."""
import numpy as np
import pytest

from test_gpu_parity import same_floats

pytestmark = pytest.mark.gpu

GRIDLET_DTYPE = np.dtype([("lower", "<i4", 3), ("level", "<i4"), ("dims", "<i4", 3), ("begin", "<u4")])


def edge_model(last, seed=7):
    """gridlets (lower, level, dims) with 1-3 unused floats between bricks;
    `last` is the final gridlet, whose brick ends the scalar buffer"""
    specs = [((0, 0, 0), 0, (8, 8, 8)), ((8, 0, 0), 0, (8, 8, 8)), ((0, 8, 0), 1, (11, 9, 10)),
             ((3, 5, 2), 0, (1, 1, 1)), ((20, 3, 4), 2, (0, 3, 2)), ((1, 1, 9), 0, (5, 1, 7)),
             ((12, 2, 6), 1, (8, 8, 8)), ((2, 30, 1), 0, (8, 3, 8)), last]
    rng = np.random.default_rng(seed)
    gl = np.zeros(len(specs), GRIDLET_DTYPE)
    pos = 0
    for i, (lower, level, dims) in enumerate(specs):
        pos += int(rng.integers(1, 4))
        if i == len(specs) - 1:
            pos += (1 - pos) % 4  # the last brick starts one float past a 16-byte boundary
        gl[i] = (lower, level, dims, pos)
        pos += (dims[0] + 1) * (dims[1] + 1) * (dims[2] + 1)
    s = rng.normal(0.0, 1.0, pos).astype(np.float32)
    s[rng.random(pos) < 0.1] = np.nan
    z = rng.random(pos) < 0.05
    s[z] = np.where(rng.random(z.sum()) < 0.5, np.float32(0.0), np.float32(-0.0))
    return gl, s


CASES = [
    # the last brick is a 1^3 gridlet: 32 bytes by the bulk copy, 1 float after it
    ("bulk+tail", ((5, 5, 5), 0, (1, 1, 1))),
    # the last brick is 2 floats past the last boundary: no bulk copy at all
    ("tail-only", ((6, 6, 6), 0, (0, 0, 1))),
]
GRIDS = [(8, 8, 8), (5, 7, 3), (64, 64, 64), (97, 33, 128)]


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.parametrize("dims", GRIDS, ids=["x".join(map(str, d)) for d in GRIDS])
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_majorant_build_edges(cuda, native, oracle, case, dims):
    from owlexastitcher_gb300 import exastitch as E
    gl, s = edge_model(case[1])
    assert len(s) % 4 != 0
    verts = np.zeros((0, 4), np.float32)
    idx = np.zeros((0, 8), np.int32)
    ctx = E.Context(0)
    model = E.ExaStitchModel(ctx, verts, idx, gl, s)
    model.setNumGridCells(dims)
    sampler = E.ExaStitchSampler(ctx)
    sampler.build(model)
    lo, hi = model.cellBounds
    ranges, _ = sampler.majorants(dims)
    f = oracle.Field(verts, idx, gl, s)
    want = f.majorants(dims, lo, hi)
    assert same_floats(ranges, want)
    touched = ranges[:, 0] <= ranges[:, 1]
    assert touched.sum() > 0 and (~touched).sum() > 0
    gr, _, _ = sampler.prim_majorants()
    assert same_floats(gr, f.gridlet_value_ranges())
    ctx.close()


def test_build_stats(cuda, native):
    """exa_get_build_stats: the build's own CUDA-event times of the majorant
    kernels (no reference counterpart)"""
    from owlexastitcher_gb300 import exastitch as E
    gl, s = edge_model(CASES[0][1])
    ctx = E.Context(0)
    assert ctx.build_stats()["majorantBlocks"] == 0
    model = E.ExaStitchModel(ctx, np.zeros((0, 4), np.float32), np.zeros((0, 8), np.int32), gl, s)
    model.setNumGridCells((16, 16, 16))
    E.ExaStitchSampler(ctx).build(model)
    st = ctx.build_stats()
    assert 0 < st["majorantBlocks"] <= len(gl)
    assert st["gridletMajorantMs"] > 0 and st["elemMajorantMs"] >= 0
    assert st["totalMs"] >= st["gridletMajorantMs"]
    assert ctx.device_errors() == 0
    ctx.close()
