"""Gridlet point location with one block table per level (exa_accel.cuh
sample_field, exa_api.cpp buildGridletTables).

The model holds gridlets of levels 0, 1 and 2 that touch and overlap each
other's boxes near the origin (the gridlets of test_majorant_build's edge
model) and one level-7 gridlet far away: one table over the finest lattice
would need far more than 2^27 blocks, so every level gets its own table.
Random points, points on gridlet faces, edges and corners, and points in the
gap between the groups sample bit for bit as the oracle's point location (every containing primitive, lowest index); the same
near points give the same answers in the model without the far gridlet,
which has one table over the finest lattice."""
import numpy as np
import pytest

from test_majorant_build import GRIDLET_DTYPE, edge_model

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def with_far_gridlet(gl, s):
    far = np.zeros(1, GRIDLET_DTYPE)
    far[0] = ((3000, 3000, 3000), 7, (2, 2, 2), len(s))
    vals = np.linspace(-1.0, 1.0, 27).astype(np.float32)
    return np.concatenate([gl, far]), np.concatenate([s, vals])


def gridlet_points(gl, rng, n):
    """random points over the near gridlets' boxes, and on their faces,
    edges and corners"""
    boxes = []
    for g in gl:
        w = float(1 << int(g["level"]))
        lo = (g["lower"].astype(np.float64) + 0.5) * w
        hi = (g["lower"].astype(np.float64) + np.maximum(g["dims"], 0) + 0.5) * w
        boxes.append((lo, hi))
    lo = np.min([b[0] for b in boxes], axis=0) - 2.0
    hi = np.max([b[1] for b in boxes], axis=0) + 2.0
    P = [rng.uniform(lo, hi, (n, 3))]
    for blo, bhi in boxes:
        k = rng.integers(0, 2, (64, 3))
        face = rng.uniform(blo, bhi, (64, 3))
        axis = rng.integers(0, 3, 64)
        face[np.arange(64), axis] = np.where(k[np.arange(64), axis] == 1, bhi[axis], blo[axis])
        corners = np.where(k == 1, bhi, blo)
        P += [face, corners]
    return np.concatenate(P).astype(np.float32)


def sample_gpu(E, gl, s, P):
    ctx = E.Context(0)
    model = E.ExaStitchModel(ctx, np.zeros((0, 4), np.float32), np.zeros((0, 8), np.int32), gl, s)
    model.setNumGridCells((16, 16, 16))
    sampler = E.ExaStitchSampler(ctx)
    sampler.build(model)
    got = sampler.sample_host(P)
    assert ctx.device_errors() == 0
    ctx.close()
    return got


def test_per_level_tables_bit_exact(cuda, native, oracle):
    from owlexastitcher_gb300 import exastitch as E
    gl, s = edge_model(((5, 5, 5), 0, (1, 1, 1)))
    glf, sf = with_far_gridlet(gl, s)
    rng = np.random.default_rng(5)
    P = gridlet_points(gl, rng, 200000)
    # points around the far gridlet and between the groups as well
    far_lo = (3000 + 0.5) * 128.0
    P = np.concatenate([P, rng.uniform(far_lo - 64, far_lo + 3 * 128 + 64, (20000, 3)).astype(np.float32),
                        rng.uniform(-100, far_lo, (20000, 3)).astype(np.float32)])
    got = sample_gpu(E, glf, sf, P)
    want = oracle.Field(np.zeros((0, 4), np.float32), np.zeros((0, 8), np.int32), glf, sf).sample(P)
    assert np.array_equal(got["primID"], want["primID"])
    assert np.array_equal(got["cellID"], want["cellID"])
    assert got["value"].tobytes() == want["value"].tobytes()
    hit = got["primID"] >= 0
    assert hit.mean() > 0.03 and np.any(got["primID"] == len(glf) - 1)
    assert len(np.unique(got["primID"][hit])) >= len(glf) - 2  # (one gridlet has no cells along x)
    # the near points in the model without the far gridlet (one table)
    near = P[:len(P) - 40000]
    one = sample_gpu(E, gl, s, near)
    assert one.tobytes() == got[:len(near)].tobytes()
