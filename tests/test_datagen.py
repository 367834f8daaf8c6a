"""The synthetic AMR / dual-mesh generator (restatement of
tools/amrMakeDualMesh): determinism and the invariants of its output."""
import numpy as np
import pytest

from conftest import dataset


@pytest.fixture(scope="module")
def small(native):
    return dataset("small")


def test_deterministic(native):
    a, b = dataset("tiny"), dataset("tiny")
    for k in ("vertices", "indices", "gridlet_scalars", "amr_cells", "amr_scalars"):
        assert getattr(a, k).tobytes() == getattr(b, k).tobytes(), k
    assert a.gridlets.tobytes() == b.gridlets.tobytes()
    c = dataset("tiny", seed=7)
    assert c.amr_scalars.tobytes() != a.amr_scalars.tobytes()


def test_hierarchy_counts(small):
    s = small.stats
    assert s["numAmrCells"] == sum(s["numCellsPerLevel"]) == len(small.amr_cells)
    assert all(n > 0 for n in s["numCellsPerLevel"])
    # the leaves tile the domain: volume of all cells == domain volume
    w = 2.0 ** small.amr_cells[:, 3]
    assert np.isclose((w ** 3).sum(), np.prod(small.domain))


def test_gridlets_are_makegrids_bricks(small):
    g = small.gridlets
    assert (g["dims"] >= 1).all() and (g["dims"] <= 8).all()
    # each brick lies inside one 8^3 macrocell of its level (makeGrids.cpp:79-93)
    assert ((g["lower"] // 8) == ((g["lower"] + g["dims"] - 1) // 8)).all()
    n = np.prod(g["dims"] + 1, axis=1)
    assert (np.diff(g["begin"].astype(np.int64)) == n[:-1]).all()
    assert int(g["begin"][-1]) + int(n[-1]) == len(small.gridlet_scalars)
    assert np.isnan(small.gridlet_scalars).sum() == small.stats["numEmptyGridletScalars"]
    assert (np.diff(g["level"]) >= 0).all()  # levels ascending


def test_elements(small):
    idx = small.indices
    nv = (idx >= 0).sum(1)
    assert set(np.unique(nv)) <= {4, 5, 6, 8}
    # -1 padding is a suffix
    for k in (4, 5, 6):
        assert (idx[nv == k][:, k:] == -1).all()
    assert idx.max() < len(small.vertices)
    assert len(np.unique(idx[idx >= 0])) == len(small.vertices)  # compacted
    # element vertices sit on cell centres and carry the cell value
    cells = small.amr_cells
    centre = cells[:, :3] + 0.5 * (2.0 ** cells[:, 3:4])
    lut = {tuple(c): v for c, v in zip(centre.astype(np.float32), small.amr_scalars)}
    for v in small.vertices[:: max(1, len(small.vertices) // 500)]:
        assert lut[tuple(v[:3])] == v[3]


def test_dual_mesh_partitions_space(small, oracle):
    f = oracle.Field(small.vertices, small.indices, small.gridlets, small.gridlet_scalars)
    lo, hi, vr = f.bounds()
    rng = np.random.default_rng(1)
    hits = [len(f.sample_all(p)) for p in rng.uniform(lo, hi, (3000, 3)).astype(np.float32)]
    assert max(hits) == 1                 # no overlaps off shared faces
    assert np.mean(np.array(hits) == 1) > 0.9
    # interpolation follows the analytic field
    P = rng.uniform(lo, hi, (3000, 3)).astype(np.float32)
    s = f.sample(P)
    ok = s["primID"] >= 0
    assert np.abs(s["value"][ok] - small.eval_field(P[ok])).mean() < 0.01
