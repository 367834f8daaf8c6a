"""On-disk inputs: '.grids' + '.scalars' (model/ExaStitchModel.cpp:44-55,
191-247), '.xf' (headless.cpp:258-298) and AMR '.cells'
(tools/amrMakeDualMesh/makeDual.cpp:932-940).  Files are written here in the
reference's byte layout from a generated dataset and read back through the
C ABI; on the GPU a loaded model builds the same majorants as the same
arrays passed in memory."""
import numpy as np
import pytest

from conftest import dataset


def _write_grids(tmp_path, ds, drop_every=7):
    """gridlets of ds as '.grids' with scalar IDs into a shuffled '.scalars'
    file; every drop_every-th ID points past the file (absent -> NaN)"""
    rng = np.random.default_rng(3)
    g = ds.gridlets
    vals = ds.gridlet_scalars.copy()
    n = len(vals)
    perm = rng.permutation(n)           # file position of each scalar
    scal = np.zeros(n, np.float32)
    scal[perm] = vals
    ids = perm.astype(np.int64)
    drop = np.zeros(n, bool)
    drop[::drop_every] = True
    drop &= ~np.isnan(vals)
    ids[drop] = n + 5
    ids[np.isnan(vals)] = -1             # absent in the generator -> invalid id
    want = vals.copy()
    want[drop] = np.nan
    buf = bytearray()
    for rec in g:
        ns = int(np.prod(rec["dims"] + 1))
        b = int(rec["begin"])
        buf += np.array(list(rec["lower"]) + [rec["level"]] + list(rec["dims"]), np.int32).tobytes()
        buf += ids[b:b + ns].astype(np.int32).tobytes()
    (tmp_path / "f.grids").write_bytes(bytes(buf))
    (tmp_path / "f.scalars").write_bytes(scal.tobytes())
    return want


def test_read_grids(tmp_path, native):
    from owlexastitcher_gb300 import exastitch as E
    ds = dataset("tiny")
    want = _write_grids(tmp_path, ds)
    gl, sc = E.read_grids(str(tmp_path / "f.grids"), str(tmp_path / "f.scalars"))
    assert len(gl) == len(ds.gridlets)
    for k in ("lower", "level", "dims"):
        assert np.array_equal(gl[k], ds.gridlets[k])
    # begin offsets follow the file order (the generator's layout is packed too)
    assert np.array_equal(gl["begin"], ds.gridlets["begin"])
    assert sc.tobytes() == want.tobytes()


def test_read_grids_errors(tmp_path, native):
    from owlexastitcher_gb300 import exastitch as E
    (tmp_path / "t.grids").write_bytes(np.array([0, 0, 0, 0, 2, 2, 2, 1, 2], np.int32).tobytes())
    with pytest.raises(E.ExaError, match="truncated"):
        E.read_grids(str(tmp_path / "t.grids"), "")
    with pytest.raises(E.ExaError, match="cannot open"):
        E.read_grids(str(tmp_path / "missing.grids"), "")
    # a missing scalars file: every scalar absent, as the loader does
    ds = dataset("tiny")
    _write_grids(tmp_path, ds)
    gl, sc = E.read_grids(str(tmp_path / "f.grids"), str(tmp_path / "none.scalars"))
    assert len(gl) == len(ds.gridlets) and np.all(np.isnan(sc))


def test_read_xf(tmp_path, native):
    from owlexastitcher_gb300 import exastitch as E
    cm = np.random.default_rng(1).uniform(0, 1, (128, 4)).astype(np.float32)
    head = np.array([0x1235abc000], np.uint64).tobytes() + np.array([110.0, 2.0, -1.0, 95.0, 5.0],
                                                                    np.float32).tobytes()
    (tmp_path / "a.xf").write_bytes(head + np.array([128], np.int32).tobytes() + cm.tobytes())
    xf = E.read_xf(str(tmp_path / "a.xf"))
    assert xf["opacityScale"] == np.float32(110.0)
    assert xf["absDomain"] == (2.0, -1.0) and xf["relDomain"] == (95.0, 5.0)
    assert xf["colorMap"].tobytes() == cm.tobytes()
    # Headless::xfRange: ordered abs [-1, 2], ordered rel [0.05, 0.95]
    a0, a1 = np.float32(-1.0), np.float32(2.0)
    r0, r1 = np.float32(0.01) * np.float32(5.0), np.float32(0.01) * np.float32(95.0)
    want = ((np.float32(1) - r0) * a0 + r0 * a1, (np.float32(1) - r1) * a0 + r1 * a1)
    assert xf["range"] == (np.float32(want[0]), np.float32(want[1]))
    assert abs(E.lib().exa_opacity_scale(110.0) - 1.1 ** 10) < 1e-5
    (tmp_path / "b.xf").write_bytes(np.array([7], np.uint64).tobytes() + bytes(40))
    with pytest.raises(E.ExaError, match="not a valid"):
        E.read_xf(str(tmp_path / "b.xf"))


def test_read_cells(tmp_path, native):
    from owlexastitcher_gb300 import exastitch as E
    rng = np.random.default_rng(2)
    cells = np.zeros(1000, np.dtype([("pos", "<i4", 3), ("level", "<i4")]))
    cells["pos"] = rng.integers(-100, 1000, (1000, 3))
    cells["level"] = rng.integers(0, 5, 1000)
    (tmp_path / "c.cells").write_bytes(cells.tobytes())
    got = E.read_cells(str(tmp_path / "c.cells"))
    assert got.tobytes() == cells.tobytes()


@pytest.mark.gpu
def test_model_load_matches_arrays(tmp_path, native):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from owlexastitcher_gb300 import exastitch as E
    ds = dataset("tiny")
    _write_grids(tmp_path, ds, drop_every=10 ** 9)
    ctx = E.Context(0)
    E._check(E.lib().exa_model_load(ctx.h, str(tmp_path / "f.grids").encode(), str(tmp_path / "f.scalars").encode()))
    E._check(E.lib().exa_model_set_num_grid_cells(ctx.h, E.vec3i(8, 8, 8)))
    s1 = E.ExaStitchSampler(ctx)
    E._check(E.lib().exa_sampler_build(ctx.h))
    r1, _ = s1.majorants((8, 8, 8))
    ctx2 = E.Context(0)
    m2 = E.ExaStitchModel(ctx2, np.zeros((0, 4), np.float32), np.zeros((0, 8), np.int32), ds.gridlets,
                          ds.gridlet_scalars)
    m2.setNumGridCells((8, 8, 8))
    s2 = E.ExaStitchSampler(ctx2)
    s2.build(m2)
    r2, _ = s2.majorants((8, 8, 8))
    assert r1.tobytes() == r2.tobytes()


def _mesh_record(v, t):
    return (np.array([len(v)], np.int32).tobytes() + np.asarray(v, np.float32).tobytes() +
            np.array([len(t)], np.int32).tobytes() + np.asarray(t, np.int32).tobytes())


def test_read_mesh(tmp_path, native):
    """TriangleMesh::load (TriangleMesh.cpp:27-76): meshes back to back; read
    as one soup with each mesh's indices offset by the vertices before it."""
    from owlexastitcher_gb300 import exastitch as E
    rng = np.random.default_rng(5)
    v1 = rng.uniform(-1, 1, (7, 3)).astype(np.float32)
    t1 = rng.integers(0, 7, (5, 3)).astype(np.int32)
    v2 = rng.uniform(-1, 1, (4, 3)).astype(np.float32)
    t2 = np.array([[0, 1, 2], [1, 2, 3]], np.int32)
    # two stray bytes at the end: too short for a count, the loader stops there
    (tmp_path / "m.mesh").write_bytes(_mesh_record(v1, t1) + _mesh_record(v2, t2) + b"\0\0")
    v, t = E.read_mesh(str(tmp_path / "m.mesh"))
    assert v.tobytes() == np.concatenate([v1, v2]).tobytes()
    assert np.array_equal(t, np.concatenate([t1, t2 + 7]))
    (tmp_path / "e.mesh").write_bytes(b"")
    v, t = E.read_mesh(str(tmp_path / "e.mesh"))
    assert v.shape == (0, 3) and t.shape == (0, 3)


def test_read_mesh_errors(tmp_path, native):
    from owlexastitcher_gb300 import exastitch as E
    v = np.zeros((3, 3), np.float32)
    (tmp_path / "b.mesh").write_bytes(_mesh_record(v, [[0, 1, 3]]))
    with pytest.raises(E.ExaError, match="broken triangle model"):
        E.read_mesh(str(tmp_path / "b.mesh"))
    (tmp_path / "n.mesh").write_bytes(_mesh_record(v, [[0, -1, 2]]))
    with pytest.raises(E.ExaError, match="broken triangle model"):
        E.read_mesh(str(tmp_path / "n.mesh"))
    (tmp_path / "t.mesh").write_bytes(_mesh_record(v, [[0, 1, 2]])[:-4])
    with pytest.raises(E.ExaError, match="truncated"):
        E.read_mesh(str(tmp_path / "t.mesh"))
    with pytest.raises(E.ExaError, match="cannot open"):
        E.read_mesh(str(tmp_path / "missing.mesh"))
