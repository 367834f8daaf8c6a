"""The AMR-cell comparison sampler (sampler/AMRCellSampler.*, model/
AMRCellModel.*): the tent-basis reconstruction over AMR cells, its majorant
grid (Grid.cu:248-285) and rendering through it.  Known answers on the
oracle (CPU), then the CUDA path against the oracle bit for bit."""
import numpy as np
import pytest

from conftest import dataset


def _uniform_cells(n=6, level=1, f=lambda p: 0.25 + 0.01 * p[..., 0] - 0.02 * p[..., 1] + 0.005 * p[..., 2]):
    w = 1 << level
    idx = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"), -1).reshape(-1, 3)
    cells = np.zeros((len(idx), 4), np.int32)
    cells[:, :3] = idx * w
    cells[:, 3] = level
    centers = (idx + 0.5) * w
    return cells, f(centers).astype(np.float32), f


def test_tent_basis_known_answers(oracle):
    """On a uniform lattice the tent basis is a partition of unity with
    linear precision: a linear field comes back (to rounding) inside the
    lattice, and a cell centre gives that cell's own scalar exactly."""
    cells, vals, f = _uniform_cells()
    fld = oracle.Field.amr(cells, vals)
    rng = np.random.default_rng(0)
    w = 2.0
    P = rng.uniform(1.0 * w, 5.0 * w, (2000, 3)).astype(np.float32)   # interior: >= half a cell from the edge
    s = fld.sample(P)
    assert (s["primID"] == 0).all()
    assert np.abs(s["value"] - f(P.astype(np.float64))).max() < 2e-6
    C = ((cells[:, :3] + 1).astype(np.float32))[::7]          # centres of level-1 cells
    s = fld.sample(C)
    assert s["value"].tobytes() == vals[::7].tobytes()
    # outside every support: no sample
    s = fld.sample(np.float32([[-5, 3, 3], [3, 3, 20]]))
    assert (s["primID"] == -1).all()


@pytest.fixture(scope="module", params=["tiny", "small"])
def scene(request, native, oracle):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from owlexastitcher_gb300 import exastitch as E
    from helpers import ramp_tf
    ds = dataset(request.param)
    ctx = E.Context(0)
    m = E.AMRCellModel.from_dataset(ctx, ds)
    dims = (8, 8, 8) if request.param == "tiny" else (32, 32, 32)
    m.setNumGridCells(dims)
    smp = E.AMRCellSampler(ctx)
    smp.build(m)
    assert smp.builtClassName() == "AMRCellSampler"
    lo, hi = m.cellBounds
    vr = m.valueRange
    tf = ramp_tf()
    xf = (np.float32(vr[0]), np.float32(vr[1]))
    smp.computeMaxOpacities(tf, xf)
    lp = E.new_launch_params()
    smp.setLPs(lp)
    fld = oracle.Field.amr(ds.amr_cells, ds.amr_scalars)
    return ds, ctx, m, smp, lp, fld, dims, lo, hi, tf, xf


@pytest.mark.gpu
class TestGpu:
    def test_bounds_and_majorants(self, scene, oracle):
        ds, ctx, m, smp, lp, fld, dims, lo, hi, tf, xf = scene
        olo, ohi, ovr = fld.bounds()
        assert np.array_equal(lo, olo) and np.array_equal(hi, ohi)
        assert tuple(np.float32(v) for v in m.valueRange) == tuple(np.float32(v) for v in ovr)
        r, ops = smp.majorants(dims)
        oranges = fld.majorants(dims, lo, hi)
        assert r.tobytes() == oranges.tobytes()
        assert ops.tobytes() == oracle.max_opacities(oranges, tf, xf).tobytes()

    def test_samples_bit_exact(self, scene):
        ds, ctx, m, smp, lp, fld, dims, lo, hi, tf, xf = scene
        rng = np.random.default_rng(4)
        P = rng.uniform(lo - 1, hi + 1, (20000, 3)).astype(np.float32)
        # points on cell centres, faces and corners of the lattices
        c = ds.amr_cells[:: max(1, len(ds.amr_cells) // 3000)]
        w = (1 << c[:, 3:4]).astype(np.float32)
        P = np.concatenate([P, c[:, :3] + 0.5 * w, c[:, :3].astype(np.float32), c[:, :3] + w]).astype(np.float32)
        gs = smp.sample_host(P)
        os_ = fld.sample(P)
        assert np.array_equal(gs["primID"], os_["primID"])
        assert gs["value"].tobytes() == os_["value"].tobytes()
        assert (gs["primID"] == 0).mean() > 0.5

    @pytest.mark.parametrize("integrator,light,ext", [(0, "directional", True), (1, "point", False),
                                                      (2, "none", False)])
    def test_render_bit_exact(self, scene, integrator, light, ext):
        import torch
        from helpers import host_lp, orbit_camera, setup_render
        from owlexastitcher_gb300 import exastitch as E
        ds, ctx, m, smp, lp, fld, dims, lo, hi, tf, xf = scene

        class O:
            pass
        o = O()
        o.f = fld
        o.tf = np.ascontiguousarray(tf, np.float32)
        o.max_ops = np.ascontiguousarray(fld.majorants(dims, lo, hi), np.float32)
        o.max_ops = __import__("pyoracle").max_opacities(o.max_ops, tf, xf)
        w, h = 40, 32
        cam = orbit_camera(lo, hi, w, h)
        setup_render(lp, cam, w, h, integrator, 2, light, ext, lo, hi)
        lp.render.dt = 0.5
        n = w * h
        fb = torch.zeros(n, dtype=torch.int32, device="cuda")
        acc = torch.zeros(n * 4, dtype=torch.float32, device="cuda")
        tT = torch.zeros(n, dtype=torch.float32, device="cuda")
        tTr = torch.zeros(n, dtype=torch.float32, device="cuda")
        lp.accumID = 0
        lp.fbPointer, lp.accumBuffer = fb.data_ptr(), acc.data_ptr()
        lp.ext.traceT, lp.ext.traceTr = tT.data_ptr(), tTr.data_ptr()
        E._check(E.lib().exa_render(ctx.h, E.C.byref(lp), w, h))
        ctx.sync()
        assert ctx.device_errors() == 0
        hl, hfb, hacc, htT, htTr = host_lp(lp, o, w, h)
        assert fld.render(bytes(hl), w, h) == 0
        assert np.array_equal(fb.cpu().numpy().view(np.uint32), hfb)
        assert acc.cpu().numpy().reshape(-1, 4).tobytes() == hacc.tobytes()
        assert tT.cpu().numpy().tobytes() == htT.tobytes()
        assert tTr.cpu().numpy().tobytes() == htTr.tobytes()
        assert len(np.unique(hfb)) > 4
        if integrator != 2:
            assert (htT >= 0).mean() > 0.2      # rays interact with the volume
        else:
            # the march composites the volume over the background gradient
            tb = (np.arange(h, dtype=np.float32) / h).repeat(w)
            bg = np.stack([(1 - tb) + tb * 0.5, (1 - tb) + tb * 0.7, (1 - tb) + tb * 1.0], 1)
            assert (np.abs(hacc[:, :3] / 2 - bg).max(1) > 1e-3).mean() > 0.2

    def test_load_from_files(self, scene, tmp_path):
        """AMRCellModel::load: '.cells' records and a raw float32 scalars file"""
        from owlexastitcher_gb300 import exastitch as E
        ds = scene[0]
        (tmp_path / "a.cells").write_bytes(ds.amr_cells.astype(np.int32).tobytes())
        (tmp_path / "a.scalars").write_bytes(ds.amr_scalars.astype(np.float32).tobytes())
        ctx = E.Context(0)
        E._check(E.lib().exa_amrcell_model_load(ctx.h, str(tmp_path / "a.cells").encode(),
                                                str(tmp_path / "a.scalars").encode()))
        b, r = E.box3f(), E.range1f()
        E._check(E.lib().exa_model_get_bounds(ctx.h, E.C.byref(b), E.C.byref(r)))
        lo, hi = scene[7], scene[8]
        assert b.lower.tolist() == lo.tolist() and b.upper.tolist() == hi.tolist()

    def test_rejections(self, scene):
        from owlexastitcher_gb300 import exastitch as E
        ds, ctx, m, smp, lp, fld, dims, lo, hi, tf, xf = scene
        with pytest.raises(E.ExaError, match="ExaStitch sampler"):
            E._check(E.lib().exa_get_prim_majorants(ctx.h, None, None, None))
        ms = m.memStats()
        assert ms["amrCellBytes"] == 16 * len(ds.amr_cells) and ms["amrScalarBytes"] == 4 * len(ds.amr_scalars)
        ctx2 = E.Context(0)
        bad = ds.amr_cells[:10].copy()
        bad[3, 0] = 5     # odd: not a multiple of a level-1 cell's width 2
        bad[3, 3] = 1
        with pytest.raises(E.ExaError, match="multiple of its width"):
            E.AMRCellModel(ctx2, bad, ds.amr_scalars[:10])
        with pytest.raises(E.ExaError, match="fewer scalars"):
            E.AMRCellModel(ctx2, ds.amr_cells[:10], ds.amr_scalars[:5])
        dup = np.concatenate([ds.amr_cells[:10], ds.amr_cells[:1]])
        m2 = E.AMRCellModel(ctx2, dup, np.concatenate([ds.amr_scalars[:10], ds.amr_scalars[:1]]))
        m2.setNumGridCells((4, 4, 4))
        with pytest.raises(E.ExaError, match="duplicate"):
            E.AMRCellSampler(ctx2).build(m2)
