"""The ExaBrick comparison sampler (model/ExaBrickModel.*, model/ABRs.*,
sampler/ExaBrickSampler.*) in the majorant-grid + DDA traversal mode: active
brick regions, the brick basis, the majorant grid (Grid.cu:362-430) and
rendering through it.  Known answers and invariants on the oracle (CPU),
then the CUDA path against the oracle bit for bit."""
import numpy as np
import pytest

from conftest import dataset


def _bricks(config):
    from owlexastitcher_gb300 import datagen
    ds = dataset(config)
    b, s = datagen.amr_to_bricks(ds.amr_cells, ds.amr_scalars)
    return ds, b, s


def _two_bricks():
    """one level-1 cell at the origin and a 2^3 level-0 brick beside it (the
    layout of the reference's test-data tool)"""
    from owlexastitcher_gb300 import datagen
    b = np.zeros(2, datagen.BRICK_DTYPE)
    b[0]["lower"], b[0]["size"], b[0]["level"], b[0]["begin"] = (0, 0, 0), (1, 1, 1), 1, 0
    b[1]["lower"], b[1]["size"], b[1]["level"], b[1]["begin"] = (2, 0, 0), (2, 2, 2), 0, 1
    return b, np.arange(9, dtype=np.float32)


def test_regions_partition_the_domains(oracle, native):
    """The regions tile the union of the brick domains without overlap and
    each lists exactly the bricks whose domain overlaps it."""
    b, s = _two_bricks()
    f = oracle.Field.bricks(b, s)
    r, leaf = f.abrs()
    dom = r["domain"].astype(np.float64)
    vol = np.prod(dom[:, 3:] - dom[:, :3], axis=1)
    # brick domains: [-1, 3]^3 (cell width 2) and [1.5, 4.5] x [-0.5, 2.5]^2
    union = 4 ** 3 + 3 * 3 * 3 - 1.5 * 3 * 3
    assert np.isclose(vol.sum(), union)
    for i in range(len(r)):
        ids = leaf[r["leafListBegin"][i]:r["leafListBegin"][i] + r["leafListSize"][i]]
        assert list(ids) == sorted(set(ids))
        c = 0.5 * (dom[i, :3] + dom[i, 3:])
        inside = []
        for k in range(2):
            cw = 2.0 ** b[k]["level"]
            lo = b[k]["lower"] - 0.5 * cw
            hi = b[k]["lower"] + (b[k]["size"] + 0.5) * cw
            inside.append(bool(np.all((c > lo) & (c < hi))))
        assert list(np.nonzero(inside)[0]) == list(ids)


def test_brick_basis_known_answers(oracle, native):
    """Inside one brick the basis is trilinear interpolation of the cell
    values at cell centres: a linear field comes back to rounding, a cell
    centre returns its value exactly."""
    from owlexastitcher_gb300 import datagen
    lin = lambda p: 0.5 + 0.03 * p[..., 0] - 0.01 * p[..., 1] + 0.02 * p[..., 2]
    b = np.zeros(1, datagen.BRICK_DTYPE)
    b[0]["lower"], b[0]["size"], b[0]["level"], b[0]["begin"] = (0, 0, 0), (6, 5, 4), 1, 0
    idx = np.stack(np.meshgrid(np.arange(6), np.arange(5), np.arange(4), indexing="ij"), -1)
    centres = (idx + 0.5) * 2.0
    s = lin(centres).transpose(2, 1, 0).reshape(-1).astype(np.float32)   # x fastest
    f = oracle.Field.bricks(b, s)
    P = np.random.default_rng(1).uniform((1, 1, 1), (11, 9, 7), (2000, 3)).astype(np.float32)
    v = f.sample(P)
    assert (v["primID"] == 0).all()
    assert np.abs(v["value"] - lin(P.astype(np.float64))).max() < 2e-6
    C = centres.reshape(-1, 3).astype(np.float32)
    # a centre has weight 1 on its own cell and 0 on the others
    assert f.sample(C)["value"].tobytes() == lin(centres.reshape(-1, 3)).astype(np.float32).tobytes()
    # outside every region: primID 0 and value 0 (the reference's empty BasisPRD)
    o = f.sample(np.float32([[40, 40, 40]]))
    assert o["primID"][0] == 0 and o["value"][0] == 0.0


def test_generated_bricks_follow_the_field(oracle, native):
    ds, b, s = _bricks("tiny")
    f = oracle.Field.bricks(b, s)
    lo, hi, vr = f.bounds()
    P = np.random.default_rng(2).uniform(lo, hi, (3000, 3)).astype(np.float32)
    v = f.sample(P)
    assert np.abs(v["value"] - ds.eval_field(P)).mean() < 0.02


@pytest.fixture(scope="module", params=["tiny", "small"])
def scene(request, native, oracle):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from owlexastitcher_gb300 import exastitch as E
    from helpers import ramp_tf
    ds, b, s = _bricks(request.param)
    ctx = E.Context(0)
    m = E.ExaBrickModel(ctx, b, s)
    dims = (8, 8, 8) if request.param == "tiny" else (32, 32, 32)
    m.setNumGridCells(dims)
    smp = E.ExaBrickSampler(ctx)
    smp.build(m)
    assert smp.builtClassName() == "ExaBrickSampler"
    lo, hi = m.cellBounds
    vr = m.valueRange
    tf = ramp_tf()
    xf = (np.float32(vr[0]), np.float32(vr[1]))
    smp.computeMaxOpacities(tf, xf)
    lp = E.new_launch_params()
    smp.setLPs(lp)
    fld = oracle.Field.bricks(b, s)
    return ds, b, s, ctx, m, smp, lp, fld, dims, lo, hi, tf, xf


@pytest.mark.gpu
class TestGpu:
    def test_regions_and_bounds(self, scene):
        ds, b, s, ctx, m, smp, lp, fld, dims, lo, hi, tf, xf = scene
        r1, l1 = m.abrs()
        r2, l2 = fld.abrs()
        assert r1.tobytes() == r2.tobytes() and np.array_equal(l1, l2)
        olo, ohi, ovr = fld.bounds()
        assert np.array_equal(lo, olo) and np.array_equal(hi, ohi)
        assert tuple(np.float32(v) for v in m.valueRange) == tuple(np.float32(v) for v in ovr)

    def test_majorants_bit_exact(self, scene, oracle):
        ds, b, s, ctx, m, smp, lp, fld, dims, lo, hi, tf, xf = scene
        r, ops = smp.majorants(dims)
        oranges = fld.majorants(dims, lo, hi)
        assert r.tobytes() == oranges.tobytes()
        assert ops.tobytes() == oracle.max_opacities(oranges, tf, xf).tobytes()

    def test_samples_bit_exact(self, scene):
        ds, b, s, ctx, m, smp, lp, fld, dims, lo, hi, tf, xf = scene
        rng = np.random.default_rng(4)
        P = rng.uniform(lo - 1, hi + 1, (20000, 3)).astype(np.float32)
        r, _ = m.abrs()
        d = r["domain"][:: max(1, len(r) // 2000)]
        P = np.concatenate([P, d[:, :3], d[:, 3:], 0.5 * (d[:, :3] + d[:, 3:])]).astype(np.float32)
        gs = smp.sample_host(P)
        os_ = fld.sample(P)
        assert np.array_equal(gs["primID"], os_["primID"])
        assert gs["value"].tobytes() == os_["value"].tobytes()

    @pytest.mark.parametrize("integrator,light,ext", [(0, "directional", True), (1, "point", False),
                                                      (2, "none", False)])
    def test_render_bit_exact(self, scene, oracle, integrator, light, ext):
        import torch
        from helpers import host_lp, orbit_camera, setup_render
        from owlexastitcher_gb300 import exastitch as E
        ds, b, s, ctx, m, smp, lp, fld, dims, lo, hi, tf, xf = scene

        class O:
            pass
        o = O()
        o.f = fld
        o.tf = np.ascontiguousarray(tf, np.float32)
        o.max_ops = oracle.max_opacities(fld.majorants(dims, lo, hi), tf, xf)
        w, h = 40, 32
        setup_render(lp, orbit_camera(lo, hi, w, h), w, h, integrator, 2, light, ext, lo, hi)
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
        """ExaBrickModel::load: '.bricks' records (size, lower, level, cell
        ids) into a scalars file"""
        from owlexastitcher_gb300 import exastitch as E
        ds, b, s, ctx0, m0, *_ = scene
        rng = np.random.default_rng(5)
        perm = rng.permutation(len(s))           # file position of each brick scalar
        vals = np.zeros(len(s), np.float32)
        vals[perm] = s
        buf = bytearray()
        for rec in b:
            n = int(np.prod(rec["size"]))
            buf += np.array(list(rec["size"]) + list(rec["lower"]) + [rec["level"]], np.int32).tobytes()
            buf += perm[rec["begin"]:rec["begin"] + n].astype(np.int32).tobytes()
        (tmp_path / "a.bricks").write_bytes(bytes(buf))
        (tmp_path / "a.scalars").write_bytes(vals.tobytes())
        ctx = E.Context(0)
        E._check(E.lib().exa_exabrick_model_load(ctx.h, str(tmp_path / "a.bricks").encode(),
                                                 str(tmp_path / "a.scalars").encode()))
        m = E.ExaBrickModel.__new__(E.ExaBrickModel)
        m.ctx = ctx
        r1, l1 = m.abrs()
        r0, l0 = m0.abrs()
        assert r1.tobytes() == r0.tobytes() and np.array_equal(l1, l0)
        ms = m.memStats()
        assert ms["bricksBytes"] == 32 * len(b) and ms["brickScalarsBytes"] == 4 * len(s)
        assert ms["abrsBytes"] == 44 * len(r0)
