"""Parity at the benchmarked sizes: the medium field (4 levels, 128^3 root
cells, ~51M cells) and the large sparse cloud (5 levels, 256^3 root cells,
~394M cells), each with its 128^3 majorant grid.

For each field, against the oracle built independently from the same
arrays:
  * the majorant value ranges (Grid.cu:134-246) and max opacities
    (Grid.cu:687-719) of all 128^3 macrocells, bit for bit;
  * 1M uniform point queries (sampler/ExaStitchSampler.h:128-140), bit for
    bit;
  * one 32-row band (16 for the cloud) of the benchmarked frame
    (renderFrame_Impl, deviceCode.cu:1268-1345: path tracing at
    1024x1024 x 16 spp, <= 8 bounces, albedo 0.8, HG g = 0.3, one
    directional light; the cloud at 1920x1080 x 64 spp, <= 16 bounces): the
    accumulation buffer and RGBA8 pixels of those rows bit for bit with the
    GPU's full frame.
"""
import numpy as np
import pytest

from helpers import GpuScene, OracleScene, host_lp, orbit_camera, setup_render
from test_gpu_parity import same_floats

pytestmark = pytest.mark.gpu

NUM_MCS = (128, 128, 128)
# (generator configuration, width, height, spp, bounces, band rows)
WORKLOADS = {
    "medium": ("medium", 1024, 1024, 16, 8, 32),
    "cloud": ("cloud", 1920, 1080, 64, 16, 16),
}


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module", params=list(WORKLOADS), ids=list(WORKLOADS))
def workload(request, cuda, native, oracle):
    from owlexastitcher_gb300 import datagen
    cfg, w, h, spp, bounces, band = WORKLOADS[request.param]
    ds = datagen.Dataset(cfg, device=0)  # the GPU generator (identical to the CPU one)
    g = GpuScene(ds, NUM_MCS)
    o = OracleScene(oracle, ds, NUM_MCS, g.lo, g.hi, g.tf, g.xf)
    yield request.param, ds, g, o, (w, h, spp, bounces, band)
    g.ctx.close()


def test_majorants_bit_exact(workload):
    name, ds, g, o, _ = workload
    ranges, ops = g.sampler.majorants(NUM_MCS)
    assert same_floats(ranges, o.ranges)
    assert ops.tobytes() == o.max_ops.tobytes()
    touched = ranges[:, 0] <= ranges[:, 1]
    assert touched.sum() > 0.2 * len(ranges)


def test_points_bit_exact(workload):
    name, ds, g, o, _ = workload
    rng = np.random.default_rng(42)
    P = rng.uniform(g.lo, g.hi, (1 << 20, 3)).astype(np.float32)
    gs = g.sampler.sample_host(P)
    os_ = o.f.sample(P)
    assert np.array_equal(gs["primID"], os_["primID"])
    assert np.array_equal(gs["cellID"], os_["cellID"])
    assert gs["value"].tobytes() == os_["value"].tobytes()
    assert (gs["primID"] >= 0).mean() > 0.3


def test_frame_band_bit_exact(workload, cuda):
    """The benchmarked frame on the GPU, a band of its rows on the oracle."""
    torch = cuda
    from owlexastitcher_gb300 import exastitch as E
    name, ds, g, o, (w, h, spp, bounces, band) = workload
    lp = setup_render(g.lp, orbit_camera(g.lo, g.hi, w, h), w, h, E.PATH_TRACING_INTEGRATOR, spp, "directional",
                      True, g.lo, g.hi)
    lp.ext.maxBounces = bounces
    lp.ext.traceT = lp.ext.traceTr = None
    lp.accumID = 0
    fb = torch.zeros(w * h, dtype=torch.int32, device="cuda")
    acc = torch.zeros(w * h * 4, dtype=torch.float32, device="cuda")
    lp.fbPointer, lp.accumBuffer = fb.data_ptr(), acc.data_ptr()
    E._check(E.lib().exa_render(g.ctx.h, E.C.byref(lp), w, h))
    g.ctx.sync()
    assert g.ctx.device_errors() == 0
    y0 = h // 2 - band // 2
    pb, pe = y0 * w, (y0 + band) * w
    hl, hfb, hacc, _, _ = host_lp(lp, o, w, h)
    assert o.f.render(bytes(hl), w, h, pb, pe) == 0
    gacc = acc.cpu().numpy().reshape(-1, 4)
    gfb = fb.cpu().numpy().view(np.uint32)
    assert gacc[pb:pe].tobytes() == hacc[pb:pe].tobytes()
    assert np.array_equal(gfb[pb:pe], hfb[pb:pe])
    assert len(np.unique(gfb[pb:pe])) > 16  # the band crosses the volume
    lp.ext.maxBounces = 8
