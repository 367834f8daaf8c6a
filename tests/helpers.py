"""Shared set-up for the parity tests: the same dataset, transfer function,
camera and launch parameters on the CUDA path and on the oracle."""
import ctypes as C

import numpy as np


def ramp_tf(n=64):
    """64-entry linear RGBA ramp."""
    t = np.linspace(0.0, 1.0, n, dtype=np.float32)
    return np.stack([t, 0.5 + 0.5 * t * (1 - t), 1.0 - t, t], axis=1).astype(np.float32)


def step_tf(n=64):
    t = np.linspace(0.0, 1.0, n, dtype=np.float32)
    a = (t > 0.5).astype(np.float32) * 0.9
    return np.stack([t, 1 - t, 0.3 + 0 * t, a], axis=1).astype(np.float32)


def two_peak_tf(n=64):
    t = np.linspace(0.0, 1.0, n, dtype=np.float32)
    a = np.exp(-((t - 0.3) / 0.07) ** 2) + np.exp(-((t - 0.75) / 0.05) ** 2)
    return np.stack([t, 0.4 + 0 * t, 1 - t, np.clip(a, 0, 1)], axis=1).astype(np.float32)


def random_tf(n=64, seed=64):
    rng = np.random.default_rng(seed)
    return rng.uniform(0, 1, (n, 4)).astype(np.float32)


def orbit_camera(lo, hi, width, height, angle=0.6, elev=0.35, dist=1.6, fovy=40.0):
    from owlexastitcher_gb300 import exastitch as E
    c = 0.5 * (lo + hi)
    r = float(np.linalg.norm(hi - lo)) * dist * 0.5 / np.tan(np.radians(fovy) * 0.5) * 0.6
    pos = c + r * np.array([np.cos(angle) * np.cos(elev), np.sin(elev), np.sin(angle) * np.cos(elev)])
    return E.camera_vectors(pos, c, [0, 1, 0], fovy, width, height)


class GpuScene:
    """Model + sampler + launch params on the CUDA path."""

    def __init__(self, ds, num_mcs, tf=None, ctx=None):
        from owlexastitcher_gb300 import exastitch as E
        self.E = E
        self.ds = ds
        self.ctx = ctx or E.Context(0)
        # the parity tests render small frames; they test the wavefront
        # renderer (the benchmarked path) unless a test picks the other
        self.ctx.set_render_path(E.RENDER_PATH_WAVEFRONT)
        self.model = E.ExaStitchModel.from_dataset(self.ctx, ds)
        self.num_mcs = tuple(num_mcs)
        self.model.setNumGridCells(self.num_mcs)
        self.sampler = E.ExaStitchSampler(self.ctx)
        self.sampler.build(self.model)
        self.lo, self.hi = self.model.cellBounds
        self.vr = self.model.valueRange
        self.tf = ramp_tf() if tf is None else tf
        self.xf = (np.float32(self.vr[0]), np.float32(self.vr[1]))
        self.sampler.computeMaxOpacities(self.tf, self.xf)
        self.lp = E.new_launch_params()
        self.sampler.setLPs(self.lp)


class OracleScene:
    """The same scene on the oracle, built independently from the arrays."""

    def __init__(self, oracle, ds, num_mcs, lo, hi, tf, xf, tf_filter=0):
        self.O = oracle
        self.f = oracle.Field(ds.vertices, ds.indices, ds.gridlets, ds.gridlet_scalars)
        self.ranges = self.f.majorants(num_mcs, lo, hi)
        self.max_ops = oracle.max_opacities(self.ranges, tf, xf, tf_filter)
        self.g_ranges = self.f.gridlet_value_ranges()
        self.g_ops = (oracle.max_opacities(self.g_ranges, tf, xf, tf_filter) if len(self.g_ranges)
                      else np.zeros(0, np.float32))
        self.e_ops = self.f.elem_max_opacities(tf, xf, tf_filter) if len(ds.indices) else np.zeros(0, np.float32)
        self.f.set_prim_opacities(self.g_ops if len(self.g_ops) else None, self.e_ops if len(self.e_ops) else None)
        self.tf = np.ascontiguousarray(tf, np.float32)


def host_lp(lp, orc, width, height, accum=None):
    """Copy of a device launch-parameter block with HOST pointers for the
    oracle; returns (lp copy, fb, accum, traceT, traceTr) arrays."""
    from owlexastitcher_gb300 import exastitch as E
    h = E.LaunchParams.from_buffer_copy(bytes(lp))
    n = width * height
    fb = np.zeros(n, np.uint32)
    acc = np.zeros((n, 4), np.float32) if accum is None else accum
    tT = np.zeros(n, np.float32)
    tTr = np.zeros(n, np.float32)
    h.transferFunc.values = orc.tf.ctypes.data
    h.maxOpacities = orc.max_ops.ctypes.data
    h.fbPointer = fb.ctypes.data
    h.accumBuffer = acc.ctypes.data
    h.ext.traceT = tT.ctypes.data
    h.ext.traceTr = tTr.ctypes.data
    h.ext.deviceErrors = None
    h.ext.stepCounters = None
    # the struct holds raw addresses: keep the arrays alive with it
    h._keep = (fb, acc, tT, tTr, orc.tf, orc.max_ops)
    return h, fb, acc, tT, tTr


def setup_render(lp, cam, width, height, integrator, spp=1, light="directional", baseline_ext=False, lo=None,
                 hi=None):
    from owlexastitcher_gb300 import exastitch as E
    org, d00, du, dv = cam
    lp.camera.org = E._v3(org)
    lp.camera.dir_00 = E._v3(d00)
    lp.camera.dir_du = E._v3(du)
    lp.camera.dir_dv = E._v3(dv)
    lp.integrator = integrator
    lp.render.spp = spp
    if light == "directional":
        lp.lights[0].pos = E._v3([0.4, 0.8, 0.45])
        lp.lights[0].intensity = 1.5
        lp.lights[0].on = 1
        lp.ext.lightType[0] = E.LIGHT_DIRECTIONAL
    elif light == "point":
        lp.lights[0].pos = E._v3(hi)   # viewer.cpp:958-962 default
        lp.lights[0].intensity = 60.0
        lp.lights[0].on = 1
        lp.ext.lightType[0] = E.LIGHT_POINT
    else:
        lp.lights[0].on = 0
    if baseline_ext:
        lp.ext.albedo = 0.8
        lp.ext.hgG = 0.3
        lp.ext.maxBounces = 8
    return lp


def oracle_only_lp(lo, hi, dims, tf, xf, width, height, integrator, spp, light="directional", baseline_ext=True):
    """Launch parameters for an oracle-only render (no GPU): identity
    transforms, the majorant grid over [lo, hi], the transfer function's
    domain and size (the table and max-opacity pointers are set by
    host_lp), culling on."""
    from owlexastitcher_gb300 import exastitch as E
    lp = E.LaunchParams()
    lp.integrator = integrator
    lp.render.dt = 1.0
    lp.transferFunc.opacityScale = 1.0
    lp.transferFunc.domain.lower, lp.transferFunc.domain.upper = float(xf[0]), float(xf[1])
    lp.transferFunc.numValues = len(tf)
    for A in (lp.voxelSpaceTransform, lp.lightSpaceTransform, lp.ext.voxelSpaceTransformInv):
        A.l.vx.x = A.l.vy.y = A.l.vz.z = 1.0
    lp.majorantGrid.dims = E.vec3i(*[int(d) for d in dims])
    lp.majorantGrid.bounds = E._box(lo, hi)
    lp.worldSpaceBounds = E._box(lo, hi)
    lp.ext.cullTransparentPrims = 1
    lp.ext.maxBounces = 1024
    lp.ext.albedo = -1.0
    setup_render(lp, orbit_camera(lo, hi, width, height), width, height, integrator, spp, light, baseline_ext)
    return lp
