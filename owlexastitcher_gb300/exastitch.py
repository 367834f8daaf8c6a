"""Python host binding of the ExaStitch C ABI (include/exastitch.h).

Mirrors the reference's plugin interface for the path:
  ExaStitchModel      -- model/ExaStitchModel.h:26-55 (+ Model, model/Model.h)
  ExaStitchSampler    -- sampler/ExaStitchSampler.h:37-106 (+ Sampler)
  LaunchParams        -- LaunchParams.h:56-119 (field order kept)
  Renderer            -- the parts of OWLRenderer (OWLRenderer.h:30-175) that
                         drive this path: setCamera, resize, render,
                         setType, setColorMap, setRange, setOpacityScale,
                         setLightSource, setShadeMode
All compute goes through libexastitch.so; there is no Python or CPU
fallback.  Device buffers are torch tensors (plumbing only).
"""
import ctypes as C
import os

import numpy as np

from . import _native

# ------------------------------------------------------------------ status
EXA_OK = 0
EXA_ERR_INVALID = 1
EXA_ERR_CUDA = 2
EXA_ERR_STATE = 3
EXA_ERR_OOM = 4
EXA_ERR_DEVICE_LIMIT = 5

PATH_TRACING_INTEGRATOR = 0
DIRECT_LIGHT_INTEGRATOR = 1
RAY_MARCHING_INTEGRATOR = 2
SHADE_MODE_DEFAULT = 0
SHADE_MODE_GRIDLETS = 1
SHADE_MODE_TEASER = 2
LIGHT_POINT = 0
LIGHT_DIRECTIONAL = 1
TF_FILTER_NEAREST = 0   # the reference's buffer lookup
TF_FILTER_LINEAR = 1    # its texture lookup (EXASTITCH_CUDA_TEXTURE_TF)
RENDER_PATH_AUTO = 0
RENDER_PATH_WAVEFRONT = 1
RENDER_PATH_SINGLE_LAUNCH = 2
DEVERR_DDA_CAP = 1
DEVERR_TRACK_CAP = 2
DEVERR_BVH_STACK = 4
DEVERR_WATCHDOG = 16
DEVERR_COPY_WAIT = 32
DEBUG_COPY_WAIT_TIMEOUT = 1


class ExaError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


# ------------------------------------------------------------------ types
class vec2f(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float)]


class vec3f(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]

    def tolist(self):
        return [self.x, self.y, self.z]


class vec4f(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float), ("w", C.c_float)]


class vec3i(C.Structure):
    _fields_ = [("x", C.c_int32), ("y", C.c_int32), ("z", C.c_int32)]


class box2f(C.Structure):
    _fields_ = [("lower", vec2f), ("upper", vec2f)]


class box3f(C.Structure):
    _fields_ = [("lower", vec3f), ("upper", vec3f)]


class range1f(C.Structure):
    _fields_ = [("lower", C.c_float), ("upper", C.c_float)]


class linear3f(C.Structure):
    _fields_ = [("vx", vec3f), ("vy", vec3f), ("vz", vec3f)]


class affine3f(C.Structure):
    _fields_ = [("l", linear3f), ("p", vec3f)]


class Gridlet(C.Structure):
    _fields_ = [("lower", vec3i), ("level", C.c_int32), ("dims", vec3i), ("begin", C.c_uint32)]


class Sample(C.Structure):
    _fields_ = [("primID", C.c_int32), ("cellID", C.c_int32), ("value", C.c_float)]


class GridTraversable(C.Structure):
    _fields_ = [("dims", vec3i), ("bounds", box3f)]


class KDTreeTraversable(C.Structure):
    _fields_ = [("nodes", C.c_void_p), ("primRefs", C.c_void_p), ("modelBounds", box3f)]


class StitchLP(C.Structure):
    _fields_ = [("sampleBVH", C.c_uint64), ("gridletBuffer", C.c_void_p), ("gridletScalarBuffer", C.c_void_p)]


class AmrCellLP(C.Structure):
    _fields_ = [("sampleBVH", C.c_uint64)]


class ExaBrickLP(C.Structure):
    _fields_ = [("sampleBVH", C.c_uint64), ("brickBuffer", C.c_void_p), ("abrBuffer", C.c_void_p),
                ("scalarBuffer", C.c_void_p), ("abrLeafListBuffer", C.c_void_p)]


class _SamplerUnion(C.Union):
    _fields_ = [("ess", StitchLP), ("acs", AmrCellLP), ("ebs", ExaBrickLP)]


class _TF(C.Structure):
    _fields_ = [("values", C.c_void_p), ("numValues", C.c_int32), ("domain", range1f), ("opacityScale", C.c_float)]


class _Camera(C.Structure):
    _fields_ = [("org", vec3f), ("dir_00", vec3f), ("dir_du", vec3f), ("dir_dv", vec3f)]


class _SubImage(C.Structure):
    _fields_ = [("value", box2f), ("selection", box2f), ("active", C.c_int32), ("selecting", C.c_int32)]


class _Render(C.Structure):
    _fields_ = [("dt", C.c_float), ("heatMapEnabled", C.c_int32), ("heatMapScale", C.c_float), ("spp", C.c_int32)]


class _ClipPlane(C.Structure):
    _fields_ = [("enabled", C.c_int32), ("N", vec3f), ("d", C.c_float)]


class _Light(C.Structure):
    _fields_ = [("pos", vec3f), ("intensity", C.c_float), ("on", C.c_int32)]


class LPExt(C.Structure):
    _fields_ = [
        ("maxBounces", C.c_int32),
        ("albedo", C.c_float),
        ("hgG", C.c_float),
        ("lightType", C.c_int32 * 4),
        ("voxelSpaceTransformInv", affine3f),
        ("cullTransparentPrims", C.c_int32),
        ("frameID", C.c_uint32),
        ("deviceErrors", C.c_void_p),
        ("stepCounters", C.c_void_p),
        ("traceT", C.c_void_p),
        ("traceTr", C.c_void_p),
        ("heatCounts", C.c_void_p),
        ("tfFilter", C.c_int32),
        ("trackStepCap", C.c_int32),
        ("ddaCellCap", C.c_int32),
        ("rowBegin", C.c_int32),
        ("rowEnd", C.c_int32),
        ("pad0", C.c_int32),
        ("pad1", C.c_int32),
    ]


class LaunchParams(C.Structure):
    """LaunchParams.h:56-119 (ExaStitch sampler, buffer transfer function)."""

    _fields_ = [
        ("sampler", _SamplerUnion),
        ("fbPointer", C.c_void_p),
        ("fbDepth", C.c_void_p),
        ("accumBuffer", C.c_void_p),
        ("accumID", C.c_int32),
        ("integrator", C.c_int32),
        ("shadeMode", C.c_int32),
        ("maxOpacities", C.c_void_p),
        ("meshBVH", C.c_uint64),
        ("majorantBVH", C.c_uint64),
        ("majorantKDTree", KDTreeTraversable),
        ("majorantGrid", GridTraversable),
        ("worldSpaceBounds", box3f),
        ("voxelSpaceTransform", affine3f),
        ("lightSpaceTransform", affine3f),
        ("transferFunc", _TF),
        ("camera", _Camera),
        ("subImage", _SubImage),
        ("render", _Render),
        ("clipPlanes", _ClipPlane * 1),
        ("lights", _Light * 4),
        ("ext", LPExt),
    ]


class RenderStats(C.Structure):
    _fields_ = [("wavefront", C.c_uint32), ("rounds", C.c_uint32), ("peakQueue", C.c_uint32),
                ("queueCapacity", C.c_uint32), ("walkLaunches", C.c_uint32), ("cameraMs", C.c_float),
                ("walkMs", C.c_float), ("eventMs", C.c_float), ("kernelLaunches", C.c_uint32)]


class BuildStats(C.Structure):
    _fields_ = [("totalMs", C.c_float), ("elemMajorantMs", C.c_float), ("gridletMajorantMs", C.c_float),
                ("majorantBlocks", C.c_uint32)]


class MemStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "elemVertexBytes", "elemIndexBytes", "gridletBytes", "emptyScalarsBytes", "nonEmptyScalarsBytes",
        "deviceFieldBytes", "deviceAccelBytes", "deviceMajorantBytes", "amrCellBytes", "amrScalarBytes", "bricksBytes", "brickScalarsBytes",
        "abrsBytes", "abrLeafListBytes")]


class SurrogateParams(C.Structure):
    _fields_ = [("log2TableSize", C.c_int32), ("baseResolution", C.c_int32), ("growth", C.c_float),
                ("importanceFraction", C.c_float), ("numSamples", C.c_uint64), ("batch", C.c_int32),
                ("learningRate", C.c_float), ("seed", C.c_uint64), ("learningRateFinal", C.c_float),
                ("pad0", C.c_int32)]


class SurrogateStats(C.Structure):
    _fields_ = [("loss", C.c_float), ("steps", C.c_int32), ("tolerance", C.c_float), ("pad0", C.c_int32),
                ("rmse", C.c_double), ("maxError", C.c_double)] + [(n, C.c_uint64) for n in (
                    "probePoints", "numMacrocells", "numSurrogateMacrocells", "tableBytes", "weightBytes",
                    "inferenceBytes", "fieldBytes", "fallbackFieldBytes")]


class SurrogateGeometry(C.Structure):
    _fields_ = [("log2TableSize", C.c_int32), ("denseMask", C.c_uint32), ("res", C.c_int32 * 16),
                ("lo", C.c_float * 3), ("inv", C.c_float * 3), ("vmin", C.c_float), ("vrange", C.c_float)]


SURROGATE_PARAMS = 64 * 32 + 64 * 64 + 64  # W1 | W2 | w3


class Xf(C.Structure):
    _fields_ = [("opacityScale", C.c_float), ("absDomain", range1f), ("relDomain", range1f), ("numColors", C.c_int32)]


class AmrCell(C.Structure):
    _fields_ = [("pos", vec3i), ("level", C.c_int32)]


class BatchFrame(C.Structure):
    _fields_ = [("org", vec3f), ("dir_00", vec3f), ("dir_du", vec3f), ("dir_dv", vec3f), ("width", C.c_int32),
                ("height", C.c_int32), ("spp", C.c_int32), ("tf", C.c_int32), ("accumID", C.c_uint32),
                ("frameID", C.c_uint32), ("fbPointer", C.c_void_p), ("accumBuffer", C.c_void_p)]


class BatchTuning(C.Structure):
    _fields_ = [("dims", vec3i), ("tileWidth", C.c_int32), ("msBest", C.c_float), ("numTrials", C.c_int32),
                ("trialDims", vec3i * 16), ("trialTileWidth", C.c_int32 * 16), ("trialMs", C.c_float * 16)]

GRIDLET_DTYPE = np.dtype([("lower", "<i4", 3), ("level", "<i4"), ("dims", "<i4", 3), ("begin", "<u4")])
SAMPLE_DTYPE = np.dtype([("primID", "<i4"), ("cellID", "<i4"), ("value", "<f4")])

EXPORTED = [
    "exa_context_create", "exa_context_destroy", "exa_last_error", "exa_sync", "exa_get_device_errors",
    "exa_version", "exa_abi_sizeof", "exa_model_create", "exa_model_get_bounds", "exa_model_set_num_grid_cells",
    "exa_model_set_voxel_space_transform", "exa_model_get_world_bounds", "exa_model_mem_stats",
    "exa_sampler_build", "exa_sampler_compute_max_opacities", "exa_sampler_set_lps", "exa_sampler_class_name",
    "exa_get_majorants", "exa_get_prim_majorants", "exa_sample_points", "exa_sample_points_host",
    "exa_launch_params_init", "exa_render", "exa_render_noalloc", "exa_get_render_stats", "exa_get_build_stats",
    "exa_surrogate_params_default", "exa_surrogate_create", "exa_surrogate_train", "exa_surrogate_evaluate",
    "exa_surrogate_get_stats", "exa_surrogate_get_geometry", "exa_surrogate_sample_points",
    "exa_surrogate_get_params", "exa_surrogate_set_params", "exa_surrogate_gradients",
    "exa_surrogate_get_macrocells", "exa_render_surrogate", "exa_batch_set_transfer_functions",
    "exa_batch_set_majorant_grid", "exa_batch_set_tile_width", "exa_render_batch", "exa_batch_autotune",
    "exa_read_grids", "exa_model_load", "exa_read_xf", "exa_xf_range", "exa_opacity_scale", "exa_read_cells",
    "exa_read_mesh", "exa_mesh_set", "exa_mesh_get_bounds",
    "exa_amrcell_model_create", "exa_amrcell_model_load", "exa_sampler_get_class_name",
    "exa_exabrick_model_create", "exa_exabrick_model_load", "exa_exabrick_get_abrs",
]
NOALLOC_MAX_SAMPLES = 1 << 20

_lib = None


def lib():
    """Loads libexastitch.so (libexastitch_checks.so, the bounds-checked
    build, where EXA_LIBRARY_VARIANT=checks) and checks the struct layouts
    against it."""
    global _lib
    if _lib is not None:
        return _lib
    variant = os.environ.get("EXA_LIBRARY_VARIANT", "")
    L = C.CDLL(_native.lib_path("libexastitch_%s.so" % variant if variant else "libexastitch.so"))
    vp, i32, u64 = C.c_void_p, C.c_int32, C.c_uint64
    ctx_p = C.c_void_p
    sig = {
        "exa_context_create": ([C.POINTER(C.c_void_p), C.c_int, u64], C.c_int),
        "exa_context_destroy": ([ctx_p], C.c_int),
        "exa_last_error": ([], C.c_char_p),
        "exa_sync": ([ctx_p], C.c_int),
        "exa_get_device_errors": ([ctx_p, C.POINTER(C.c_uint32)], C.c_int),
        "exa_version": ([], C.c_char_p),
        "exa_abi_sizeof": ([i32], u64),
        "exa_model_create": ([ctx_p, vp, u64, vp, u64, vp, u64, vp, u64], C.c_int),
        "exa_model_get_bounds": ([ctx_p, C.POINTER(box3f), C.POINTER(range1f)], C.c_int),
        "exa_model_set_num_grid_cells": ([ctx_p, vec3i], C.c_int),
        "exa_model_set_voxel_space_transform": ([ctx_p, box3f, box3f], C.c_int),
        "exa_model_get_world_bounds": ([ctx_p, C.POINTER(box3f)], C.c_int),
        "exa_model_mem_stats": ([ctx_p, C.POINTER(MemStats)], C.c_int),
        "exa_sampler_build": ([ctx_p], C.c_int),
        "exa_sampler_compute_max_opacities": ([ctx_p, vp, i32, range1f], C.c_int),
        "exa_sampler_set_lps": ([ctx_p, C.POINTER(LaunchParams)], C.c_int),
        "exa_set_transfer_function_filter": ([ctx_p, i32], C.c_int),
        "exa_set_render_path": ([ctx_p, i32], C.c_int),
        "exa_debug_set_flags": ([ctx_p, C.c_uint32], C.c_int),
        "exa_sampler_class_name": ([], C.c_char_p),
        "exa_get_majorants": ([ctx_p, vp, vp], C.c_int),
        "exa_get_prim_majorants": ([ctx_p, vp, vp, vp], C.c_int),
        "exa_sample_points": ([ctx_p, vp, u64, vp, i32], C.c_int),
        "exa_sample_points_host": ([ctx_p, vp, u64, vp, i32], C.c_int),
        "exa_launch_params_init": ([C.POINTER(LaunchParams)], C.c_int),
        "exa_render": ([ctx_p, C.POINTER(LaunchParams), i32, i32], C.c_int),
        "exa_render_noalloc": ([ctx_p, C.POINTER(LaunchParams), i32, i32], C.c_int),
        "exa_get_render_stats": ([ctx_p, C.POINTER(RenderStats)], C.c_int),
        "exa_get_build_stats": ([ctx_p, C.POINTER(BuildStats)], C.c_int),
        "exa_surrogate_params_default": ([C.POINTER(SurrogateParams)], None),
        "exa_surrogate_create": ([ctx_p, C.POINTER(SurrogateParams)], C.c_int),
        "exa_surrogate_train": ([ctx_p, i32, C.POINTER(C.c_float)], C.c_int),
        "exa_surrogate_evaluate": ([ctx_p, C.c_float, u64], C.c_int),
        "exa_surrogate_get_stats": ([ctx_p, C.POINTER(SurrogateStats)], C.c_int),
        "exa_surrogate_get_geometry": ([ctx_p, C.POINTER(SurrogateGeometry)], C.c_int),
        "exa_surrogate_sample_points": ([ctx_p, vp, u64, vp], C.c_int),
        "exa_surrogate_get_params": ([ctx_p, vp, vp], C.c_int),
        "exa_surrogate_set_params": ([ctx_p, vp, vp], C.c_int),
        "exa_surrogate_gradients": ([ctx_p, vp, i32, vp, vp, vp], C.c_int),
        "exa_surrogate_get_macrocells": ([ctx_p, vp, vp, vp], C.c_int),
        "exa_render_surrogate": ([ctx_p, C.POINTER(LaunchParams), i32, i32], C.c_int),
        "exa_batch_set_transfer_functions": ([ctx_p, i32, vp, vp, vp, vp], C.c_int),
        "exa_batch_set_majorant_grid": ([ctx_p, vec3i], C.c_int),
        "exa_batch_set_tile_width": ([ctx_p, i32], C.c_int),
        "exa_render_batch": ([ctx_p, C.POINTER(LaunchParams), vp, i32, i32], C.c_int),
        "exa_batch_autotune": ([ctx_p, C.POINTER(LaunchParams), vp, i32, i32, C.POINTER(BatchTuning)], C.c_int),
        "exa_read_grids": ([C.c_char_p, C.c_char_p, vp, C.POINTER(u64), vp, C.POINTER(u64)], C.c_int),
        "exa_model_load": ([ctx_p, C.c_char_p, C.c_char_p], C.c_int),
        "exa_read_xf": ([C.c_char_p, C.POINTER(Xf), vp, i32], C.c_int),
        "exa_xf_range": ([C.POINTER(Xf)], range1f),
        "exa_opacity_scale": ([C.c_float], C.c_float),
        "exa_read_cells": ([C.c_char_p, vp, C.POINTER(u64)], C.c_int),
        "exa_read_mesh": ([C.c_char_p, vp, C.POINTER(u64), vp, C.POINTER(u64)], C.c_int),
        "exa_mesh_set": ([ctx_p, vp, u64, vp, u64], C.c_int),
        "exa_mesh_get_bounds": ([ctx_p, C.POINTER(box3f)], C.c_int),
        "exa_amrcell_model_create": ([ctx_p, vp, u64, vp, u64], C.c_int),
        "exa_amrcell_model_load": ([ctx_p, C.c_char_p, C.c_char_p], C.c_int),
        "exa_sampler_get_class_name": ([ctx_p], C.c_char_p),
        "exa_exabrick_model_create": ([ctx_p, vp, u64, vp, u64], C.c_int),
        "exa_exabrick_model_load": ([ctx_p, C.c_char_p, C.c_char_p], C.c_int),
        "exa_exabrick_get_abrs": ([ctx_p, vp, C.POINTER(u64), vp, C.POINTER(u64)], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    for key, st in ((0, LaunchParams), (1, Gridlet), (2, Sample), (3, MemStats), (4, LPExt), (5, SurrogateParams),
                    (6, SurrogateStats), (7, SurrogateGeometry), (8, BatchFrame), (9, BatchTuning), (10, Xf), (11, AmrCell),
                    (12, RenderStats), (13, BuildStats)):
        if L.exa_abi_sizeof(key) != C.sizeof(st):
            raise RuntimeError(f"ABI layout mismatch for {st.__name__}: C {L.exa_abi_sizeof(key)} vs ctypes {C.sizeof(st)}")
    for key, dt in ((14, BRICK_DTYPE), (15, ABR_DTYPE)):
        if L.exa_abi_sizeof(key) != dt.itemsize:
            raise RuntimeError(f"ABI layout mismatch for key {key}: C {L.exa_abi_sizeof(key)} vs numpy {dt.itemsize}")
    _lib = L
    return L


def _check(rc):
    if rc != EXA_OK:
        raise ExaError(rc, lib().exa_last_error().decode())


def _np_ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _v3(x):
    return vec3f(float(x[0]), float(x[1]), float(x[2]))


def _box(lo, hi):
    return box3f(_v3(lo), _v3(hi))


# ------------------------------------------------------------------ classes
STREAM_PRIVATE = (1 << 64) - 1


class Context:
    """One device + one CUDA stream: torch's current stream by default (so
    torch events and copies order with the library's kernels), or
    STREAM_PRIVATE for a stream the context owns."""

    def __init__(self, device=0, stream=None):
        if stream is None:
            import torch
            stream = torch.cuda.current_stream(device).cuda_stream
        self.device = device
        h = C.c_void_p()
        _check(lib().exa_context_create(C.byref(h), device, int(stream)))
        self.h = h

    def sync(self):
        _check(lib().exa_sync(self.h))

    def set_render_path(self, p):
        """RENDER_PATH_AUTO (small frames in one launch, the rest by the
        wavefront renderer), RENDER_PATH_WAVEFRONT or
        RENDER_PATH_SINGLE_LAUNCH; every choice renders the same frame"""
        _check(lib().exa_set_render_path(self.h, int(p)))

    def set_tf_filter(self, f):
        """TF_FILTER_NEAREST or TF_FILTER_LINEAR for the next
        computeMaxOpacities and the renders after it"""
        _check(lib().exa_set_transfer_function_filter(self.h, int(f)))

    def render_stats(self):
        st = RenderStats()
        _check(lib().exa_get_render_stats(self.h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in RenderStats._fields_}

    def build_stats(self):
        st = BuildStats()
        _check(lib().exa_get_build_stats(self.h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in BuildStats._fields_}

    def device_errors(self):
        b = C.c_uint32()
        _check(lib().exa_get_device_errors(self.h, C.byref(b)))
        return b.value

    def close(self):
        if getattr(self, "h", None):
            lib().exa_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Model:
    """model/Model.h:29-65: the calls every model kind shares."""

    @property
    def cellBounds(self):
        b, r = box3f(), range1f()
        _check(lib().exa_model_get_bounds(self.ctx.h, C.byref(b), C.byref(r)))
        return np.array(b.lower.tolist(), np.float32), np.array(b.upper.tolist(), np.float32)

    @property
    def valueRange(self):
        b, r = box3f(), range1f()
        _check(lib().exa_model_get_bounds(self.ctx.h, C.byref(b), C.byref(r)))
        return (r.lower, r.upper)

    def setNumGridCells(self, dims):
        _check(lib().exa_model_set_num_grid_cells(self.ctx.h, vec3i(*[int(d) for d in dims])))

    def setVoxelSpaceTransform(self, remap_from, remap_to):
        _check(lib().exa_model_set_voxel_space_transform(self.ctx.h, _box(*remap_from), _box(*remap_to)))

    def getBounds(self):
        b = box3f()
        _check(lib().exa_model_get_world_bounds(self.ctx.h, C.byref(b)))
        return np.array(b.lower.tolist(), np.float32), np.array(b.upper.tolist(), np.float32)

    def memStats(self):
        m = MemStats()
        _check(lib().exa_model_mem_stats(self.ctx.h, C.byref(m)))
        return {f: getattr(m, f) for f, _ in MemStats._fields_}


class AMRCellModel(_Model):
    """model/AMRCellModel.h:26-44: AMR leaf cells (pos[3], level; 16 B
    records) with one scalar each."""

    def __init__(self, ctx, cells, scalars):
        self.ctx = ctx
        self.cells = np.ascontiguousarray(cells, np.int32).reshape(-1, 4)
        self.scalars = np.ascontiguousarray(scalars, np.float32)
        _check(lib().exa_amrcell_model_create(ctx.h, _np_ptr(self.cells), len(self.cells), _np_ptr(self.scalars),
                                              len(self.scalars)))

    @classmethod
    def from_dataset(cls, ctx, ds):
        return cls(ctx, ds.amr_cells, ds.amr_scalars)


BRICK_DTYPE = np.dtype([("lower", "<i4", 3), ("size", "<i4", 3), ("level", "<i4"), ("begin", "<u4")])
ABR_DTYPE = np.dtype([("domain", "<f4", 6), ("valueRange", "<f4", 2), ("leafListBegin", "<i4"),
                      ("leafListSize", "<i4"), ("finestLevelCellWidth", "<f4")])


class ExaBrickModel(_Model):
    """model/ExaBrickModel.h:27-52: bricks of same-level cells (BRICK_DTYPE)
    and their scalars; the active brick regions are built on creation."""

    def __init__(self, ctx, bricks, scalars):
        self.ctx = ctx
        self.bricks = np.ascontiguousarray(bricks, BRICK_DTYPE)
        self.scalars = np.ascontiguousarray(scalars, np.float32)
        _check(lib().exa_exabrick_model_create(ctx.h, _np_ptr(self.bricks), len(self.bricks), _np_ptr(self.scalars),
                                               len(self.scalars)))

    def abrs(self):
        """(regions as ABR_DTYPE, leaf list int32)"""
        n, nl = C.c_uint64(), C.c_uint64()
        _check(lib().exa_exabrick_get_abrs(self.ctx.h, None, C.byref(n), None, C.byref(nl)))
        r = np.zeros(n.value, ABR_DTYPE)
        leaf = np.zeros(nl.value, np.int32)
        _check(lib().exa_exabrick_get_abrs(self.ctx.h, _np_ptr(r), C.byref(n), _np_ptr(leaf), C.byref(nl)))
        return r, leaf


class ExaStitchModel(_Model):
    """model/ExaStitchModel.h:26-55, built from in-memory arrays."""

    def __init__(self, ctx, vertices, indices, gridlets, gridlet_scalars):
        self.ctx = ctx
        self.vertices = np.ascontiguousarray(vertices, np.float32).reshape(-1, 4)
        self.indices = np.ascontiguousarray(indices, np.int32).reshape(-1, 8)
        self.gridlets = np.ascontiguousarray(gridlets, GRIDLET_DTYPE)
        self.gridlet_scalars = np.ascontiguousarray(gridlet_scalars, np.float32)
        _check(lib().exa_model_create(ctx.h, _np_ptr(self.vertices), len(self.vertices), _np_ptr(self.indices),
                                      len(self.indices), _np_ptr(self.gridlets), len(self.gridlets),
                                      _np_ptr(self.gridlet_scalars), len(self.gridlet_scalars)))

    @classmethod
    def from_dataset(cls, ctx, ds):
        return cls(ctx, ds.vertices, ds.indices, ds.gridlets, ds.gridlet_scalars)


class ExaStitchSampler:
    """sampler/ExaStitchSampler.h:37-106 (exa_sampler_build picks the
    sampler that goes with the context's model; AMRCellSampler below is the
    same wrapper for the AMR-cell model)."""

    def __init__(self, ctx):
        self.ctx = ctx
        self.model = None
        self.num_mcs = None

    @staticmethod
    def className():
        return lib().exa_sampler_class_name().decode()

    def builtClassName(self):
        return lib().exa_sampler_get_class_name(self.ctx.h).decode()

    def build(self, model):
        _check(lib().exa_sampler_build(self.ctx.h))
        self.model = model
        return True

    def computeMaxOpacities(self, colorMap, xfRange):
        cm = np.ascontiguousarray(colorMap, np.float32).reshape(-1, 4)
        self._cmap = cm
        _check(lib().exa_sampler_compute_max_opacities(self.ctx.h, _np_ptr(cm), len(cm), range1f(*xfRange)))

    def setLPs(self, lp):
        _check(lib().exa_sampler_set_lps(self.ctx.h, C.byref(lp)))

    def majorants(self, num_mcs):
        n = int(np.prod(num_mcs))
        ranges = np.zeros((n, 2), np.float32)
        ops = np.zeros(n, np.float32)
        _check(lib().exa_get_majorants(self.ctx.h, _np_ptr(ranges), _np_ptr(ops)))
        return ranges, ops

    def prim_majorants(self):
        ng = len(self.model.gridlets)
        ne = len(self.model.indices)
        gr = np.zeros((ng, 2), np.float32)
        gop = np.zeros(ng, np.float32)
        eop = np.zeros(ne, np.float32)
        _check(lib().exa_get_prim_majorants(self.ctx.h, _np_ptr(gr) if ng else None, _np_ptr(gop) if ng else None,
                                            _np_ptr(eop) if ne else None))
        return gr, gop, eop

    def sample_device(self, pos_dev, out_dev, n, cull=False):
        """pos_dev / out_dev: device addresses (e.g. torch data_ptr())."""
        _check(lib().exa_sample_points(self.ctx.h, pos_dev, n, out_dev, int(bool(cull))))

    def sample_host(self, pos, cull=False):
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        out = np.zeros(len(pos), SAMPLE_DTYPE)
        _check(lib().exa_sample_points_host(self.ctx.h, _np_ptr(pos), len(pos), _np_ptr(out), int(bool(cull))))
        return out


class AMRCellSampler(ExaStitchSampler):
    """sampler/AMRCellSampler.h:26-56: tent-basis reconstruction over AMR
    cells."""

    @staticmethod
    def className():
        return "AMRCellSampler"

    def prim_majorants(self):
        raise ExaError(EXA_ERR_STATE, "the AMR-cell sampler has no per-primitive majorants")


class ExaBrickSampler(ExaStitchSampler):
    """sampler/ExaBrickSampler.h:30-96 (grid + DDA traversal, ABR sampling)."""

    @staticmethod
    def className():
        return "ExaBrickSampler"

    def prim_majorants(self):
        raise ExaError(EXA_ERR_STATE, "the ExaBrick sampler has no per-primitive majorants")


def new_launch_params():
    lp = LaunchParams()
    _check(lib().exa_launch_params_init(C.byref(lp)))
    return lp


def camera_vectors(pos, at, up, fovy_deg, width, height):
    """Pinhole camera in the SimpleCamera convention the renderer's
    setCamera takes: dir = dir_00 + (x+rx)*dir_du + (y+ry)*dir_dv."""
    pos, at, up = (np.asarray(v, np.float64) for v in (pos, at, up))
    d = at - pos
    d /= np.linalg.norm(d)
    u = np.cross(d, up)
    u /= np.linalg.norm(u)
    v = np.cross(u, d)
    h = 2.0 * np.tan(np.radians(fovy_deg) * 0.5)
    aspect = width / float(height)
    du = u * (h * aspect / width)
    dv = v * (h / height)
    d00 = d - 0.5 * width * du - 0.5 * height * dv
    return pos.astype(np.float32), d00.astype(np.float32), du.astype(np.float32), dv.astype(np.float32)


class Renderer:
    """The OWLRenderer calls that drive this path (OWLRenderer.cpp:309-807),
    on device buffers held as torch tensors."""

    def __init__(self, ctx, model, num_mcs=(128, 128, 128)):
        import torch
        self.torch = torch
        self.ctx = ctx
        self.model = model
        self.num_mcs = tuple(int(d) for d in num_mcs)
        model.setNumGridCells(self.num_mcs)
        self.sampler = ExaStitchSampler(ctx)
        self.sampler.build(model)
        self.lp = new_launch_params()
        self.sampler.setLPs(self.lp)
        self.accumID = 0
        self.spp = 1
        self.fbSize = (0, 0)
        self.absDomain = tuple(model.valueRange)
        self.relDomain = (0.0, 100.0)
        self.colorMap = None
        self.fb = None
        self.accum = None
        self.learned = False  # render with the learned field (Surrogate) where it is valid

    def _xf_range(self):
        a0, a1 = self.absDomain
        r0, r1 = self.relDomain
        return (np.float32(a0 + (r0 / 100.0) * (a1 - a0)), np.float32(a0 + (r1 / 100.0) * (a1 - a0)))

    def setColorMap(self, cm):
        self.colorMap = np.ascontiguousarray(cm, np.float32).reshape(-1, 4)
        self.sampler.computeMaxOpacities(self.colorMap, self._xf_range())
        self.sampler.setLPs(self.lp)
        self.accumID = 0

    def setRange(self, lo, hi):
        self.absDomain = (float(lo), float(hi))
        if self.colorMap is not None:
            self.sampler.computeMaxOpacities(self.colorMap, self._xf_range())
            self.sampler.setLPs(self.lp)

    def setMesh(self, vertices, indices):
        """surface mesh (OWLRenderer.cpp:446-545): float3 vertices, int3
        triangles; an empty triangle list removes it"""
        set_mesh(self.ctx, vertices, indices)
        self.sampler.setLPs(self.lp)
        self.accumID = 0

    def setOpacityScale(self, s):
        self.lp.transferFunc.opacityScale = float(np.power(np.float32(1.1), np.float32(s - 100)))

    def setType(self, integrator):
        self.lp.integrator = int(integrator)
        self.accumID = 0

    def setShadeMode(self, sm):
        self.lp.shadeMode = int(sm)
        self.accumID = 0

    def setLightSource(self, i, pos, intensity, on, kind=LIGHT_POINT):
        self.lp.lights[i].pos = _v3(pos)
        self.lp.lights[i].intensity = float(intensity)
        self.lp.lights[i].on = int(bool(on))
        self.lp.ext.lightType[i] = int(kind)
        self.accumID = 0

    def setCamera(self, org, dir_00, dir_du, dir_dv):
        c = self.lp.camera
        c.org, c.dir_00, c.dir_du, c.dir_dv = _v3(org), _v3(dir_00), _v3(dir_du), _v3(dir_dv)
        self.accumID = 0

    def resize(self, w, h):
        if (w, h) != self.fbSize:
            t = self.torch
            self.fb = t.zeros(w * h, dtype=t.int32, device=f"cuda:{self.ctx.device}")
            self.accum = t.zeros(w * h * 4, dtype=t.float32, device=f"cuda:{self.ctx.device}")
            self.fbSize = (w, h)
            self.accumID = 0

    def render(self, fbPointer=None):
        """OWLRenderer::render (OWLRenderer.cpp:610-622): one frame of spp
        samples per pixel, accumulated progressively."""
        w, h = self.fbSize
        self.lp.fbPointer = fbPointer if fbPointer is not None else self.fb.data_ptr()
        self.lp.accumBuffer = self.accum.data_ptr()
        self.lp.accumID = self.accumID
        self.accumID += 1
        self.lp.render.dt = 1.0
        self.lp.render.spp = max(self.spp, 1)
        fn = lib().exa_render_surrogate if self.learned else lib().exa_render
        _check(fn(self.ctx.h, C.byref(self.lp), w, h))

    def checkpoint(self, path):
        """Saves the progressive render's state: the accumulation buffer (the
        running per-pixel sums of deviceCode.cu:1329-1332), the next frame's
        accumID and the frame size and spp.  Every sample's random numbers
        follow from (pixel, accumID, frameID, sample), so a renderer restored
        from it continues with exactly the frames an uninterrupted one
        renders."""
        w, h = self.fbSize
        np.savez(path, accum=self.accum.cpu().numpy(), accumID=np.int64(self.accumID), width=np.int64(w),
                 height=np.int64(h), spp=np.int64(self.spp), frameID=np.int64(self.lp.ext.frameID))

    def restore(self, path):
        """Continues a progressive render saved by checkpoint() (same model,
        camera and transfer function)."""
        with np.load(path) as z:
            self.resize(int(z["width"]), int(z["height"]))
            self.spp = int(z["spp"])
            self.lp.ext.frameID = int(z["frameID"])
            self.accum.copy_(self.torch.from_numpy(z["accum"]).to(self.accum.device))
            self.accumID = int(z["accumID"])


class Surrogate:
    """The learned field of a context: hash-grid encoding + MLP trained on
    the exact sampler's values (exa_surrogate_* in exastitch.h)."""

    def __init__(self, ctx, **params):
        self.ctx = ctx
        p = SurrogateParams()
        lib().exa_surrogate_params_default(C.byref(p))
        for k, v in params.items():
            setattr(p, k, v)
        self.params = p
        _check(lib().exa_surrogate_create(ctx.h, C.byref(p)))
        g = SurrogateGeometry()
        _check(lib().exa_surrogate_get_geometry(ctx.h, C.byref(g)))
        self.geometry = g
        self.table_floats = 2 * 16 * (1 << p.log2TableSize)

    def train(self, steps):
        loss = C.c_float(0.0)
        _check(lib().exa_surrogate_train(self.ctx.h, int(steps), C.byref(loss)))
        return float(loss.value)

    def evaluate(self, tolerance=0.02, points=1 << 24):
        _check(lib().exa_surrogate_evaluate(self.ctx.h, float(tolerance), int(points)))

    def stats(self):
        st = SurrogateStats()
        _check(lib().exa_surrogate_get_stats(self.ctx.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in SurrogateStats._fields_ if k != "pad0"}

    def params_host(self):
        w = np.zeros(SURROGATE_PARAMS, np.float32)
        t = np.zeros(self.table_floats, np.float32)
        _check(lib().exa_surrogate_get_params(self.ctx.h, _np_ptr(w), _np_ptr(t)))
        return w, t

    def set_params(self, weights=None, table=None):
        wp = _np_ptr(np.ascontiguousarray(weights, np.float32)) if weights is not None else None
        tp = _np_ptr(np.ascontiguousarray(table, np.float32)) if table is not None else None
        keep = (weights, table)
        _check(lib().exa_surrogate_set_params(self.ctx.h, wp, tp))
        del keep

    def gradients(self, pairs):
        pairs = np.ascontiguousarray(pairs, np.float32).reshape(-1, 4)
        gw = np.zeros(SURROGATE_PARAMS, np.float32)
        gt = np.zeros(self.table_floats, np.float32)
        loss = C.c_float(0.0)
        _check(lib().exa_surrogate_gradients(self.ctx.h, _np_ptr(pairs), len(pairs), _np_ptr(gw), _np_ptr(gt),
                                             C.byref(loss)))
        return gw, gt, float(loss.value)

    def sample_device(self, pos_dev, out_dev, n):
        _check(lib().exa_surrogate_sample_points(self.ctx.h, C.c_void_p(pos_dev), int(n), C.c_void_p(out_dev)))

    def macrocells(self, num_mcs):
        mode = np.zeros(num_mcs, np.uint8)
        err = np.zeros(num_mcs, np.float64)
        maj = np.zeros(num_mcs, np.float32)
        _check(lib().exa_surrogate_get_macrocells(self.ctx.h, _np_ptr(mode), _np_ptr(err), _np_ptr(maj)))
        return mode, err, maj


class Batch:
    """Many frames in one wavefront (exa_render_batch): per-frame camera,
    size, spp, transfer function and output buffers."""

    def __init__(self, ctx):
        self.ctx = ctx
        self._keep = None

    def set_transfer_functions(self, tfs, xf_ranges, opacity_scales=None):
        maps = [np.ascontiguousarray(t, np.float32).reshape(-1, 4) for t in tfs]
        ptrs = (C.c_void_p * len(maps))(*[m.ctypes.data for m in maps])
        counts = np.array([len(m) for m in maps], np.int32)
        ranges = np.ascontiguousarray(np.array(xf_ranges, np.float32).reshape(-1, 2))
        scales = np.ones(len(maps), np.float32) if opacity_scales is None else np.asarray(opacity_scales, np.float32)
        _check(lib().exa_batch_set_transfer_functions(self.ctx.h, len(maps), ptrs, _np_ptr(counts), _np_ptr(ranges),
                                                      _np_ptr(scales)))

    def set_majorant_grid(self, dims):
        _check(lib().exa_batch_set_majorant_grid(self.ctx.h, vec3i(*[int(d) for d in dims])))

    def set_tile_width(self, w):
        _check(lib().exa_batch_set_tile_width(self.ctx.h, int(w)))

    @staticmethod
    def frames(specs):
        """specs: dicts with cam (org, dir_00, dir_du, dir_dv), width, height,
        spp, tf, and optional accumID, frameID, fb, accum (device pointers)"""
        arr = (BatchFrame * len(specs))()
        for f, sp in zip(arr, specs):
            org, d00, du, dv = sp["cam"]
            f.org, f.dir_00, f.dir_du, f.dir_dv = _v3(org), _v3(d00), _v3(du), _v3(dv)
            f.width, f.height, f.spp, f.tf = sp["width"], sp["height"], sp["spp"], sp["tf"]
            f.accumID, f.frameID = sp.get("accumID", 0), sp.get("frameID", 0)
            f.fbPointer, f.accumBuffer = sp.get("fb"), sp.get("accum")
        return arr

    def render(self, lp, frames, graph=True):
        self._keep = frames
        _check(lib().exa_render_batch(self.ctx.h, C.byref(lp), C.cast(frames, C.c_void_p), len(frames), int(graph)))

    def autotune(self, lp, frames, sample_every=8):
        t = BatchTuning()
        _check(lib().exa_batch_autotune(self.ctx.h, C.byref(lp), C.cast(frames, C.c_void_p), len(frames),
                                        int(sample_every), C.byref(t)))
        return {"dims": (t.dims.x, t.dims.y, t.dims.z), "tileWidth": t.tileWidth, "msBest": t.msBest,
                "trials": [((t.trialDims[i].x, t.trialDims[i].y, t.trialDims[i].z), t.trialTileWidth[i], t.trialMs[i])
                           for i in range(t.numTrials)]}


# ------------------------------------------------------------- file formats
def read_grids(grids_file, scalars_file):
    """'.grids' + '.scalars' -> (gridlets structured array, gridlet scalars)"""
    L = lib()
    ng, ns = C.c_uint64(0), C.c_uint64(0)
    g, sf = os.fsencode(grids_file), os.fsencode(scalars_file) if scalars_file else None
    _check(L.exa_read_grids(g, sf, None, C.byref(ng), None, C.byref(ns)))
    gl = np.zeros(ng.value, GRIDLET_DTYPE)
    sc = np.zeros(ns.value, np.float32)
    _check(L.exa_read_grids(g, sf, _np_ptr(gl), C.byref(ng), _np_ptr(sc), C.byref(ns)))
    return gl, sc


def read_xf(xf_file):
    """'.xf' -> dict(opacityScale, absDomain, relDomain, colorMap, range)"""
    L = lib()
    xf = Xf()
    _check(L.exa_read_xf(os.fsencode(xf_file), C.byref(xf), None, 0))
    cm = np.zeros((xf.numColors, 4), np.float32)
    _check(L.exa_read_xf(os.fsencode(xf_file), C.byref(xf), _np_ptr(cm), xf.numColors))
    r = L.exa_xf_range(C.byref(xf))
    return {"opacityScale": xf.opacityScale, "absDomain": (xf.absDomain.lower, xf.absDomain.upper),
            "relDomain": (xf.relDomain.lower, xf.relDomain.upper), "colorMap": cm, "range": (r.lower, r.upper)}


def read_cells(cells_file):
    """AMR '.cells' -> structured array (pos[3], level)"""
    L = lib()
    n = C.c_uint64(0)
    _check(L.exa_read_cells(os.fsencode(cells_file), None, C.byref(n)))
    out = np.zeros(n.value, np.dtype([("pos", "<i4", 3), ("level", "<i4")]))
    _check(L.exa_read_cells(os.fsencode(cells_file), _np_ptr(out), C.byref(n)))
    return out


def read_mesh(mesh_file):
    """triangle-mesh file (TriangleMesh.cpp:27-76) -> (float32 [n, 3]
    vertices, int32 [m, 3] triangles), all meshes of the file concatenated"""
    L = lib()
    nv, nt = C.c_uint64(0), C.c_uint64(0)
    _check(L.exa_read_mesh(os.fsencode(mesh_file), None, C.byref(nv), None, C.byref(nt)))
    v = np.zeros((nv.value, 3), np.float32)
    t = np.zeros((nt.value, 3), np.int32)
    _check(L.exa_read_mesh(os.fsencode(mesh_file), _np_ptr(v), C.byref(nv), _np_ptr(t), C.byref(nt)))
    return v, t


def set_mesh(ctx, vertices, indices):
    """the context's surface mesh (exa_mesh_set); no triangles removes it"""
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(indices, np.int32).reshape(-1, 3)
    _check(lib().exa_mesh_set(ctx.h, _np_ptr(v), len(v), _np_ptr(t), len(t)))


def mesh_bounds(ctx):
    b = box3f()
    _check(lib().exa_mesh_get_bounds(ctx.h, C.byref(b)))
    return (np.array([b.lower.x, b.lower.y, b.lower.z], np.float32),
            np.array([b.upper.x, b.upper.y, b.upper.z], np.float32))
