"""ctypes bindings for the CPU oracle (oracle/liboracle.so) and, where it was
built, the reference-header library (oracle/_ref/libexaref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the CPU
baseline leg of bench.py.  The product package never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libexaref.so")
# the owlExaStitcher source tree (only where it is present): the
# EXA_REFERENCE_TREE environment variable, else the build container's mount
REF_TREE = os.environ.get("EXA_REFERENCE_TREE", "/root/reference")


def build(ref=True):
    """Compile the oracle (and the reference-header library when the
    reference tree exists)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])
    if ref and os.path.isdir(REF_TREE):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", "REF=" + REF_TREE])


# ---------------------------------------------------------------- types
class Vec3f(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class Vec3i(C.Structure):
    _fields_ = [("x", C.c_int32), ("y", C.c_int32), ("z", C.c_int32)]


class Box3f(C.Structure):
    _fields_ = [("lower", Vec3f), ("upper", Vec3f)]


class Range1f(C.Structure):
    _fields_ = [("lower", C.c_float), ("upper", C.c_float)]


class Sample(C.Structure):
    _fields_ = [("primID", C.c_int32), ("cellID", C.c_int32), ("value", C.c_float)]


GRIDLET_DTYPE = np.dtype([("lower", "<i4", 3), ("level", "<i4"), ("dims", "<i4", 3), ("begin", "<u4")])
SAMPLE_DTYPE = np.dtype([("primID", "<i4"), ("cellID", "<i4"), ("value", "<f4")])


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def v3(x):
    return Vec3f(float(x[0]), float(x[1]), float(x[2]))


def box(lo, hi):
    return Box3f(v3(lo), v3(hi))


_lib = None
_ref = None


ABR_DTYPE = np.dtype([("domain", "<f4", 6), ("valueRange", "<f4", 2), ("leafListBegin", "<i4"),
                      ("leafListSize", "<i4"), ("finestLevelCellWidth", "<f4")])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.oc_log.restype = C.c_float
        L.oc_log.argtypes = [C.c_float]
        L.oc_sincos_turns.argtypes = [C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.oc_mix64.restype = C.c_uint64
        L.oc_mix64.argtypes = [C.c_uint64]
        L.oc_intersect_gridlet.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_int), Vec3f, vp, vp]
        L.oc_intersect_pyr.argtypes = [C.POINTER(C.c_float), Vec3f, vp]
        L.oc_intersect_wedge.argtypes = [C.POINTER(C.c_float), Vec3f, vp]
        L.oc_intersect_hex.argtypes = [C.POINTER(C.c_float), Vec3f, vp]
        L.oc_intersect_elem.argtypes = [C.POINTER(C.c_float), Vec3f, vp, vp]
        L.oc_project_on_grid.restype = Vec3i
        L.oc_project_on_grid.argtypes = [Vec3f, Vec3i, Box3f]
        L.oc_dda3.restype = C.c_int
        L.oc_dda3.argtypes = [Vec3f, Vec3f, C.c_float, C.c_float, Vec3i, Box3f, C.c_int, vp, vp, vp]
        L.oc_field_create.restype = vp
        L.oc_field_create.argtypes = [vp, C.c_uint64, vp, C.c_uint64, vp, C.c_uint64, vp, C.c_uint64]
        L.oc_field_destroy.argtypes = [vp]
        L.oc_field_set_prim_opacities.argtypes = [vp, vp, vp]
        L.oc_field_set_mesh.argtypes = [vp, vp, vp, C.c_uint64]
        L.oc_field_set_amr.restype = C.c_int
        L.oc_field_set_bricks.restype = C.c_int
        L.oc_field_set_bricks.argtypes = [vp, vp, C.c_uint64, vp, C.c_uint64]
        L.oc_field_abrs.argtypes = [vp, C.POINTER(vp), C.POINTER(C.c_uint64), C.POINTER(vp), C.POINTER(C.c_uint64)]
        L.oc_field_set_amr.argtypes = [vp, vp, C.c_uint64, vp, C.c_uint64]
        L.oc_field_bounds.argtypes = [vp, C.POINTER(Box3f), C.POINTER(Range1f)]
        L.oc_sample.restype = Sample
        L.oc_sample.argtypes = [vp, Vec3f, C.c_int]
        L.oc_sample_points.argtypes = [vp, vp, C.c_uint64, vp, C.c_int, C.c_int]
        L.oc_sample_all.restype = C.c_int
        L.oc_sample_all.argtypes = [vp, Vec3f, C.c_int, C.c_int, vp, vp, vp]
        L.oc_build_majorants.argtypes = [vp, Vec3i, Box3f, vp]
        L.oc_compute_max_opacities.argtypes = [vp, C.c_uint64, vp, C.c_int, Range1f, C.c_int, vp]
        L.oc_gridlet_value_ranges.argtypes = [vp, vp]
        L.oc_elem_max_opacities.argtypes = [vp, vp, C.c_int, Range1f, C.c_int, vp]
        L.oc_lookup_tf.argtypes = [vp, C.c_float, vp]
        L.oc_render.restype = C.c_uint32
        L.oc_render.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int64, C.c_int64, C.c_int]
        L.oc_render_f64.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int64, C.c_int64, vp, C.c_int]
        L.os_bf16.restype = C.c_float
        L.os_bf16.argtypes = [C.c_float]
        L.os_set_exact.argtypes = [C.c_int]
        L.os_half.restype = C.c_float
        L.os_half.argtypes = [C.c_float]
        L.os_geom_init.argtypes = [vp, C.c_int, C.c_int, C.c_float, vp, vp, C.c_float, C.c_float]
        L.os_encode.argtypes = [vp, vp, vp, C.c_int, vp]
        L.os_forward.argtypes = [vp, vp, vp, vp, C.c_int64, vp]
        L.os_gradients.restype = C.c_double
        L.os_gradients.argtypes = [vp, vp, vp, vp, C.c_int, vp, vp]
        _lib = L
    return _lib


def ref():
    """The reference-header library, or None where it was not built."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        R = C.CDLL(REF_PATH)
        vp = C.c_void_p
        R.ref_intersect_gridlet.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_int), vp, vp, vp]
        for n in ("tet", "pyr", "wedge", "hex"):
            getattr(R, "ref_intersect_" + n).argtypes = [C.POINTER(C.c_float), vp, vp]
        R.ref_project_on_grid.argtypes = [vp, vp, vp, vp]
        R.ref_gridlet_bounds.argtypes = [vp, vp]
        R.ref_dda3.restype = C.c_int
        R.ref_dda3.argtypes = [vp, vp, C.c_float, C.c_float, vp, vp, C.c_int, vp, vp, vp]
        _ref = R
    return _ref


# ---------------------------------------------------------------- helpers
def log(x):
    return lib().oc_log(float(x))


def sincos_turns(u):
    s, c = C.c_float(), C.c_float()
    lib().oc_sincos_turns(float(u), C.byref(s), C.byref(c))
    return s.value, c.value


class Field:
    """Oracle view of an ExaStitch field (arrays are kept alive here)."""

    def __init__(self, vertices, indices, gridlets, scalars):
        self.vertices = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 4)
        self.indices = np.ascontiguousarray(indices, dtype=np.int32).reshape(-1, 8)
        self.gridlets = np.ascontiguousarray(gridlets, dtype=GRIDLET_DTYPE)
        self.scalars = np.ascontiguousarray(scalars, dtype=np.float32)
        self._gops = None
        self._eops = None
        self.h = lib().oc_field_create(
            _ptr(self.vertices), len(self.vertices), _ptr(self.indices), len(self.indices),
            _ptr(self.gridlets), len(self.gridlets), _ptr(self.scalars), len(self.scalars))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.oc_field_destroy(self.h)
            self.h = None

    def set_prim_opacities(self, gridlet_ops, elem_ops):
        self._gops = None if gridlet_ops is None else np.ascontiguousarray(gridlet_ops, dtype=np.float32)
        self._eops = None if elem_ops is None else np.ascontiguousarray(elem_ops, dtype=np.float32)
        lib().oc_field_set_prim_opacities(self.h, _ptr(self._gops), _ptr(self._eops))

    @classmethod
    def amr(cls, cells, scalars):
        """a field of AMR cells (int32 [n, 4]: pos, level) with their scalars,
        reconstructed by the AMR-cell sampler's tent basis"""
        f = cls(np.zeros((0, 4), np.float32), np.zeros((0, 8), np.int32), np.zeros(0, GRIDLET_DTYPE),
                np.zeros(0, np.float32))
        f._cells = np.ascontiguousarray(cells, dtype=np.int32).reshape(-1, 4)
        f._cscal = np.ascontiguousarray(scalars, dtype=np.float32)
        rc = lib().oc_field_set_amr(f.h, _ptr(f._cells), len(f._cells), _ptr(f._cscal), len(f._cscal))
        if rc:
            raise ValueError(f"bad AMR cells ({rc})")
        return f

    @classmethod
    def bricks(cls, bricks, scalars):
        """a field of ExaBricks (BRICK_DTYPE records) and their scalars,
        reconstructed by the ExaBrick basis over the active brick regions"""
        f = cls(np.zeros((0, 4), np.float32), np.zeros((0, 8), np.int32), np.zeros(0, GRIDLET_DTYPE),
                np.zeros(0, np.float32))
        f._bricks = np.ascontiguousarray(bricks)
        f._bscal = np.ascontiguousarray(scalars, dtype=np.float32)
        rc = lib().oc_field_set_bricks(f.h, _ptr(f._bricks), len(f._bricks), _ptr(f._bscal), len(f._bscal))
        if rc:
            raise ValueError(f"bad bricks ({rc})")
        return f

    def abrs(self):
        """(regions as ABR_DTYPE, leaf list int32)"""
        a, la = C.c_void_p(), C.c_void_p()
        n, nl = C.c_uint64(), C.c_uint64()
        lib().oc_field_abrs(self.h, C.byref(a), C.byref(n), C.byref(la), C.byref(nl))
        regions, leaf = np.zeros(0, ABR_DTYPE), np.zeros(0, np.int32)
        if n.value:
            regions = np.frombuffer((C.c_char * (n.value * ABR_DTYPE.itemsize)).from_address(a.value), ABR_DTYPE).copy()
        if nl.value:
            leaf = np.frombuffer((C.c_char * (nl.value * 4)).from_address(la.value), np.int32).copy()
        return regions, leaf

    def set_mesh(self, vertices, indices):
        """surface mesh: float3 vertices, int3 triangles (kept alive here)"""
        self._mv = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        self._mi = np.ascontiguousarray(indices, dtype=np.int32).reshape(-1, 3)
        lib().oc_field_set_mesh(self.h, _ptr(self._mv), _ptr(self._mi), len(self._mi))

    def bounds(self):
        b, r = Box3f(), Range1f()
        lib().oc_field_bounds(self.h, C.byref(b), C.byref(r))
        lo = np.array([b.lower.x, b.lower.y, b.lower.z], np.float32)
        hi = np.array([b.upper.x, b.upper.y, b.upper.z], np.float32)
        return lo, hi, (r.lower, r.upper)

    def sample(self, pos, cull=0, nthreads=0):
        pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
        out = np.zeros(len(pos), SAMPLE_DTYPE)
        lib().oc_sample_points(self.h, _ptr(pos), len(pos), _ptr(out), int(cull), int(nthreads))
        return out

    def sample_all(self, p, cull=0, max_out=16):
        kinds = np.zeros(max_out, np.int32)
        ids = np.zeros(max_out, np.int32)
        vals = np.zeros(max_out, np.float32)
        n = lib().oc_sample_all(self.h, v3(p), int(cull), max_out, _ptr(kinds), _ptr(ids), _ptr(vals))
        return [(int(kinds[i]), int(ids[i]), float(vals[i])) for i in range(n)]

    def majorants(self, dims, lo, hi):
        n = int(dims[0]) * int(dims[1]) * int(dims[2])
        out = np.zeros((n, 2), np.float32)
        lib().oc_build_majorants(self.h, Vec3i(*[int(d) for d in dims]), box(lo, hi), _ptr(out))
        return out

    def gridlet_value_ranges(self):
        out = np.zeros((len(self.gridlets), 2), np.float32)
        lib().oc_gridlet_value_ranges(self.h, _ptr(out))
        return out

    def elem_max_opacities(self, cmap, xf_range, tf_filter=0):
        cmap = np.ascontiguousarray(cmap, dtype=np.float32).reshape(-1, 4)
        out = np.zeros(len(self.indices), np.float32)
        lib().oc_elem_max_opacities(self.h, _ptr(cmap), len(cmap), Range1f(*xf_range), int(tf_filter), _ptr(out))
        return out

    def render(self, lp_bytes, width, height, pixel_begin=0, pixel_end=None, nthreads=0):
        if pixel_end is None:
            pixel_end = width * height
        return lib().oc_render(self.h, lp_bytes, width, height, pixel_begin, pixel_end, nthreads)

    def render_f64(self, lp_bytes, width, height, pixel_begin=0, pixel_end=None, nthreads=0):
        if pixel_end is None:
            pixel_end = width * height
        out = np.zeros((pixel_end - pixel_begin, 3), np.float64)
        lib().oc_render_f64(self.h, lp_bytes, width, height, pixel_begin, pixel_end, _ptr(out), nthreads)
        return out


def max_opacities(ranges, cmap, xf_range, tf_filter=0):
    """tf_filter: 0 nearest (the reference's buffer lookup), 1 linear (its
    texture lookup)"""
    ranges = np.ascontiguousarray(ranges, dtype=np.float32).reshape(-1, 2)
    cmap = np.ascontiguousarray(cmap, dtype=np.float32).reshape(-1, 4)
    out = np.zeros(len(ranges), np.float32)
    lib().oc_compute_max_opacities(_ptr(ranges), len(ranges), _ptr(cmap), len(cmap), Range1f(*xf_range),
                                   int(tf_filter), _ptr(out))
    return out


def lookup_tf(lp_bytes, values):
    """RGBA of the transfer-function lookup of a launch-parameter block (its
    filter, domain and table; the table pointer is the caller's) at each of
    the float32 values"""
    values = np.ascontiguousarray(values, np.float32).ravel()
    out = np.zeros((len(values), 4), np.float32)
    for i, v in enumerate(values):
        lib().oc_lookup_tf(lp_bytes, float(v), out[i].ctypes.data)
    return out


def project_on_grid(V, dims, lo, hi):
    r = lib().oc_project_on_grid(v3(V), Vec3i(*[int(d) for d in dims]), box(lo, hi))
    return (r.x, r.y, r.z)


def dda3(org, dirv, tmin, tmax, dims, lo, hi, max_cells=4096):
    ids = np.zeros(max_cells, np.int64)
    t0 = np.zeros(max_cells, np.float32)
    t1 = np.zeros(max_cells, np.float32)
    n = lib().oc_dda3(v3(org), v3(dirv), float(tmin), float(tmax), Vec3i(*[int(d) for d in dims]),
                      box(lo, hi), max_cells, _ptr(ids), _ptr(t0), _ptr(t1))
    return ids[:n], t0[:n], t1[:n]


def intersect_gridlet(pos, gridlet, scalars):
    g = np.ascontiguousarray(np.array([gridlet], dtype=GRIDLET_DTYPE) if not isinstance(gridlet, np.ndarray) else gridlet.reshape(1))
    s = np.ascontiguousarray(scalars, dtype=np.float32)
    v, c = C.c_float(0), C.c_int(-1)
    hit = lib().oc_intersect_gridlet(C.byref(v), C.byref(c), v3(pos), _ptr(g), _ptr(s))
    return bool(hit), v.value, c.value


def intersect_elem(pos, verts):
    """verts: (n,4) with n in {4,5,6,8}."""
    verts = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 4)
    idx = np.full(8, -1, np.int32)
    idx[: len(verts)] = np.arange(len(verts))
    v = C.c_float(0)
    hit = lib().oc_intersect_elem(C.byref(v), v3(pos), _ptr(idx), _ptr(verts))
    return bool(hit), v.value


# ---------------------------------------------------------------- reference
def ref_intersect_elem(pos, verts):
    R = ref()
    verts = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 4)
    P = np.ascontiguousarray(pos, dtype=np.float32)
    name = {4: "tet", 5: "pyr", 6: "wedge", 8: "hex"}[len(verts)]
    v = C.c_float(0)
    hit = getattr(R, "ref_intersect_" + name)(C.byref(v), _ptr(P), _ptr(verts))
    return bool(hit), v.value


def ref_intersect_gridlet(pos, gridlet, scalars):
    R = ref()
    g = np.ascontiguousarray(np.array([gridlet], dtype=GRIDLET_DTYPE) if not isinstance(gridlet, np.ndarray) else gridlet.reshape(1))
    s = np.ascontiguousarray(scalars, dtype=np.float32)
    P = np.ascontiguousarray(pos, dtype=np.float32)
    v, c = C.c_float(0), C.c_int(-1)
    hit = R.ref_intersect_gridlet(C.byref(v), C.byref(c), _ptr(P), _ptr(g), _ptr(s))
    return bool(hit), v.value, c.value


def ref_project_on_grid(V, dims, lo, hi):
    R = ref()
    V = np.ascontiguousarray(V, np.float32)
    d = np.ascontiguousarray(dims, np.int32)
    b = np.ascontiguousarray(np.concatenate([lo, hi]), np.float32)
    out = np.zeros(3, np.int32)
    R.ref_project_on_grid(_ptr(V), _ptr(d), _ptr(b), _ptr(out))
    return tuple(int(x) for x in out)


def ref_dda3(org, dirv, tmin, tmax, dims, lo, hi, max_cells=4096):
    R = ref()
    o = np.ascontiguousarray(org, np.float32)
    dv = np.ascontiguousarray(dirv, np.float32)
    d = np.ascontiguousarray(dims, np.int32)
    b = np.ascontiguousarray(np.concatenate([lo, hi]), np.float32)
    ids = np.zeros(max_cells, np.int64)
    t0 = np.zeros(max_cells, np.float32)
    t1 = np.zeros(max_cells, np.float32)
    n = R.ref_dda3(_ptr(o), _ptr(dv), float(tmin), float(tmax), _ptr(d), _ptr(b), max_cells,
                   _ptr(ids), _ptr(t0), _ptr(t1))
    return ids[:n], t0[:n], t1[:n]


# ------------------------------------------------------------ learned field
class SurGeom(C.Structure):
    """os_geom (oracle.h); same layout as exa_surrogate_geometry."""
    _fields_ = [("log2T", C.c_int32), ("denseMask", C.c_uint32), ("res", C.c_int32 * 16),
                ("lo", C.c_float * 3), ("inv", C.c_float * 3), ("vmin", C.c_float), ("vrange", C.c_float)]


def sur_geom(log2T, base_res, growth, lo, hi, vmin, vmax):
    g = SurGeom()
    lo = np.ascontiguousarray(lo, np.float32)
    hi = np.ascontiguousarray(hi, np.float32)
    lib().os_geom_init(C.byref(g), int(log2T), int(base_res), float(growth), _ptr(lo), _ptr(hi), float(vmin),
                       float(vmax))
    return g


def sur_encode(geom, table, pos, half=False):
    table = np.ascontiguousarray(table, np.float32)
    p = np.ascontiguousarray(pos, np.float32)
    out = np.zeros(32, np.float32)
    lib().os_encode(C.byref(geom), _ptr(table), _ptr(p), int(bool(half)), _ptr(out))
    return out


def sur_forward(geom, weights, table, pos):
    """normalised outputs y of the inference path (binary16 table)"""
    w = np.ascontiguousarray(weights, np.float32)
    t = np.ascontiguousarray(table, np.float32)
    p = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    y = np.zeros(len(p), np.float64)
    lib().os_forward(C.byref(geom), _ptr(w), _ptr(t), _ptr(p), len(p), _ptr(y))
    return y


def sur_gradients(geom, weights, table, pairs):
    w = np.ascontiguousarray(weights, np.float32)
    t = np.ascontiguousarray(table, np.float32)
    pr = np.ascontiguousarray(pairs, np.float32).reshape(-1, 4)
    gw = np.zeros(len(w), np.float64)
    gt = np.zeros(len(t), np.float64)
    loss = lib().os_gradients(C.byref(geom), _ptr(w), _ptr(t), _ptr(pr), len(pr), _ptr(gw), _ptr(gt))
    return gw, gt, loss
