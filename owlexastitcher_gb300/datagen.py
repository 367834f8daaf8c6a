"""Synthetic AMR datasets and their ExaStitch dual mesh (ctypes over
libexagen.so, the C++ restatement of tools/amrMakeDualMesh).

The configurations mirror the benchmark workloads:
  small  -- 3 levels, 32^3 root cells, 32 Gaussians + 4-octave value noise
  medium -- 4 levels, 128^3 root cells, 256 Gaussians + noise
  cloud  -- 5 levels, 256^3 root cells, sparse exp(3 fBm) cloud
"""
import ctypes as C
import os

import numpy as np

from . import _native

GRIDLET_DTYPE = np.dtype([("lower", "<i4", 3), ("level", "<i4"), ("dims", "<i4", 3), ("begin", "<u4")])

FIELD_GAUSSIANS = 0
FIELD_CLOUD = 1


class GenParams(C.Structure):
    _fields_ = [
        ("numLevels", C.c_int32),
        ("rootDims", C.c_int32 * 3),
        ("fieldKind", C.c_int32),
        ("numGaussians", C.c_int32),
        ("seed", C.c_uint64),
        ("refineThreshold", C.c_float),
        ("noiseAmplitude", C.c_float),
        ("noiseOctaves", C.c_int32),
        ("cloudEmptyFraction", C.c_float),
        ("balance", C.c_int32),
        ("numThreads", C.c_int32),
    ]


class GenStats(C.Structure):
    _fields_ = [
        ("numAmrCells", C.c_uint64),
        ("numCellsPerLevel", C.c_uint64 * 16),
        ("numPerfectCubes", C.c_uint64),
        ("numTets", C.c_uint64),
        ("numPyramids", C.c_uint64),
        ("numWedges", C.c_uint64),
        ("numHexes", C.c_uint64),
        ("numVertices", C.c_uint64),
        ("numGridlets", C.c_uint64),
        ("numGridletScalars", C.c_uint64),
        ("numEmptyGridletScalars", C.c_uint64),
        ("numSkippedDegenerate", C.c_uint64),
        ("seconds", C.c_double),
        ("fieldMin", C.c_float),
        ("fieldMax", C.c_float),
        ("stageSeconds", C.c_double * 6),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(_native.lib_path("libexagen.so"))
        vp = C.c_void_p
        u64p = C.POINTER(C.c_uint64)
        L.exa_gen_params_default.argtypes = [C.POINTER(GenParams)]
        L.exa_gen_run.restype = C.c_int
        L.exa_gen_run.argtypes = [C.POINTER(GenParams), C.POINTER(vp)]
        L.exa_gen_run_gpu.restype = C.c_int
        L.exa_gen_run_gpu.argtypes = [C.POINTER(GenParams), C.c_int32, C.POINTER(vp)]
        L.exa_gen_free.argtypes = [vp]
        L.exa_gen_get_stats.argtypes = [vp, C.POINTER(GenStats)]
        for n in ("vertices", "indices", "gridlets", "gridlet_scalars", "amr_cells", "amr_scalars"):
            f = getattr(L, "exa_gen_" + n)
            f.restype = vp
            f.argtypes = [vp, u64p]
        L.exa_gen_eval_field.argtypes = [vp, vp, C.c_uint64, vp]
        L.exa_gen_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def params(config="small", **overrides):
    p = GenParams()
    lib().exa_gen_params_default(C.byref(p))
    if config == "small":
        pass
    elif config == "medium":
        # refinement threshold chosen so the hierarchy has ~50M cells, the
        # size the medium workload is specified with (51.1M at seed 1234)
        p.numLevels = 4
        p.rootDims[:] = [128, 128, 128]
        p.numGaussians = 256
        p.refineThreshold = 0.67
    elif config == "cloud":
        p.numLevels = 5
        p.rootDims[:] = [256, 256, 256]
        p.fieldKind = FIELD_CLOUD
        p.noiseOctaves = 6
        # refinement thresholds 0.09, 0.18, 0.36, 0.72 of the [0, 1] cloud
        # density for the four refined levels: ~400M cells at 256^3 roots
        p.refineThreshold = 0.09
        p.cloudEmptyFraction = 0.7
    elif config == "tiny":
        p.numLevels = 3
        p.rootDims[:] = [8, 8, 8]
        p.numGaussians = 6
    else:
        raise ValueError("unknown config " + config)
    for k, v in overrides.items():
        if k == "rootDims":
            p.rootDims[:] = list(v)
        else:
            setattr(p, k, v)
    return p


class Dataset:
    """Generated ExaStitch arrays (numpy copies) plus the analytic field.
    device=None runs the CPU generator, device=k its GPU version on CUDA
    device k (identical output)."""

    def __init__(self, config="small", device=None, **overrides):
        self.config = config
        self.device = device
        self.params = params(config, **overrides)
        h = C.c_void_p()
        if device is None:
            rc = lib().exa_gen_run(C.byref(self.params), C.byref(h))
        else:
            rc = lib().exa_gen_run_gpu(C.byref(self.params), int(device), C.byref(h))
        if rc != 0:
            raise RuntimeError("exa_gen_run: " + lib().exa_gen_last_error().decode())
        self._h = h
        st = GenStats()
        lib().exa_gen_get_stats(h, C.byref(st))
        self.stats = {f: getattr(st, f) for f, _ in GenStats._fields_ if f not in ("numCellsPerLevel", "stageSeconds")}
        self.stats["stageSeconds"] = list(st.stageSeconds)
        self.stats["numCellsPerLevel"] = list(st.numCellsPerLevel)[: self.params.numLevels]
        self.vertices = self._arr("vertices", np.float32, 4)
        self.indices = self._arr("indices", np.int32, 8)
        self.gridlets = self._arr("gridlets", GRIDLET_DTYPE, None)
        self.gridlet_scalars = self._arr("gridlet_scalars", np.float32, None)
        self.amr_cells = self._arr("amr_cells", np.int32, 4)
        self.amr_scalars = self._arr("amr_scalars", np.float32, None)
        lvl = self.params.numLevels - 1
        self.domain = np.array([d << lvl for d in self.params.rootDims], np.float32)

    def _arr(self, name, dtype, width):
        n = C.c_uint64()
        p = getattr(lib(), "exa_gen_" + name)(self._h, C.byref(n))
        count = n.value * (width or 1)
        if count == 0:
            shape = (0, width) if width else (0,)
            return np.zeros(shape, dtype)
        nbytes = count * np.dtype(dtype).itemsize
        buf = (C.c_char * nbytes).from_address(p)
        a = np.frombuffer(buf, dtype=dtype).copy()
        return a.reshape(-1, width) if width else a

    def eval_field(self, pos):
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        out = np.zeros(len(pos), np.float32)
        lib().exa_gen_eval_field(self._h, pos.ctypes.data_as(C.c_void_p), len(pos), out.ctypes.data_as(C.c_void_p))
        return out

    def close(self):
        if self._h:
            lib().exa_gen_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def field_bytes(self):
        """Bytes of the ExaStitch field arrays (memStats total)."""
        return (self.vertices.nbytes + self.indices.nbytes + self.gridlets.nbytes + self.gridlet_scalars.nbytes)


BRICK_DTYPE = np.dtype([("lower", "<i4", 3), ("size", "<i4", 3), ("level", "<i4"), ("begin", "<u4")])


def amr_to_bricks(cells, scalars, max_len=8):
    """ExaBricks (model/ABRs.h: same-level cell boxes with their scalars,
    x fastest) from AMR leaf cells: per level, runs of consecutive cells
    along x within 8-aligned segments of a row become bricks of size
    (run, 1, 1).  Returns (bricks as BRICK_DTYPE, scalars in brick order)."""
    cells = np.asarray(cells, np.int64).reshape(-1, 4)
    scalars = np.asarray(scalars, np.float32)
    out_b, out_s = [], []
    begin = 0
    for L in np.unique(cells[:, 3]):
        sel = np.nonzero(cells[:, 3] == L)[0]
        q = cells[sel, :3] >> int(L)
        order = np.lexsort((q[:, 0], q[:, 1], q[:, 2]))
        q, idx = q[order], sel[order]
        cont = np.zeros(len(q), bool)
        cont[1:] = ((q[1:, 2] == q[:-1, 2]) & (q[1:, 1] == q[:-1, 1]) & (q[1:, 0] == q[:-1, 0] + 1) &
                    (q[1:, 0] // max_len == q[:-1, 0] // max_len))
        starts = np.nonzero(~cont)[0]
        lens = np.diff(np.append(starts, len(q)))
        b = np.zeros(len(starts), BRICK_DTYPE)
        b["lower"] = q[starts] << int(L)
        b["size"][:, 0] = lens
        b["size"][:, 1:] = 1
        b["level"] = L
        b["begin"] = begin + starts
        begin += len(q)
        out_b.append(b)
        out_s.append(scalars[idx])
    if not out_b:
        return np.zeros(0, BRICK_DTYPE), np.zeros(0, np.float32)
    return np.concatenate(out_b), np.concatenate(out_s)



def main(argv=None):
    """Writes a configuration's dual-mesh arrays (vertices, indices,
    gridlets, gridlet_scalars) to an uncompressed .npz file:
        python -m owlexastitcher_gb300.datagen --config medium --out medium.npz"""
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="small")
    ap.add_argument("--out", required=True)
    ap.add_argument("--balance", type=int, default=None)
    a = ap.parse_args(argv)
    kw = {} if a.balance is None else {"balance": a.balance}
    ds = Dataset(a.config, **kw)
    with open(a.out, "wb") as f:
        np.savez(f, vertices=ds.vertices, indices=ds.indices, gridlets=ds.gridlets,
                 gridlet_scalars=ds.gridlet_scalars)


if __name__ == "__main__":
    main()
