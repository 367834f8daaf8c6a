"""The listing rules of the point-location structures, restated on the CPU
(the GPU tests check the kernels' answers against the oracle):

* gridlet block tables (exa_api.cpp buildGridletTables, exa_accel.cuh
  table_block / query_table): a gridlet is listed in every block whose open
  interior meets its closed extent, blocks start on multiples of their
  width, and a query exactly on a block's low face also looks at the block
  below -- so every gridlet whose closed box holds a point is among the
  candidates the query looks at, for any block width and origin;
* element cells (exa_build.cu k_elem_cells_*, exa_accel.cuh
  elem_cell_entry): an element is listed in every cell its closed AABB
  touches by cell(p) = floor((p - origin) * (1 / width)), the width a power
  of two, so the multiplication is the exact quotient and the mapping is
  monotonic: a point inside an element's AABB maps to a cell that lists it."""
import numpy as np


def table_candidates(gl, lt, shift, origin, p):
    """the gridlets a query at p looks at: the lists of its block and, on a
    block's low face, of the block below (doubled lattice units, as the
    builder computes extents)"""
    w = 1 << shift
    u = p / (1 << lt) - 0.5
    fu = np.floor(u)
    b0, nb = [], []
    for a in range(3):
        iu = int(fu[a]) - origin[a]
        b = iu >> shift
        face = fu[a] == u[a] and (iu & (w - 1)) == 0
        b0.append(b - 1 if face else b)
        nb.append(2 if face else 1)
    out = set()
    for gi, (lower, level, dims) in enumerate(gl):
        r = 1 << (level - lt)
        lo2 = [(2 * lower[a] + 1) * r - 1 for a in range(3)]
        hi2 = [(2 * (lower[a] + max(dims[a], 1)) + 1) * r - 1 for a in range(3)]
        w2 = 2 * w
        bl = [(lo2[a] - 2 * origin[a]) // w2 for a in range(3)]
        bh = [(hi2[a] - 2 * origin[a] + w2 - 1) // w2 - 1 for a in range(3)]
        hit = all(any(bl[a] <= b0[a] + k <= bh[a] for k in range(nb[a])) for a in range(3))
        if hit:
            out.add(gi)
    return out


def contains(g, p):
    lower, level, dims = g
    cw = float(1 << level)
    lo = (np.array(lower, np.float64) + 0.5) * cw
    hi = (np.array(lower, np.float64) + np.array(dims, np.float64) + 0.5) * cw
    return bool(np.all(lo <= p) and np.all(p <= hi))


def test_gridlet_table_lists_every_containing_gridlet():
    rng = np.random.default_rng(17)
    for trial in range(40):
        lt = 0
        gl = []
        for _ in range(12):
            level = int(rng.integers(0, 3))
            lower = [int(v) for v in rng.integers(-6, 10, 3)]
            dims = [int(v) for v in rng.integers(0, 9, 3)]
            gl.append((lower, level, dims))
        shift = int(rng.choice([3, 4]))
        # the builder's origin: the lowest extent, rounded down to the block width
        lo = min(min(((2 * g[0][a] + 1) * (1 << g[1]) - 1) // 2 for a in range(3)) for g in gl)
        origin = [(lo >> shift) << shift] * 3
        pts = []
        for g in gl:
            lower, level, dims = g
            cw = float(1 << level)
            lo_b = (np.array(lower) + 0.5) * cw
            hi_b = (np.array(lower) + np.array(dims) + 0.5) * cw
            pts.append(rng.uniform(lo_b, hi_b + 1e-9, (6, 3)))
            pts.append(np.where(rng.random((6, 3)) < 0.5, lo_b, hi_b))  # corners and faces
        for p in np.concatenate(pts):
            want = {i for i, g in enumerate(gl) if contains(g, p)}
            got = table_candidates(gl, lt, shift, origin, p)
            assert want <= got, (trial, p, want - got)


def test_element_cells_hold_every_element_aabb():
    rng = np.random.default_rng(23)
    for _ in range(30):
        n = 40
        lo = rng.uniform(-20, 20, (n, 3)).astype(np.float32)
        hi = (lo + rng.exponential(2.0, (n, 3))).astype(np.float32)
        origin = lo.min(axis=0)
        width = np.float32(2.0 ** int(rng.integers(1, 4)))
        inv = np.float32(1.0) / width
        assert inv * width == 1 and np.float32(1.0) / inv == width
        ncell = (np.ceil((hi.max(axis=0) - origin) / width) + 1).astype(np.int64)

        def cell(p):
            return np.clip(np.floor((p - origin) * inv).astype(np.int64), -1, ncell)

        lists = {}
        for e in range(n):
            c0 = np.maximum(cell(lo[e]), 0)
            c1 = np.minimum(cell(hi[e]), ncell - 1)
            for z in range(c0[2], c1[2] + 1):
                for y in range(c0[1], c1[1] + 1):
                    for x in range(c0[0], c1[0] + 1):
                        lists.setdefault((x, y, z), []).append(e)
        for e in range(n):
            P = rng.uniform(lo[e], hi[e], (20, 3)).astype(np.float32)
            P = np.concatenate([P, lo[e][None], hi[e][None]])
            for p in P:
                # the multiplication by the power-of-two reciprocal is the
                # division the cell mapping is defined by
                assert np.array_equal(np.floor((p - origin) * inv), np.floor((p - origin) / width))
                assert e in lists.get(tuple(int(v) for v in cell(p)), []), (e, p)
