"""Live cross-check of the oracle against the reference headers compiled
in oracle/_ref (only where the reference tree was available to build it)."""
import numpy as np
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def ref(oracle):
    if oracle.ref() is None:
        pytest.skip("oracle/_ref not built here (reference tree absent)")
    return oracle


def test_random_elements_live(ref):
    rng = np.random.default_rng(99)
    from golden.make_golden import SHAPES
    for nv, base in SHAPES.items():
        for _ in range(300):
            V = np.zeros((nv, 4), np.float32)
            V[:, :3] = (base + rng.normal(0, 0.1, base.shape)) * rng.uniform(0.5, 8)
            V[:, 3] = rng.uniform(0, 1, nv)
            P = rng.uniform(V[:, :3].min(0), V[:, :3].max(0)).astype(np.float32)
            a, b = ref.intersect_elem(P, V), ref.ref_intersect_elem(P, V)
            assert a[0] == b[0] and (not a[0] or np.float32(a[1]).tobytes() == np.float32(b[1]).tobytes())


def test_dataset_gridlets_live(ref):
    from conftest import dataset
    d = dataset("tiny")
    rng = np.random.default_rng(3)
    for gi in range(len(d.gridlets)):
        g = d.gridlets[gi]
        cw = 2.0 ** g["level"]
        lo, hi = (g["lower"] + 0.5) * cw, (g["lower"] + g["dims"] + 0.5) * cw
        for p in rng.uniform(lo, hi, (50, 3)).astype(np.float32):
            a = ref.intersect_gridlet(p, g, d.gridlet_scalars)
            b = ref.ref_intersect_gridlet(p, g, d.gridlet_scalars)
            assert a[0] == b[0] and (not a[0] or (a[2] == b[2] and np.float32(a[1]).tobytes() == np.float32(b[1]).tobytes()))


def test_dda_rays_from_outside_live(ref):
    """rays that start outside the grid box (as camera rays do), with tmin > 0
    for half of them and a direction component of 1e-6 for some: the cells and
    their entry / exit distances equal DDA.h's bit for bit (the golden
    vectors start every ray inside the box)"""
    rng = np.random.default_rng(7)
    cells = 0
    for i in range(600):
        dims = rng.integers(1, 40, 3).astype(np.int32)
        lo = rng.uniform(-10, 10, 3).astype(np.float32)
        hi = (lo + rng.uniform(1, 100, 3)).astype(np.float32)
        org = rng.uniform(lo - (hi - lo), hi + (hi - lo)).astype(np.float32)
        d = rng.uniform(lo, hi).astype(np.float64) - org
        d = (d / np.linalg.norm(d)).astype(np.float32)
        if i % 7 == 0:
            d[rng.integers(0, 3)] = np.float32(1e-6)
        tmin = np.float32(0.0 if i % 2 else rng.uniform(0, 20))
        tmax = np.float32(1e10 if i % 3 else rng.uniform(0, 150))
        a = ref.dda3(org, d, tmin, tmax, dims, lo, hi, 1024)
        b = ref.ref_dda3(org, d, tmin, tmax, dims, lo, hi, 1024)
        assert np.array_equal(a[0], b[0]), i
        assert a[1].tobytes() == b[1].tobytes() and a[2].tobytes() == b[2].tobytes(), i
        cells += len(b[0])
    assert cells > 10000


def test_degenerate_elements_live(ref):
    """flattened, collapsed and twisted elements (the Newton inversion may stop
    at its iteration cap): the oracle's hit flag and value equal the
    reference headers' bit for bit; the GPU test of the same elements
    compares the CUDA path with the oracle"""
    from test_gpu_elements_golden import degenerate_elements
    hits = 0
    for nv in (4, 5, 6, 8):
        V, P = degenerate_elements(np.random.default_rng(31), nv, 1024)
        for i in range(len(V)):
            for p in P[i]:
                a, b = ref.intersect_elem(p, V[i]), ref.ref_intersect_elem(p, V[i])
                assert a[0] == b[0], (nv, i, p)
                assert not a[0] or np.float32(a[1]).tobytes() == np.float32(b[1]).tobytes(), (nv, i, p)
                hits += bool(b[0])
    assert hits > 1000


def test_extreme_gridlets_live(ref):
    """gridlets of levels up to 19 at lattice coordinates of +-5000 with NaN
    holes and signed zeros; points inside, on faces and corners, on cell
    planes, around the box, and with a NaN or infinite coordinate: the hit,
    the cell and the value's bits equal Gridlet.h's"""
    rng = np.random.default_rng(9)
    hits = 0
    for i in range(4000):
        g = np.zeros(1, ref.GRIDLET_DTYPE)[0]
        dims = rng.integers(0, 9, 3)
        level = int(rng.integers(0, 20))
        lower = rng.integers(-5000, 5000, 3)
        g["lower"], g["level"], g["dims"], g["begin"] = lower, level, dims, 0
        ns = int(np.prod(dims + 1))
        sc = rng.uniform(-1, 1, ns).astype(np.float32)
        sc[rng.uniform(size=ns) < 0.15] = np.nan
        if i % 9 == 0:
            sc[rng.uniform(size=ns) < 0.5] = -0.0
        cw = float(2 ** level)
        lo, hi = (lower + 0.5) * cw, (lower + dims + 0.5) * cw
        k = i % 5
        if k == 0:
            p = rng.uniform(lo, hi)
        elif k == 1:
            p = np.where(rng.random(3) < 0.5, lo, hi)
        elif k == 2:
            p = lo + cw * rng.integers(0, 9, 3)
        elif k == 3:
            p = rng.uniform(lo, hi)
            p[rng.integers(0, 3)] = [np.nan, np.inf, -np.inf][i % 3]
        else:
            p = rng.uniform(lo - cw, hi + cw)
        p = p.astype(np.float32)
        a, b = ref.intersect_gridlet(p, g, sc), ref.ref_intersect_gridlet(p, g, sc)
        assert a[0] == b[0], (i, p)
        assert not a[0] or (a[2] == b[2] and np.float32(a[1]).tobytes() == np.float32(b[1]).tobytes()), (i, p)
        hits += bool(b[0])
    assert hits > 500


def test_extreme_projections_live(ref):
    """projectOnGrid for boxes of 1e-3 to 1e5 units at +-1e4, grids with a
    single cell along an axis, and points far outside, up to 1e30, exactly on
    the box and on cell faces: the cell equals Grid.cuh's"""
    rng = np.random.default_rng(4)
    for i in range(4000):
        dims = rng.integers(1, 512, 3).astype(np.int32)
        if i % 5 == 0:
            dims[rng.integers(0, 3)] = 1
        lo = rng.uniform(-1e4, 1e4, 3).astype(np.float32)
        ext = np.float32(10.0) ** rng.uniform(-3, 5, 3)
        hi = (lo + ext).astype(np.float32)
        k = i % 4
        if k == 0:
            V = rng.uniform(lo - 10 * ext, hi + 10 * ext)
        elif k == 1:
            V = rng.uniform(-1e30, 1e30, 3)
        elif k == 2:
            V = np.where(rng.random(3) < 0.5, lo, hi)
        else:
            V = lo + ext * rng.integers(0, 8, 3) / 7.0
        V = V.astype(np.float32)
        assert ref.project_on_grid(V, dims, lo, hi) == ref.ref_project_on_grid(V, dims, lo, hi), (i, V)
