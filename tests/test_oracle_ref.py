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
