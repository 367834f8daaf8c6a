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
