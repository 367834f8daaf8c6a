"""The oracle's restatement against golden vectors produced by the
reference's own headers (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def bits(x):
    return np.float32(x).tobytes()


@pytest.mark.parametrize("nv", [4, 5, 6, 8])
def test_elements_match_reference(oracle, nv):
    g = np.load(os.path.join(GOLD, "elements.npz"))
    V, P, hit, val = g[f"V_{nv}"], g[f"P_{nv}"], g[f"hit_{nv}"], g[f"val_{nv}"]
    assert hit.sum() > 20  # the fixture exercises both outcomes
    for i in range(len(P)):
        h, v = oracle.intersect_elem(P[i], V[i])
        assert h == bool(hit[i]), i
        if h:
            assert bits(v) == bits(val[i]), (i, v, val[i])


def test_gridlets_match_reference(oracle):
    g = np.load(os.path.join(GOLD, "gridlets.npz"))
    G, S = g["gridlets"], g["scalars"]
    for i in range(len(G)):
        h, v, c = oracle.intersect_gridlet(g["P"][i], G[i], S)
        assert h == bool(g["hit"][i]), i
        if h:
            assert bits(v) == bits(g["val"][i]) and c == g["cell"][i], i


def test_dda_matches_reference(oracle):
    g = np.load(os.path.join(GOLD, "dda.npz"))
    off = 0
    for i in range(len(g["counts"])):
        n = int(g["counts"][i])
        ids, t0, t1 = oracle.dda3(g["org"][i], g["dir"][i], 0.0, g["tmax"][i], g["dims"][i], g["lo"][i], g["hi"][i], 512)
        assert len(ids) == n, i
        assert np.array_equal(ids, g["ids"][off:off + n]), i
        assert t0.tobytes() == g["t0"][off:off + n].tobytes(), i
        assert t1.tobytes() == g["t1"][off:off + n].tobytes(), i
        off += n


def test_project_on_grid_matches_reference(oracle):
    g = np.load(os.path.join(GOLD, "project.npz"))
    for i in range(len(g["V"])):
        assert oracle.project_on_grid(g["V"][i], g["dims"][i], g["lo"][i], g["hi"][i]) == tuple(g["out"][i]), i
