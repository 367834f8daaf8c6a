"""Generates the golden vectors in tests/golden/ from the reference's own
sampling headers (Gridlet.h, Plane.h, UElems.h, Grid.cuh, DDA.h) compiled
unmodified into oracle/_ref/libexaref.so (see oracle/Makefile).

    python tests/golden/make_golden.py

Each fixture stores seeded inputs and the reference outputs; the oracle and
(through the oracle) the CUDA path are checked against them where the
reference tree is absent.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import pyoracle as O  # noqa: E402

SHAPES = {
    4: np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32),
    5: np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0.5, 0.5, 1]], np.float32),
    6: np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [0, 1, 1]], np.float32),
    8: np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], np.float32),
}


def elements(rng, n_per_type=400):
    out = {}
    for nv, base in SHAPES.items():
        V = np.zeros((n_per_type, nv, 4), np.float32)
        P = np.zeros((n_per_type, 3), np.float32)
        hit = np.zeros(n_per_type, np.int32)
        val = np.zeros(n_per_type, np.float32)
        for i in range(n_per_type):
            V[i, :, :3] = (base + rng.normal(0, 0.08, base.shape)) * rng.uniform(0.5, 4) + rng.uniform(-50, 50, 3)
            V[i, :, 3] = rng.uniform(-1, 1, nv)
            lo, hi = V[i, :, :3].min(0), V[i, :, :3].max(0)
            if i % 4 == 0:  # a vertex or an edge midpoint: boundary cases
                a, b = rng.integers(0, nv, 2)
                P[i] = 0.5 * (V[i, a, :3] + V[i, b, :3])
            else:
                P[i] = rng.uniform(lo, hi)
            h, v = O.ref_intersect_elem(P[i], V[i])
            hit[i], val[i] = h, v if h else 0.0
        out[nv] = (V, P, hit, val)
    return out


def gridlets(rng, n=600):
    G = np.zeros(n, O.GRIDLET_DTYPE)
    S = []
    P = np.zeros((n, 3), np.float32)
    hit = np.zeros(n, np.int32)
    val = np.zeros(n, np.float32)
    cell = np.zeros(n, np.int32)
    off = 0
    for i in range(n):
        dims = rng.integers(1, 9, 3)
        level = int(rng.integers(0, 5))
        lower = rng.integers(0, 64, 3)
        ns = int(np.prod(dims + 1))
        sc = rng.uniform(-1, 1, ns).astype(np.float32)
        sc[rng.uniform(size=ns) < 0.08] = np.nan
        G[i]["lower"], G[i]["level"], G[i]["dims"], G[i]["begin"] = lower, level, dims, off
        cw = float(2 ** level)
        lo, hi = (lower + 0.5) * cw, (lower + dims + 0.5) * cw
        if i % 5 == 0:  # on a face / the upper boundary
            P[i] = rng.uniform(lo, hi)
            ax = rng.integers(0, 3)
            P[i, ax] = (hi if i % 10 == 0 else lo + cw * rng.integers(0, dims[ax] + 1))[ax] if i % 10 == 0 else lo[ax] + cw * rng.integers(0, dims[ax] + 1)
        else:
            P[i] = rng.uniform(lo - 0.2 * cw, hi + 0.2 * cw)
        S.append(sc)
        g1 = G[i].copy()
        g1["begin"] = 0
        h, v, c = O.ref_intersect_gridlet(P[i], g1, sc)
        hit[i], val[i], cell[i] = h, (v if h else 0.0), (c if h else -1)
        off += ns
    return G, np.concatenate(S), P, hit, val, cell


def ddas(rng, n=400, max_cells=512):
    rows = []
    for i in range(n):
        dims = rng.integers(1, 40, 3).astype(np.int32)
        lo = rng.uniform(-10, 10, 3).astype(np.float32)
        hi = (lo + rng.uniform(1, 100, 3)).astype(np.float32)
        org = rng.uniform(lo, hi).astype(np.float32)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        d = d.astype(np.float32)
        if i % 5 == 0:
            d[rng.integers(0, 3)] = np.float32(1e-5)
        tmax = np.float32(1e10 if i % 3 else rng.uniform(0, 50))
        ids, t0, t1 = O.ref_dda3(org, d, 0.0, tmax, dims, lo, hi, max_cells)
        rows.append((dims, lo, hi, org, d, tmax, ids, t0, t1))
    return rows


def projections(rng, n=2000):
    dims = rng.integers(1, 300, (n, 3)).astype(np.int32)
    lo = rng.uniform(-10, 10, (n, 3)).astype(np.float32)
    hi = (lo + rng.uniform(1, 100, (n, 3))).astype(np.float32)
    V = rng.uniform(lo - 5, hi + 5).astype(np.float32)
    out = np.array([O.ref_project_on_grid(V[i], dims[i], lo[i], hi[i]) for i in range(n)], np.int32)
    return dims, lo, hi, V, out


def main():
    O.build(ref=True)
    if O.ref() is None:
        raise SystemExit("oracle/_ref/libexaref.so is not built (the reference tree is required)")
    rng = np.random.default_rng(20231203)
    el = elements(rng)
    np.savez_compressed(os.path.join(HERE, "elements.npz"),
                        **{f"{k}_{n}": a for n, (V, P, h, v) in el.items() for k, a in
                           (("V", V), ("P", P), ("hit", h), ("val", v))})
    G, S, P, h, v, c = gridlets(rng)
    np.savez_compressed(os.path.join(HERE, "gridlets.npz"), gridlets=G, scalars=S, P=P, hit=h, val=v, cell=c)
    rows = ddas(rng)
    np.savez_compressed(
        os.path.join(HERE, "dda.npz"),
        dims=np.array([r[0] for r in rows]), lo=np.array([r[1] for r in rows]), hi=np.array([r[2] for r in rows]),
        org=np.array([r[3] for r in rows]), dir=np.array([r[4] for r in rows]),
        tmax=np.array([r[5] for r in rows], np.float32), counts=np.array([len(r[6]) for r in rows], np.int32),
        ids=np.concatenate([r[6] for r in rows]), t0=np.concatenate([r[7] for r in rows]),
        t1=np.concatenate([r[8] for r in rows]))
    dims, lo, hi, V, out = projections(rng)
    np.savez_compressed(os.path.join(HERE, "project.npz"), dims=dims, lo=lo, hi=hi, V=V, out=out)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
