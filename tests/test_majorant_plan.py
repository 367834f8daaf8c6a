"""The staging plan of the majorant build kernel (brick_plan in
owlexastitcher_gb300/csrc/exa_build.cu), restated and checked on the CPU
over random bricks: the bulk copy starts and ends on 16-byte boundaries,
stays inside the scalar buffer and the staging buffer, and together with
the thread-loaded tail covers the brick exactly.  The GPU parity tests
(test_majorant_build.py) check the kernel itself."""
import warnings

import numpy as np

K_BRICK_CAP = 736  # floats per staging buffer (kBrickCap)


def brick_plan(begin, dims, n_scalars, stage=True):
    n = (dims[0] + 1) * (dims[1] + 1) * (dims[2] + 1)
    s0, s1 = begin, begin + n
    f0 = s0 & ~3
    lead = s0 - f0
    staged = stage and s1 - f0 + 3 <= K_BRICK_CAP
    f1 = (s1 + 3) & ~3
    fend = n_scalars & ~3
    if f1 > fend:
        f1 = fend if fend > f0 else f0
    bulk = (f1 - f0) * 4 if staged else 0
    tail = s1 - f1 if staged and s1 > f1 else 0
    return f0, bulk, lead, tail, staged, n


def test_brick_plan_bounds():
    rng = np.random.default_rng(3)
    staged_cases = tail_cases = tail_only = unstaged = 0
    for _ in range(100000):
        dims = tuple(int(d) for d in rng.integers(0, 13, 3))
        n = (dims[0] + 1) * (dims[1] + 1) * (dims[2] + 1)
        begin = int(rng.integers(0, 1 << 20))
        # often place the brick at the very end of the buffer
        n_scalars = begin + n + (0 if rng.random() < 0.5 else int(rng.integers(0, 9)))
        f0, bulk, lead, tail, staged, n = brick_plan(begin, dims, n_scalars)
        if not staged:
            unstaged += 1
            assert bulk == 0 and tail == 0
            continue
        staged_cases += 1
        assert f0 % 4 == 0 and bulk % 16 == 0        # 16-byte aligned source (256-byte aligned base) and size
        assert f0 * 4 + bulk <= n_scalars * 4         # the copy stays inside the scalar buffer
        assert bulk // 4 + tail <= K_BRICK_CAP        # ... and inside the staging buffer
        assert f0 <= begin and lead == begin - f0 and 0 <= lead < 4
        if bulk:
            assert f0 + bulk // 4 + tail >= begin + n  # the brick is covered
        assert f0 + bulk // 4 + tail <= n_scalars     # thread loads stay inside the buffer
        if tail:
            tail_cases += 1
            assert f0 + bulk // 4 + tail == begin + n
            assert tail <= 3 or bulk == 0
            if bulk == 0:
                tail_only += 1
    assert staged_cases and tail_cases and tail_only and unstaged


def test_brick_plan_covers_8cubed_at_any_alignment():
    for lead in range(4):
        for extra in range(4):
            begin = 4096 + lead
            f0, bulk, _, tail, staged, n = brick_plan(begin, (8, 8, 8), begin + 729 + extra)
            assert staged and n == 729
            assert f0 + bulk // 4 + tail >= begin + n and bulk // 4 + tail <= K_BRICK_CAP


# --- the separable form of the build (k_gridlet_majorants_sep) -----------
K_SEP_WIN = 9      # kSepWin
K_SEP_POOL = 729   # kSepPool (the x step's results)


def _axis_ranges(rng, d):
    """per cell index of one axis its macrocell interval [m0, m1], from the
    inclusive overlap test of cells [c, c + w] with unit macrocells, as
    Grid.cu:172-183 tests per axis; sometimes clamped to a grid that ends
    inside the gridlet (cells past its end reach no macrocell)"""
    w = float(rng.choice([0.25, 0.5, 1.0, 2.0]))
    off = float(rng.uniform(0, 4)) if rng.random() < 0.7 else float(rng.integers(0, 4))  # also on boundaries
    n = int(rng.integers(2, 8)) if rng.random() < 0.2 else 1 << 20
    out = []
    for i in range(d):
        clo, chi = off + i * w, off + (i + 1) * w
        m0, m1 = int(np.ceil(clo - 1)), min(int(np.floor(chi)), n - 1)
        out.append((m0, m1) if m0 <= m1 else (0, -1))
    return out


def _per_cell(vals, R):
    """the per-cell loop: every cell updates the macrocells of its per-axis
    ranges with the min / max of its non-NaN corners"""
    out = {}
    nz, ny, nx = vals.shape
    for k in range(nz - 1):
        for j in range(ny - 1):
            for i in range(nx - 1):
                c = vals[k:k + 2, j:j + 2, i:i + 2]
                if np.all(np.isnan(c)):
                    continue
                lo, hi = np.nanmin(c), np.nanmax(c)
                for mz in range(R[2][k][0], R[2][k][1] + 1):
                    for my in range(R[1][j][0], R[1][j][1] + 1):
                        for mx in range(R[0][i][0], R[0][i][1] + 1):
                            a, b = out.get((mx, my, mz), (np.inf, -np.inf))
                            out[(mx, my, mz)] = (min(a, lo), max(b, hi))
    return out


def _separable(vals, R):
    """the kernel's steps: per axis the corner interval of each window
    macrocell, then the x reduction and the y and z reductions (which the
    kernel runs as two steps or, for the widest windows, as one); None where
    the kernel sends the gridlet to the general kernel"""
    nz, ny, nx = vals.shape
    d = (nx - 1, ny - 1, nz - 1)
    if any(all(r[0] > r[1] for r in R[a]) for a in range(3)):
        return None, None
    lo_m = [min(r[0] for r in R[a] if r[0] <= r[1]) for a in range(3)]
    hi_m = [max(r[1] for r in R[a] if r[0] <= r[1]) for a in range(3)]
    w = [hi_m[a] - lo_m[a] + 1 for a in range(3)]
    if max(w) > K_SEP_WIN or w[0] * ny * nz > K_SEP_POOL:
        return None, None
    iv = []
    for a in range(3):
        ivs = []
        for off in range(w[a]):
            m = lo_m[a] + off
            js = [j for j in range(d[a] + 1)
                  if (j > 0 and R[a][j - 1][0] <= m <= R[a][j - 1][1]) or (j < d[a] and R[a][j][0] <= m <= R[a][j][1])]
            if js and js != list(range(js[0], js[-1] + 1)):
                return None, None  # a gap
            ivs.append((js[0], js[-1]) if js else (1, 0))
        iv.append(ivs)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)  # all-NaN rows
        X = np.empty((w[0], nz, ny, 2))
        for mx in range(w[0]):
            a, b = iv[0][mx]
            seg = vals[:, :, a:b + 1]
            X[mx, :, :, 0] = np.where(np.all(np.isnan(seg), axis=2), 1e30, np.nanmin(seg, axis=2)) if b >= a else 1e30
            X[mx, :, :, 1] = np.where(np.all(np.isnan(seg), axis=2), -1e30, np.nanmax(seg, axis=2)) if b >= a else -1e30
    covered = all(R[0][i][0] <= R[0][i][1] for i in range(d[0]))
    own = (X[..., 0].min(), X[..., 1].max()) if covered else None
    out = {}
    for mx in range(w[0]):
        for my in range(w[1]):
            for mz in range(w[2]):
                (ya, yb), (za, zb) = iv[1][my], iv[2][mz]
                if yb < ya or zb < za:
                    continue
                lo = X[mx, za:zb + 1, ya:yb + 1, 0].min()
                hi = X[mx, za:zb + 1, ya:yb + 1, 1].max()
                if lo <= hi:
                    out[(lo_m[0] + mx, lo_m[1] + my, lo_m[2] + mz)] = (lo, hi)
    return out, own


def test_separable_build_equals_per_cell_loop():
    """On random bricks (with NaN corners) and random per-axis macrocell
    ranges, the separable reductions give the per-cell loop's macrocell
    ranges, and the folded own range is the min / max over every scalar."""
    rng = np.random.default_rng(11)
    checked = fallback = folded = 0
    for _ in range(400):
        d = [int(v) for v in rng.integers(1, 9, 3)]
        vals = rng.normal(size=(d[2] + 1, d[1] + 1, d[0] + 1)).astype(np.float32)
        vals[rng.random(vals.shape) < 0.15] = np.nan
        R = [_axis_ranges(rng, d[a]) for a in range(3)]
        got, own = _separable(vals, R)
        if got is None:
            fallback += 1
            continue
        checked += 1
        want = _per_cell(vals, R)
        assert set(got) == set(want)
        for key in want:
            assert got[key] == want[key], key
        if own is not None:
            folded += 1
            if np.all(np.isnan(vals)):
                assert own == (1e30, -1e30)
            else:
                assert own == (np.nanmin(vals), np.nanmax(vals))
    assert checked > 200 and 150 < folded < checked and fallback > 0


def test_sep_index_division():
    """SepDiv: k / d as (k * (2^21 / d + 1)) >> 21 is exact wherever
    k * d < 2^21, and the 32-bit product does not overflow for k < 2048;
    the kernel decodes indices k < 729 with divisors d <= 81"""
    for d in range(1, 82):
        inv = (1 << 21) // d + 1
        k = np.arange(0, (1 << 21) // d + 1, dtype=np.uint64)
        k = k[k * d < (1 << 21)]
        assert np.array_equal((k * inv) >> 21, k // d), d
        assert np.all(k[k < 2048] * inv < (1 << 32))
    assert 728 * 81 < (1 << 21)
