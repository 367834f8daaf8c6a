"""The staging plan of the majorant build kernel (brick_plan in
owlexastitcher_gb300/csrc/exa_build.cu), restated and checked on the CPU
over random bricks: the bulk copy starts and ends on 16-byte boundaries,
stays inside the scalar buffer and the staging buffer, and together with
the thread-loaded tail covers the brick exactly.  The GPU parity tests
(test_majorant_build.py) check the kernel itself."""
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
