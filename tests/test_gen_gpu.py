"""The GPU version of the dual-mesh generator (exa_gen_run_gpu) against the
CPU restatement of tools/amrMakeDualMesh (exa_gen_run): identical arrays
and statistics, bit for bit, over field kinds, level counts, root shapes
that fill neither whole bit-set words nor whole 8^3 macrocells, and with
the 2:1 balance on and off."""
import numpy as np
import pytest

from conftest import dataset

pytestmark = pytest.mark.gpu

CASES = [
    ("tiny", {}),
    ("small", {}),
    ("small", {"balance": 0}),
    ("small", {"numLevels": 1}),
    ("small", {"rootDims": (5, 7, 3), "numLevels": 4, "refineThreshold": 0.3}),
    ("cloud", {"rootDims": (48, 40, 36), "numLevels": 4}),
    ("cloud", {"rootDims": (64, 64, 64)}),
    ("medium", {}),
]


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.parametrize("config,kw", CASES, ids=[f"{c}-{'-'.join(f'{k}{v}' for k, v in kw.items())}" for c, kw in CASES])
def test_gpu_generator_bit_exact(cuda, native, config, kw):
    a = dataset(config, **kw)
    b = dataset(config, device=0, **kw)
    for k in ("vertices", "indices", "gridlet_scalars", "amr_cells", "amr_scalars"):
        x, y = getattr(a, k), getattr(b, k)
        assert x.shape == y.shape, k
        assert x.tobytes() == y.tobytes(), k
    assert a.gridlets.tobytes() == b.gridlets.tobytes()
    for k, v in a.stats.items():
        if k in ("seconds", "stageSeconds"):
            continue
        assert b.stats[k] == v, k
    assert a.stats["numAmrCells"] > 0 and len(a.gridlets) > 0
    if config != "tiny" and kw.get("numLevels", 2) > 1:
        assert len(a.indices) > 0
