"""The bounds-checked build (EXA_CHECKS=1, libexastitch_checks.so): every
index the kernels read through is tested before the access and a bad one
raises EXA_DEVERR_BOUNDS (exa_sync then fails) instead of reading out of
range.  compute-sanitizer is closed on this machine; this build runs the small
parity suite -- samples, majorants and bit-exact frames of all integrators
on the balanced and unbalanced small fields -- in a separate process."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_parity_suite_under_bounds_checks(native):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from owlexastitcher_gb300 import build
    lib = build.build_exastitch(variant="checks")
    assert lib.endswith("libexastitch_checks.so")
    env = dict(os.environ, EXA_LIBRARY_VARIANT="checks")
    r = subprocess.run([sys.executable, "-m", "pytest", os.path.join(ROOT, "tests", "test_gpu_parity.py"), "-m", "gpu",
                        "-q", "-x", "-k", "small", "-p", "no:cacheprovider"], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert " passed" in r.stdout and "failed" not in r.stdout
