"""Project-written log / sincos used on the free-flight and phase-function
path (both sides of the parity check use them): accuracy against binary64."""
import numpy as np


def test_log_accuracy(oracle):
    rng = np.random.default_rng(0)
    u = rng.integers(0, 1 << 24, 50000)
    x = (1.0 - u * 2.0 ** -24).astype(np.float32)          # the free-flight argument 1-u
    x = np.concatenate([x, np.float32([1.0, 2.0 ** -24, 0.5, 0.70710677, 1.4142135]),
                        rng.uniform(1e-30, 1e30, 2000).astype(np.float32)])
    ours = np.array([oracle.log(v) for v in x], np.float64)
    ref = np.log(x.astype(np.float64))
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    err = np.abs(ours - ref) / np.where(ref == 0, 1, ulp)
    assert err[ref != 0].max() < 2.0
    assert ours[x == 1.0][0] == 0.0


def test_sincos_accuracy(oracle):
    u = np.concatenate([np.linspace(0, 1, 4001, endpoint=False), np.random.default_rng(1).uniform(0, 1, 20000)])
    u = u.astype(np.float32)
    sc = np.array([oracle.sincos_turns(v) for v in u])
    th = 2 * np.pi * u.astype(np.float64)
    assert np.abs(sc[:, 0] - np.sin(th)).max() < 2e-7
    assert np.abs(sc[:, 1] - np.cos(th)).max() < 2e-7
    assert np.abs(sc[:, 0] ** 2 + sc[:, 1] ** 2 - 1).max() < 1e-6
