"""The FP32 forms' near Coulomb pairs (within 6 A of a site) take their
real-space term q erfc(alpha r) / r in double-float on the FP32 pipe:
erfc from its Maclaurin series (ff.cuh ff_erfc), sqrt and 1 / r by one Newton
step each. Checked against FP64 on the host (math.erfc): erfc within 1e-11
relative over [0, 2] (erf to ~1e-14; 1 - erf, down to 0.0047 at x = 2,
loses up to 8 bits of it); the pair term within 1e-11 relative over the
near range (a pair closer than 1e-5 A, clamped as in FP64, only finite),
and NaN (the kernels' FP64 fallback) where alpha r lies beyond 2."""
import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(lib, mode, data, n, alpha=0.0):
    A, _ = lib
    L = A.load_library()
    out = np.zeros(n)
    data = np.ascontiguousarray(data, dtype=np.float64)
    dp = ctypes.POINTER(ctypes.c_double)
    assert L.alea_test_ff_near(mode, data.ctypes.data_as(dp), out.ctypes.data_as(dp), n, alpha) == 0
    return out


def test_erfc_series_matches_fp64(lib):
    x = np.concatenate([np.linspace(0.0, 2.0, 4001), np.random.default_rng(1).uniform(0, 2, 4000)])
    got = _run(lib, 0, x, len(x))
    want = np.array([math.erfc(v) for v in x])
    rel = np.abs(got - want) / want
    assert rel.max() <= 1e-11, (rel.max(), x[np.argmax(rel)])


@pytest.mark.parametrize("alpha", [0.3097, 0.25, 0.33])
def test_near_pair_term_matches_fp64(lib, alpha):
    rng = np.random.default_rng(int(alpha * 1e4))
    n = 20000
    r = np.concatenate([rng.uniform(1e-3, 6.0, n - 3), [1e-7, 6.0, 2.0 / alpha + 0.01]])
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    d = u * r[:, None]
    q = rng.uniform(-1.2, 1.2, n)
    data = np.column_stack([d, q])
    got = _run(lib, 1, data, n, alpha)
    rr = np.maximum(np.linalg.norm(d, axis=1), 1e-6)
    want = q * np.array([math.erfc(alpha * v) for v in rr]) / rr
    inside = alpha * rr <= 2.0 - 1e-6
    assert np.isnan(got[alpha * rr > 2.0 + 1e-6]).all()
    assert np.isfinite(got[inside]).all()
    ok = inside & (rr > 1e-5)
    assert ok.sum() >= n - 50
    rel = np.abs(got[ok] - want[ok]) / np.abs(want[ok])
    assert rel.max() <= 1e-11, rel.max()
