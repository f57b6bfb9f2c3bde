"""The double-float coefficients of the erfc series the FP32 forms use for near
Coulomb pairs (aleator_gb300/csrc/ff.cuh, kErfSeries): d_n = (-1)^n (2 /
sqrt(pi)) 4^n / (n! (2n + 1)), so that erf(x) = x sum_n d_n (x^2 / 4)^n
(the Maclaurin series). Checked on the host: each (hi, lo) pair equals d_n
within 2^-48 relative (two FP32 significands), and the 30-term sum gives erf within 1e-14 over the
series' range [0, 2] (the device evaluates the same sum in double-float;
tests/test_gpu_ff_near.py checks that against FP64 erfc)."""
import math
import re
from fractions import Fraction
from pathlib import Path

import numpy as np

HDR = Path(__file__).resolve().parents[1] / "aleator_gb300" / "csrc" / "ff.cuh"


def _coefficients():
    text = HDR.read_text()
    body = text[text.index("kErfSeries["):]
    body = body[body.index("{") + 1:body.index("};")]
    pairs = re.findall(r"\{\s*([-+0-9a-fA-Fx.p]+)f\s*,\s*([-+0-9a-fA-Fx.p]+)f\s*\}", body)
    return [(float.fromhex(h), float.fromhex(l)) for h, l in pairs]


def _exact(n):
    # 2 / sqrt(pi) to 30 digits times the rational part
    two_over_sqrt_pi = Fraction("1.128379167095512573896158903121545171688")
    return float(two_over_sqrt_pi * Fraction((-1) ** n * 4 ** n, math.factorial(n) * (2 * n + 1)))


def test_coefficients_are_the_series():
    c = _coefficients()
    assert len(c) == 30
    for n, (hi, lo) in enumerate(c):
        assert np.float32(hi) == hi and np.float32(lo) == lo  # FP32 pairs
        want = _exact(n)
        assert abs((hi + lo) - want) <= 2.0 ** -48 * abs(want), n


def test_series_sums_to_erf_over_its_range():
    c = [hi + lo for hi, lo in _coefficients()]
    worst = 0.0
    for x in np.linspace(0.0, 2.0, 2001):
        w = x * x / 4.0
        s = 0.0
        for d in reversed(c):
            s = s * w + d
        worst = max(worst, abs(x * s - math.erf(x)))
    assert worst <= 1e-14, worst
