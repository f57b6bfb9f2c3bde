"""Vectorised host-side Philox4x32-10 streams (numpy, integer-exact).

Same bijection and stream layout as the device generator and as the
reference's Philox4x32Rng (counter_based_rng.cc:13-79): key = (seed lo, seed
hi), counter = (call lo, call hi, stream lo, stream hi), u64 = out0 << 32 |
out1, uniform = (u64 >> 11) * 2^-53. Used to generate seeded synthetic
workloads identically on every host.
"""
from __future__ import annotations

import numpy as np

_M0 = np.uint64(0xD2511F53)
_M1 = np.uint64(0xCD9E8D57)
_W0 = np.uint32(0x9E3779B9)
_W1 = np.uint32(0xBB67AE85)
_MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    c0, c1, c2, c3 = (np.asarray(v, dtype=np.uint32) for v in (c0, c1, c2, c3))
    k0 = np.asarray(k0, dtype=np.uint32)
    k1 = np.asarray(k1, dtype=np.uint32)
    with np.errstate(over="ignore"):
        for r in range(10):
            if r > 0:
                k0 = (k0 + _W0).astype(np.uint32)
                k1 = (k1 + _W1).astype(np.uint32)
            p0 = _M0 * c0.astype(np.uint64)
            p1 = _M1 * c2.astype(np.uint64)
            hi0 = (p0 >> np.uint64(32)).astype(np.uint32)
            lo0 = (p0 & _MASK).astype(np.uint32)
            hi1 = (p1 >> np.uint64(32)).astype(np.uint32)
            lo1 = (p1 & _MASK).astype(np.uint32)
            c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
    return c0, c1, c2, c3


def u64(seed: int, stream: int, first: int, n: int) -> np.ndarray:
    calls = np.arange(first, first + n, dtype=np.uint64)
    c0 = (calls & _MASK).astype(np.uint32)
    c1 = (calls >> np.uint64(32)).astype(np.uint32)
    c2 = np.full(n, stream & 0xFFFFFFFF, dtype=np.uint32)
    c3 = np.full(n, (stream >> 32) & 0xFFFFFFFF, dtype=np.uint32)
    o0, o1, _, _ = philox4x32_10(c0, c1, c2, c3, np.uint32(seed & 0xFFFFFFFF),
                                 np.uint32((seed >> 32) & 0xFFFFFFFF))
    return (o0.astype(np.uint64) << np.uint64(32)) | o1.astype(np.uint64)


def uniforms(seed: int, stream: int, first: int, n: int) -> np.ndarray:
    return (u64(seed, stream, first, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
