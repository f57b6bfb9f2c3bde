"""Device Philox4x32-10 streams: bit-exact to the reference's KATs, to its
golden streams and to the oracle over a long stream (counter-indexed fill)."""
import numpy as np
import pytest

from conftest import golden
from test_oracle_golden import KAT

pytestmark = pytest.mark.gpu


def test_kat_on_device(lib):
    A, _ = lib
    out = A.philox4x32_10([k[0] for k in KAT], [k[1] for k in KAT])
    assert out.tolist() == [k[2] for k in KAT]


def test_golden_streams(lib):
    A, _ = lib
    g = golden("philox")
    assert np.array_equal(A.philox_u64(42, 0, 0, 4096), g["u64_42_0"])
    assert np.array_equal(A.philox_u64(7, 3, 1000, 1024), g["u64_7_3_skip1000"])
    assert np.array_equal(A.philox_u64(0xDEADBEEFCAFEF00D, 0x0123456789ABCDEF, (1 << 32) - 8, 64),
                          g["u64_big"])
    assert np.array_equal(A.philox_uniform(42, 0, 0, 4096), g["uniform_42_0"])
    assert np.array_equal(A.philox_uniform(2026, 999, 0, 1024), g["uniform_2026_999"])


def test_million_draws_match_oracle(lib, orc):
    A, _ = lib
    from aleator_gb300 import philox_np
    n = 1_000_000
    got = A.philox_u64(42, 0, 0, n)
    assert np.array_equal(got, philox_np.u64(42, 0, 0, n))
    # a window far along the stream, crossing the 2^32 call-index boundary
    first = (1 << 32) - 500
    assert np.array_equal(A.philox_u64(7, (1 << 33) + 1, first, 1000),
                          orc.philox_u64(7, (1 << 33) + 1, first, 1000))
    u = A.philox_uniform(7, 3, 0, n)
    assert (u >= 0).all() and (u < 1).all()
    assert np.array_equal(u, philox_np.uniforms(7, 3, 0, n))


def test_empty_and_edge(lib):
    A, _ = lib
    assert A.philox_u64(1, 1, 0, 0).size == 0
    assert np.array_equal(A.philox_u64(1, 1, (1 << 64) - 2, 2), np.array(
        [__import__("oracle").Oracle().philox_u64(1, 1, (1 << 64) - 2, 2)]).reshape(-1))
