"""The allocation-free Ewald propose entry point (alea_ewald_propose_no_alloc).

It serves callers that must not let a library allocate device memory (an
engine that owns every device buffer in its own pool, or that cannot accept the
device-wide synchronisation an allocation may imply). This test plays such a
caller: it owns the input and output buffers (made here with torch), calls the
entry point twice in a row through the C ABI, and checks each result against
the existing entry point alea_ewald_state_propose within the FP64 tolerance of
the other Ewald tests (1e-10 relative, 1 K floor). The file is collected last
so that a run stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _co2(c):
    return np.array([[c[0], c[1], c[2] - 1.16, -0.35], [c[0], c[1], c[2], 0.7],
                     [c[0], c[1], c[2] + 1.16, -0.35]])


def test_no_alloc_propose_matches_state_propose(lib):
    A, _ = lib
    import torch
    from aleator_gb300._lib import _lattice, _D

    g = golden("grid_cubic")
    alpha, kmax = 0.31, 6
    p = A.ParticleData(g["x"], g["y"], g["z"], g["charge"], g["species"])
    state = A.EwaldIncrementalState(A.Ewald(alpha, 12.0, kmax), p, g["lattice"])
    # a committed molecule, so the cache is not just the framework's
    state.commit_insertion(_co2((10.0, 11.0, 12.0)))
    k, w = A.ewald_reciprocal_terms(g["lattice"], alpha, kmax)
    raw = state.raw_state_for_testing()
    nk = len(w)
    dev = torch.device("cuda:0")
    dk = torch.tensor(k.reshape(-1), dtype=torch.float64, device=dev)
    dw = torch.tensor(w, dtype=torch.float64, device=dev)
    dre = torch.tensor(raw[:nk], dtype=torch.float64, device=dev)
    dim = torch.tensor(raw[nk:2 * nk], dtype=torch.float64, device=dev)
    out = torch.zeros(4, dtype=torch.float64, device=dev)
    lat = _lattice(g["lattice"])
    lib_ = A.load_library()
    stream = torch.cuda.current_stream().cuda_stream

    trials = [
        (np.zeros((0, 4)), _co2((3.0, 4.0, 5.0))),                  # insertion
        (_co2((10.0, 11.0, 12.0)), _co2((10.5, 11.2, 12.9))),       # move
    ]
    for removed, added in trials:
        rem = np.ascontiguousarray(removed.reshape(-1))
        add = np.ascontiguousarray(added.reshape(-1))
        status = lib_.alea_ewald_propose_no_alloc(
            dk.data_ptr(), dw.data_ptr(), dre.data_ptr(), dim.data_ptr(), nk, alpha,
            ctypes.byref(lat), rem.ctypes.data_as(_D), len(rem) // 4, add.ctypes.data_as(_D),
            len(add) // 4, out.data_ptr(), stream)
        assert status == 0, status
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        want = state.propose(removed, added)
        assert abs(got[3] - want) <= 1e-10 * max(1.0, abs(want)), (got, want)
        assert abs((got[0] + got[1] + got[2]) - got[3]) <= 1e-12 * max(1.0, abs(got[3]))


def _call(lib_, ptrs, nk, alpha, lat, removed, added, out, stream):
    from aleator_gb300._lib import _D
    rem = np.ascontiguousarray(np.asarray(removed, dtype=np.float64).reshape(-1))
    add = np.ascontiguousarray(np.asarray(added, dtype=np.float64).reshape(-1))
    return lib_.alea_ewald_propose_no_alloc(*ptrs, nk, alpha, ctypes.byref(lat),
                                            rem.ctypes.data_as(_D), len(rem) // 4,
                                            add.ctypes.data_as(_D), len(add) // 4,
                                            out.data_ptr(), stream)


def test_no_alloc_deletion_and_no_terms(lib):
    """A deletion (no added sites) against state.propose, and a call with no
    reciprocal terms (only the finishing kernel runs): its self and exclusion
    parts against the host formulas, its reciprocal part zero."""
    A, _ = lib
    import math
    import torch
    from aleator_gb300._lib import _lattice

    g = golden("grid_cubic")
    alpha, kmax = 0.31, 6
    p = A.ParticleData(g["x"], g["y"], g["z"], g["charge"], g["species"])
    state = A.EwaldIncrementalState(A.Ewald(alpha, 12.0, kmax), p, g["lattice"])
    mol = _co2((10.0, 11.0, 12.0))
    state.commit_insertion(mol)
    k, w = A.ewald_reciprocal_terms(g["lattice"], alpha, kmax)
    raw = state.raw_state_for_testing()
    nk = len(w)
    dev = torch.device("cuda:0")
    bufs = [torch.tensor(a, dtype=torch.float64, device=dev)
            for a in (k.reshape(-1), w, raw[:nk], raw[nk:2 * nk])]
    ptrs = [b.data_ptr() for b in bufs]
    out = torch.zeros(4, dtype=torch.float64, device=dev)
    lat = _lattice(g["lattice"])
    lib_ = A.load_library()
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):  # two calls in a row
        assert _call(lib_, ptrs, nk, alpha, lat, mol, np.zeros((0, 4)), out, stream) == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        want = state.propose(mol, np.zeros((0, 4)))
        assert abs(got[3] - want) <= 1e-10 * max(1.0, abs(want)), (got, want)
    # no terms: self and exclusion of one inserted CO2, in closed form
    kc = 167100.9468982874  # the Coulomb constant in K·Å/e² (ewald.hpp:62)
    assert _call(lib_, [None] * 4, 0, alpha, lat, np.zeros((0, 4)), mol, out, stream) == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert got[0] == 0.0
    q = mol[:, 3]
    pairs = [(0, 1, 1.16), (0, 2, 2.32), (1, 2, 1.16)]
    excl = -sum(q[i] * q[j] * math.erf(alpha * r) / r for i, j, r in pairs)
    self_ = -alpha / math.sqrt(math.pi) * float((q * q).sum())
    assert abs(got[1] - kc * self_) <= 1e-12 * abs(kc * self_)
    assert abs(got[2] - kc * excl) <= 1e-12 * abs(kc * excl)
    assert got[3] == got[0] + got[1] + got[2]


def test_no_alloc_at_the_term_limit(lib):
    """Exactly 262144 synthetic terms (every slot of the fixed scratch array in
    use), an insertion and a move of three sites, two calls in a row, against
    an FP64 host sum of the same terms; the tolerance is 1e-10 of the sum of
    the terms' magnitudes (the cancellation-free scale of the sum)."""
    A, _ = lib
    import torch
    from aleator_gb300._lib import _lattice

    nk = 262144
    rng = np.random.default_rng(5)
    k = rng.uniform(-2.0, 2.0, (nk, 3))
    w = rng.uniform(0.0, 1e-2, nk)
    sre, sim = rng.normal(0.0, 3.0, nk), rng.normal(0.0, 3.0, nk)
    lattice = np.eye(3) * 31.0
    dev = torch.device("cuda:0")
    bufs = [torch.tensor(a, dtype=torch.float64, device=dev) for a in (k.reshape(-1), w, sre, sim)]
    ptrs = [b.data_ptr() for b in bufs]
    out = torch.zeros(4, dtype=torch.float64, device=dev)
    lat = _lattice(lattice)
    lib_ = A.load_library()
    stream = torch.cuda.current_stream().cuda_stream
    pref = 167100.9468982874 * 2.0 * np.pi / 31.0 ** 3  # kC 2 pi / V (ewald.hpp:62)
    for removed, added in ((np.zeros((0, 4)), _co2((3.0, 4.0, 5.0))),
                           (_co2((3.0, 4.0, 5.0)), _co2((7.5, 2.25, 9.0)))):
        re = np.zeros(nk)
        im = np.zeros(nk)
        for sign, sites in ((1.0, added), (-1.0, removed)):
            for x, y, z, q in sites:
                ph = k @ np.array([x, y, z])
                re += sign * q * np.cos(ph)
                im += sign * q * np.sin(ph)
        terms = w * (((sre + re) ** 2 + (sim + im) ** 2) - (sre ** 2 + sim ** 2))
        for _ in range(2):
            assert _call(lib_, ptrs, nk, 0.3, lat, removed, added, out, stream) == 0
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            want = pref * terms.sum()
            assert abs(got[0] - want) <= 1e-10 * pref * np.abs(terms).sum(), (got[0], want)


def test_no_alloc_rejects_oversize(lib):
    A, _ = lib
    from aleator_gb300._lib import _lattice, _D

    g = golden("grid_cubic")
    lat = _lattice(g["lattice"])
    lib_ = A.load_library()
    add = np.ascontiguousarray(_co2((1.0, 2.0, 3.0)).reshape(-1))
    status = lib_.alea_ewald_propose_no_alloc(None, None, None, None, 262145, 0.3,
                                              ctypes.byref(lat), None, 0, add.ctypes.data_as(_D),
                                              3, 1, None)
    assert status == 1
    buf = ctypes.create_string_buffer(512)
    lib_.alea_last_error(buf, 512)
    assert b"262144" in buf.value
    # site counts whose sum wraps around 2^64 are rejected, not copied
    for n_removed, n_added in ((2 ** 64 - 1, 2), (65, 0), (40, 25)):
        status = lib_.alea_ewald_propose_no_alloc(None, None, None, None, 0, 0.3,
                                                  ctypes.byref(lat), add.ctypes.data_as(_D),
                                                  n_removed, add.ctypes.data_as(_D), n_added, 1,
                                                  None)
        assert status == 1, (n_removed, n_added)
