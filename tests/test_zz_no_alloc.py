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
