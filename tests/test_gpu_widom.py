"""Widom insertion on the GPU against the reference's per-trial energies
(golden, made by the reference's own MonteCarloEngine primitives) and the
oracle. FP64 per-trial dU within 1e-10 relative (1 K floor); K_H within
1e-9 relative; FP32 form per-trial within 1e-5 relative with a kT floor
(|d dU| <= 1e-5 * max(kT, |dU|), kT = 298 K) on trials that carry Boltzmann
weight (dU <= 1e4 K), and its K_H within 1e-5 relative."""
import numpy as np
import pytest

import oracle as O
from conftest import golden, rel_err

KT = 298.0

pytestmark = pytest.mark.gpu


class _FW:
    guest_species = {"CH4": 4, "CO2_C": 5, "CO2_O": 6}


def _setup(A, charged):
    from aleator_gb300 import workloads as W
    g = golden("grid_cubic")
    ff = A.LennardJones(g["eps"], g["sigma"], 12.8, A.SHIFTED)
    p = A.ParticleData(g["x"], g["y"], g["z"], g["charge"], g["species"])
    guest = W.co2_guest(_FW) if charged else W.ch4_guest(_FW)
    return g, ff, p, guest


def test_ch4_per_trial_and_henry(lib):
    A, _ = lib
    g, ff, p, guest = _setup(A, False)
    w = golden("widom_ch4")
    widom = A.Widom(ff, p, g["lattice"], guest, 298.0)
    r, per = widom.run(42, 0, len(w["per_trial"]), per_trial=True)
    assert rel_err(per, w["per_trial"]).max() <= 1e-10
    assert abs(r["henry"] / float(w["kh"]) - 1) <= 1e-9
    w32 = A.Widom(ff, p, g["lattice"], guest, 298.0, precision=A.FP32)
    r32, per32 = w32.run(42, 0, len(w["per_trial"]), per_trial=True)
    keep = w["per_trial"] <= 1e4
    assert rel_err(per32[keep], w["per_trial"][keep], floor=KT).max() <= 1e-5
    assert abs(r32["henry"] / float(w["kh"]) - 1) <= 1e-5


def test_co2_charged_per_trial_and_henry(lib):
    A, _ = lib
    g, ff, p, guest = _setup(A, True)
    c = golden("widom_co2")
    ew = A.Ewald(float(c["alpha"]), 12.0, int(c["kmax"]))
    widom = A.Widom(ff, p, g["lattice"], guest, 298.0, ewald=ew)
    r, per = widom.run(42, 0, len(c["per_trial"]), per_trial=True)
    assert rel_err(per, c["per_trial"]).max() <= 1e-10
    assert abs(r["henry"] / float(c["kh"]) - 1) <= 1e-9
    w32 = A.Widom(ff, p, g["lattice"], guest, 298.0, ewald=ew, precision=A.FP32)
    _, per32 = w32.run(42, 0, len(c["per_trial"]), per_trial=True)
    keep = c["per_trial"] <= 1e4
    assert rel_err(per32[keep], c["per_trial"][keep], floor=KT).max() <= 1e-5


def test_triclinic_charged(lib):
    A, _ = lib
    from aleator_gb300 import workloads as W
    t = golden("triclinic")
    ff = A.LennardJones(t["eps"], t["sigma"], 10.0, A.SHIFTED)
    p = A.ParticleData(t["x"], t["y"], t["z"], t["charge"], t["species"])
    widom = A.Widom(ff, p, t["lattice"], W.co2_guest(_FW), 298.0, ewald=A.Ewald(0.35, 10.0, 5))
    r, per = widom.run(7, 3, len(t["widom_per_trial"]), per_trial=True)
    assert rel_err(per, t["widom_per_trial"]).max() <= 1e-10
    assert abs(r["henry"] / float(t["widom_kh"]) - 1) <= 1e-9


def test_counter_windows_and_draw_order(lib, orc):
    """Trials far along the stream (counter-indexed) and the clang draw order,
    against the oracle; K_H over windows combines exactly as one run."""
    A, _ = lib
    g, ff, p, guest = _setup(A, True)
    ew = dict(alpha=0.31, rc=12.0, kmax=6)
    widom = A.Widom(ff, p, g["lattice"], guest, 298.0, ewald=A.Ewald(0.31, 12.0, 6))
    odict = dict(eps=g["eps"], sigma=g["sigma"], cutoff=12.8, truncation=O.SHIFTED)
    for first, order in [(10_000_000, A.ALEA_DRAWS_RIGHT_TO_LEFT), (0, A.ALEA_DRAWS_LEFT_TO_RIGHT),
                         ((1 << 31) + 77, A.ALEA_DRAWS_RIGHT_TO_LEFT)]:
        r, per = widom.run(9, 4, 300, first_trial=first, draw_order=order, per_trial=True)
        _, ref = orc.widom(odict, ew, g["lattice"], g["x"], g["y"], g["z"], g["charge"],
                           g["species"], guest, 298.0, 9, 4, 300, first_trial=first,
                           draw_order=order, threads=8, per_trial=True)
        assert rel_err(per, ref).max() <= 1e-10


def test_large_run_statistics(lib, orc):
    """1e5 CH4 trials (the 424-atom workload): K_H vs the oracle over the same
    trials, and the reported standard error is consistent."""
    A, _ = lib
    g, ff, p, guest = _setup(A, False)
    widom = A.Widom(ff, p, g["lattice"], guest, 298.0)
    n = 100_000
    r = widom.run(42, 0, n)
    odict = dict(eps=g["eps"], sigma=g["sigma"], cutoff=12.8, truncation=O.SHIFTED)
    kh = orc.widom(odict, None, g["lattice"], g["x"], g["y"], g["z"], None, g["species"], guest,
                   298.0, 42, 0, n, threads=16)
    assert abs(r["henry"] / kh - 1) <= 1e-9
    assert 0 < r["rel_std_error"] < 0.1
