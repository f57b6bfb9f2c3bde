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


@pytest.mark.parametrize("trunc", ["TRUNCATED", "SHIFTED", "LINEAR_FORCE_SHIFTED"])
def test_fp32_uncharged_triclinic_vs_fp64(lib, trunc):
    """FP32 form, uncharged probe (FP32 displacements and images, pairs within
    1.25 sigma and, for plain truncation, pairs at the cutoff redone in
    double-float) on triclinic cells of the batched-screening kind, every
    truncation: per trial within 1e-5 x max(kT, |dU|) of the FP64 form (itself
    pinned to the oracle) on trials with dU <= 1e4 K, and K_H within 1e-5."""
    A, _ = lib
    from aleator_gb300 import workloads as W
    fws = W.random_triclinic_frameworks(8, seed=31)
    checked = 0
    for i, fw in enumerate(fws):
        ff = A.LennardJones(fw.eps, fw.sigma, 12.8, getattr(A, trunc))
        p = A.ParticleData.from_framework(fw)
        guest = W.ch4_guest(fw)
        r64, per64 = A.Widom(ff, p, fw.lattice, guest, 298.0).run(5, i, 20000, per_trial=True)
        r32, per32 = A.Widom(ff, p, fw.lattice, guest, 298.0, precision=A.FP32).run(
            5, i, 20000, per_trial=True)
        keep = per64 <= 1e4
        assert (per32[~keep] > 1e4 * (1 - 1e-5)).all()
        if keep.sum() < 50:  # a dense cell: no trial carries Boltzmann weight
            continue
        checked += 1
        assert rel_err(per32[keep], per64[keep], floor=KT).max() <= 1e-5, (i, trunc)
        assert abs(r32["henry"] / r64["henry"] - 1) <= 1e-5
    assert checked >= 2


def test_fp32_charged_c4_per_trial_vs_fp64(lib):
    """The FP32 form on the learned-proposal workload (charged 424-atom cell,
    charges up to 1.2 e, rigid CO2, Ewald for 1e-6 with kMax 10), 65 536 trials:
    per trial within 1e-5 x max(kT, |dU|) of the FP64 form on trials that carry
    Boltzmann weight (dU <= 1e4 K), and K_H within 1e-5. Its reciprocal phases
    are double-float and its Coulomb pairs within 4.5 A FP64: with FP32 phases
    or FP32 near pairs this workload's errors reach ~5e-5 of kT."""
    A, _ = lib
    from aleator_gb300 import workloads as W
    fw = W.cubic_framework(charged=True)
    alpha, kmax = W.ewald_parameters(fw.lattice, 12.0)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    ew = A.Ewald(alpha, 12.0, kmax)
    out = {}
    for prec in (A.FP64, A.FP32):
        w = A.Widom(ff, p, fw.lattice, W.co2_guest(fw), 298.0, ewald=ew, precision=prec)
        out[prec] = w.run(7, 3, 1 << 16, per_trial=True)
    (r64, d64), (r32, d32) = out[A.FP64], out[A.FP32]
    keep = d64 <= 1e4
    assert keep.sum() > 1000
    assert rel_err(d32[keep], d64[keep], floor=KT).max() <= 1e-5
    assert abs(r32["henry"] / r64["henry"] - 1) <= 1e-5
