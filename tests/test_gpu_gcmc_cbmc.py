"""Orientation-biased insertion and deletion (k orientation trials with the
Rosenbluth weight in the acceptance ratios; no counterpart in the reference
engine, which inserts with one random orientation).

Detailed balance, two ways:
* an ideal gas of rigid CO2 (every epsilon and charge zero): every trial
  weight is 1, so the stationary count stays Poisson with mean f V / T
  (within 3 standard errors over independent chains, variance within 8 %),
  also with a strongly non-uniform learned proposal on top;
* charged CO2 in the cubic test framework (charges scaled by 0.15, Ewald):
  chains with 6 orientation trials (with and without the learned proposal)
  reach the same mean loading as chains with the reference's moves (within 4
  combined standard errors, chain to chain), with a higher insertion
  acceptance. A Rosenbluth factor missing from either ratio, or a trial drawn
  about the wrong point, would shift the loading.
k = 1 is the reference's move: after switching k back to 1 a chain follows
the oracle move for move."""
import numpy as np
import pytest

import oracle as O
from aleator_gb300 import workloads as W
from test_gpu_gcmc import _compare

pytestmark = pytest.mark.gpu

T = 298.0


def _loading(chains, n, equil, prod):
    chains.run(equil)
    before = [chains.info(c)["sum_molecules"] for c in range(n)]
    sq0 = [chains.info(c)["sum_molecules_sq"] for c in range(n)]
    chains.run(prod)
    mean = np.array([(chains.info(c)["sum_molecules"] - before[c]) / prod for c in range(n)])
    sq = np.array([(chains.info(c)["sum_molecules_sq"] - sq0[c]) / prod for c in range(n)])
    return mean, sq


@pytest.mark.parametrize("with_proposal,fp32", [(False, False), (True, False), (False, True)])
def test_orientation_trials_ideal_gas_poisson(lib, with_proposal, fp32):
    """(fp32: the FP32 form, which evaluates all k trials in one pass.)"""
    A, _ = lib
    fw = W.cubic_framework(seed=11)
    ff = A.LennardJones(np.zeros_like(fw.eps), fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData(fw.x, fw.y, fw.z, None, fw.species)
    guest = dict(W.co2_guest(fw), charge=[0.0, 0.0, 0.0])
    V = abs(np.linalg.det(np.asarray(fw.lattice).reshape(3, 3)))
    lam = 10.0
    f_pa = lam * T / V / O.PASCAL_TO_INTERNAL
    n = 128
    chains = A.GcmcChains(ff, p, fw.lattice, guest, T, [f_pa] * n, list(range(300, 300 + n)),
                          [2] * n, max_molecules=200, precision=A.FP32 if fp32 else A.FP64)
    chains.set_orientation_trials(6)
    if with_proposal:
        P = A.Proposal(seed=23)
        rng = np.random.default_rng(6)
        w = P.get_params()
        P.set_params((rng.normal(0, 1, w.size) * 0.25).astype(np.float32))
        P.tabulate(16, 0.1)
        chains.set_proposal(P)
    mean, sq = _loading(chains, n, 10000, 60000)
    se = mean.std(ddof=1) / np.sqrt(n)
    assert abs(mean.mean() - lam) <= 3 * se + 1e-9, (mean.mean(), lam, se)
    var = sq.mean() - mean.mean() ** 2
    assert abs(var / lam - 1) <= 0.08, (var, lam)


@pytest.mark.parametrize("with_proposal", [False, True])
def test_orientation_trials_keep_the_loading(lib, with_proposal):
    A, _ = lib
    fw = W.cubic_framework(seed=12, charged=True)
    fw.charge = fw.charge * 0.15
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    guest = W.co2_guest(fw)
    ew = A.Ewald(0.31, 12.0, 5)
    fug = A.peng_robinson_fugacity(*W.CO2_CRITICAL, T, 2e5)
    n = 152
    res = {}
    for name, k in (("plain", 1), ("biased", 6)):
        ch = A.GcmcChains(ff, p, fw.lattice, guest, T, [fug] * n, list(range(700, 700 + n)),
                          [3 if k == 1 else 4] * n, ewald=ew, max_molecules=400,
                          precision=A.FP32)
        if k > 1:
            ch.set_orientation_trials(k)
            if with_proposal:
                widom = A.Widom(ff, p, fw.lattice, guest, T, ewald=ew, precision=A.FP32)
                P = A.Proposal(seed=4)
                P.fit(widom, n_samples=1 << 17, rounds=2, epochs=15, cells=32, uniform_share=0.2)
                ch.set_proposal(P)
        mean, _ = _loading(ch, n, 20000, 60000)
        att = np.array([ch.info(c)["attempted"] for c in range(n)]).sum(0)
        acc = np.array([ch.info(c)["accepted"] for c in range(n)]).sum(0)
        res[name] = (mean.mean(), mean.std(ddof=1) / np.sqrt(n), acc[2] / att[2])
    (mp, sp, ap), (mb, sb, ab) = res["plain"], res["biased"]
    print(f"\nloading plain {mp:.3f} +/- {sp:.3f} (insert acc {ap:.4f}); "
          f"biased {mb:.3f} +/- {sb:.3f} (insert acc {ab:.4f})")
    assert mp > 1.0
    assert abs(mp - mb) <= 4 * np.hypot(sp, sb), res
    assert ab > ap


def test_one_orientation_trial_is_the_reference_move(lib, orc):
    A, _ = lib
    fw = W.cubic_framework(seed=12, charged=True)
    fw.charge = fw.charge * 0.15
    ew = dict(alpha=0.31, rc=12.0, kmax=5)
    fug = orc.pr_fugacity(*W.CO2_CRITICAL, T, 1e6)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    gpu = A.GcmcChains(ff, p, fw.lattice, W.co2_guest(fw), T, [fug], [3], [7],
                       ewald=A.Ewald(0.31, 12.0, 5))
    gpu.set_orientation_trials(4)
    gpu.set_orientation_trials(1)
    od = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    cpu = orc.gcmc(od, ew, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, W.co2_guest(fw),
                   T, fug, 3, 7)
    gpu.run(1500)
    cpu.run(1500)
    _compare(gpu, cpu, charged=True)
    with pytest.raises(ValueError):
        gpu.set_orientation_trials(17)


@pytest.mark.parametrize("k", [3, 6])
def test_fused_trials_follow_the_pass_by_pass_form(lib, k):
    """The FP32 form evaluates all k <= 8 trial orientations of a biased
    insertion or deletion in one pass; the FP64 form evaluates them one pass
    each. From the same seeds the two take the same draws, so move by move
    they make the same decisions, and each move's energy change agrees as the
    FP32 form's does for plain moves (test_gpu_gcmc_fp32.py): a biased
    insertion's (the picked trial's energy) or deletion's (minus the
    molecule's own) within 1e-5 x max(kT, |dU|); a translation's or
    rotation's, a difference of two molecule energies, within 1e-5 x max(kT,
    |dU|, E), E the largest molecule energy met. A decision can flip where a
    ratio falls within that error of its uniform draw; each chain is compared
    up to such a point, which must lie beyond most of the run."""
    A, _ = lib
    fw = W.cubic_framework(seed=12, charged=True)
    fw.charge = fw.charge * 0.3
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    guest = W.co2_guest(fw)
    alpha, kmax = W.ewald_parameters(fw.lattice, 12.0)
    ew = A.Ewald(alpha, 12.0, kmax)
    fug = A.peng_robinson_fugacity(*W.CO2_CRITICAL, T, 10e5)
    n = 4
    pair = []
    for prec in (A.FP64, A.FP32):
        ch = A.GcmcChains(ff, p, fw.lattice, guest, T, [fug] * n, list(range(40, 40 + n)),
                          [5] * n, ewald=ew, max_molecules=300, precision=prec)
        ch.set_orientation_trials(k)
        pair.append(ch)
    g64, g32 = pair
    live = [True] * n
    prev = [g64.info(c)["attempted"] for c in range(n)]
    e_scale = [0.0] * n
    compared = {0: 0, 1: 0, 2: 0, 3: 0}
    moves = 600
    for step in range(moves):
        g64.run(1)
        g32.run(1)
        for c in range(n):
            a, b = g64.info(c), g32.info(c)
            took = np.array(a["attempted"]) - np.array(prev[c])
            prev[c] = a["attempted"]
            if not live[c]:
                continue
            if a["call_index"] != b["call_index"] or a["molecules"] != b["molecules"] or \
                    a["accepted"] != b["accepted"] or a["attempted"] != b["attempted"]:
                live[c] = False  # a decision flipped: the chains part here
                continue
            if took.sum() == 0 or not np.isfinite(a["last_du"]):
                continue  # nothing to act on: no energy evaluated
            move = int(np.argmax(took))
            du64, du32 = a["last_du"], b["last_du"]
            if abs(du64) > 1e5:  # an overlapping trial: both reject whatever its size
                continue
            if move >= 2:
                e_scale[c] = max(e_scale[c], abs(du64))
                assert abs(du32 - du64) <= 1e-5 * max(T, abs(du64)), (step, c, move, du64, du32)
            else:
                assert abs(du32 - du64) <= 1e-5 * max(T, abs(du64), e_scale[c]), \
                    (step, c, move, du64, du32, e_scale[c])
            compared[move] += 1
    assert sum(compared.values()) >= 0.6 * n * moves, compared
    assert compared[2] >= 100 and compared[3] >= 20, compared


@pytest.mark.parametrize("k", [3, 6])
def test_orientation_trials_follow_the_oracle(lib, orc, k):
    """The FP64 form's orientation-biased insertions and deletions against
    the oracle's restatement of them (the same draws, in the same order, and
    the same arithmetic): move for move the same counters, particle order and
    positions (1e-9), and the same Ewald energy (1e-10)."""
    A, _ = lib
    fw = W.cubic_framework(seed=12, charged=True)
    fw.charge = fw.charge * 0.15
    ew = dict(alpha=0.31, rc=12.0, kmax=5)
    fug = orc.pr_fugacity(*W.CO2_CRITICAL, T, 1e6)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    gpu = A.GcmcChains(ff, p, fw.lattice, W.co2_guest(fw), T, [fug], [3], [7],
                       ewald=A.Ewald(0.31, 12.0, 5))
    gpu.set_orientation_trials(k)
    od = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    cpu = orc.gcmc(od, ew, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, W.co2_guest(fw),
                   T, fug, 3, 7)
    cpu.set_orientation_trials(k)
    for _ in range(3):
        gpu.run(400)
        cpu.run(400)
        _compare(gpu, cpu, charged=True)
    acc = gpu.info()["accepted"]
    assert acc[2] > 0 and acc[3] > 0, acc
