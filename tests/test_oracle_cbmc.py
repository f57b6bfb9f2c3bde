"""The oracle's orientation-biased insertion and deletion (no reference
counterpart; the GPU chains' FP64 draw order and arithmetic), on the CPU.

Detailed balance: an ideal gas of rigid CO2 (every epsilon and charge zero)
has every trial weight 1, so with k trials the chain's molecule count stays
Poisson with mean lambda = f V / T: the time-averaged mean within 3 standard
errors over independent chains and the variance within 10 % of lambda. k = 1
is the reference's move: it draws and decides as the plain oracle chain."""
import numpy as np

import oracle as O
from aleator_gb300 import workloads as W

T = 298.0


def _ideal(orc, k, seed):
    fw = W.cubic_framework(seed=11)
    od = dict(eps=np.zeros_like(fw.eps), sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    guest = dict(W.co2_guest(fw), charge=[0.0, 0.0, 0.0])
    V = abs(np.linalg.det(np.asarray(fw.lattice).reshape(3, 3)))
    lam = 6.0
    f_pa = lam * T / V / O.PASCAL_TO_INTERNAL
    g = orc.gcmc(od, None, fw.lattice, fw.x, fw.y, fw.z, None, fw.species, guest, T, f_pa, seed, 2)
    g.set_orientation_trials(k)
    return g, lam


def test_orientation_trials_keep_an_ideal_gas_poisson(orc):
    means, sq = [], []
    for seed in range(6):
        g, lam = _ideal(orc, 6, 300 + seed)
        g.run(2000)
        samples = []
        for _ in range(1500):
            g.run(8)
            samples.append(g.molecules())
        s = np.array(samples, dtype=float)
        means.append(s.mean())
        sq.append((s * s).mean())
    means, sq = np.array(means), np.array(sq)
    se = means.std(ddof=1) / np.sqrt(len(means))
    assert abs(means.mean() - lam) <= 3 * se + 1e-9, (means.mean(), lam, se)
    var = sq.mean() - means.mean() ** 2
    assert abs(var / lam - 1) <= 0.10, (var, lam)


def test_one_trial_is_the_plain_move(orc):
    fw = W.cubic_framework(seed=12, charged=True)
    fw.charge = fw.charge * 0.15
    od = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    ew = dict(alpha=0.31, rc=12.0, kmax=5)
    fug = orc.pr_fugacity(*W.CO2_CRITICAL, T, 1e6)
    a = orc.gcmc(od, ew, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, W.co2_guest(fw), T,
                 fug, 3, 7)
    b = orc.gcmc(od, ew, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, W.co2_guest(fw), T,
                 fug, 3, 7)
    b.set_orientation_trials(4)
    b.set_orientation_trials(1)
    a.run(400)
    b.run(400)
    assert a.calls() == b.calls() and a.molecules() == b.molecules()
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.counters(), b.counters())
