"""GCMC chains inserting and deleting with the learned proposal.

Detailed balance: for an ideal gas (every epsilon and charge zero) the
stationary molecule count is Poisson with mean f V / T whatever the
insertion density, so with a strongly non-uniform proposal the chains'
mean count must still match f V / T (within 3 standard errors over
independent chains) and their variance their mean (within 8 %); a density
factor missing from either acceptance ratio would shift both.

Loading: CH4 in the cubic test framework, chains with a proposal fitted to
the framework's own Widom trials against chains with the reference's uniform
insertion: equal mean loading within 3 combined standard errors (chain to
chain)."""
import numpy as np
import pytest

import oracle as O
from aleator_gb300 import workloads as W
from oracle import proposal_oracle as PO

pytestmark = pytest.mark.gpu

T = 298.0


def test_ideal_gas_poisson_with_biased_proposal(lib):
    A, _ = lib
    fw = W.cubic_framework(seed=11)
    eps = np.zeros_like(fw.eps)
    ff = A.LennardJones(eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData(fw.x, fw.y, fw.z, None, fw.species)
    guest = W.ch4_guest(fw)
    m = np.asarray(fw.lattice).reshape(3, 3)
    V = abs(np.linalg.det(m))
    lam = 12.0
    f_int = lam * T / V
    f_pa = f_int / O.PASCAL_TO_INTERNAL
    n = 128
    chains = A.GcmcChains(ff, p, fw.lattice, guest, T, [f_pa] * n, list(range(100, 100 + n)),
                          [0] * n, max_molecules=200)
    # a clearly non-uniform proposal: a random network, tabulated with a floor
    P = A.Proposal(seed=21)
    rng = np.random.default_rng(5)
    w = P.get_params()
    P.set_params((rng.normal(0, 1, w.size) * 0.25).astype(np.float32))
    P.tabulate(16, 0.1)
    lp = P.log_density(PO.cell_centres(16))
    assert np.exp(lp).max() / np.exp(lp).min() > 8.0  # really non-uniform
    chains.set_proposal(P)
    chains.run(10000)  # equilibrate
    before = [(chains.info(c)["sum_molecules"], chains.info(c)["sum_molecules_sq"]) for c in range(n)]
    steps = 100000
    chains.run(steps)
    mean = np.array([(chains.info(c)["sum_molecules"] - before[c][0]) / steps for c in range(n)])
    sq = np.array([(chains.info(c)["sum_molecules_sq"] - before[c][1]) / steps for c in range(n)])
    se = mean.std(ddof=1) / np.sqrt(n)
    assert abs(mean.mean() - lam) <= 3 * se + 1e-9, (mean.mean(), lam, se)
    # variance pooled over all chains and steps (the within-chain variance
    # alone misses the spread of the chain means: the count decorrelates over
    # hundreds of moves when the proposal is far from the ideal gas's)
    var = sq.mean() - mean.mean() ** 2
    assert abs(var / lam - 1) <= 0.08, (var, lam)


def test_learned_loading_matches_uniform(lib, orc):
    A, _ = lib
    fw = W.cubic_framework(seed=11)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    guest = W.ch4_guest(fw)
    fug = orc.pr_fugacity(*W.METHANE_CRITICAL, T, 1e6)
    n = 48
    widom = A.Widom(ff, p, fw.lattice, guest, T)
    P = A.Proposal(seed=2)
    P.fit(widom, n_samples=1 << 17, rounds=2, epochs=20, cells=32)
    out = {}
    for name, prop in (("uniform", None), ("learned", P)):
        ch = A.GcmcChains(ff, p, fw.lattice, guest, T, [fug] * n, list(range(500, 500 + n)),
                          [1] * n, max_molecules=400)
        if prop is not None:
            ch.set_proposal(prop)
        ch.run(20000)
        before = [ch.info(c)["sum_molecules"] for c in range(n)]
        steps = 40000
        ch.run(steps)
        out[name] = np.array([(ch.info(c)["sum_molecules"] - before[c]) / steps for c in range(n)])
    mu, ml = out["uniform"], out["learned"]
    se = np.hypot(mu.std(ddof=1), ml.std(ddof=1)) / np.sqrt(n)
    assert mu.mean() > 0.5  # an adsorbing state point
    assert abs(ml.mean() - mu.mean()) <= 3 * se, (ml.mean(), mu.mean(), se)


def test_guest_sites_export(lib):
    """Each chain's guest sites: the tail of particles(), with the template's
    charges and LJ species."""
    A, _ = lib
    fw = W.cubic_framework(seed=12, charged=True)
    fw.charge = fw.charge * 0.15
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    guest = W.co2_guest(fw)
    fug = A.peng_robinson_fugacity(*W.CO2_CRITICAL, T, 1e6)
    ch = A.GcmcChains(ff, p, fw.lattice, guest, T, [fug] * 2, [3, 4], [0, 0],
                      ewald=A.Ewald(0.31, 12.0, 5), precision=A.FP32)
    ch.run(3000)
    for c in range(2):
        sites, sp = ch.guest_sites(c)
        nm = ch.molecules(c)
        assert nm > 0 and sites.shape == (3 * nm, 4) and sp.shape == (3 * nm,)
        assert np.array_equal(sites[:, :3], ch.positions(c)[len(fw.x):])
        qs = dict(zip(np.asarray(guest["lj_species"]).tolist(), np.asarray(guest["charge"]).tolist()))
        assert np.allclose(sites[:, 3], [qs[int(t)] for t in sp])
        assert sorted(np.unique(sp).tolist()) == sorted(set(qs))


def test_fit_at_loading_keeps_the_loading(lib, orc):
    """A proposal refitted on Widom trials in the loaded state (framework plus
    the chains' adsorbed guests): chains inserting with it keep the uniform
    chains' mean loading (within 3 combined standard errors)."""
    A, _ = lib
    fw = W.cubic_framework(seed=11)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    guest = W.ch4_guest(fw)
    fug = orc.pr_fugacity(*W.METHANE_CRITICAL, T, 1e6)
    n = 48
    out = {}
    for name in ("uniform", "learned"):
        ch = A.GcmcChains(ff, p, fw.lattice, guest, T, [fug] * n, list(range(700, 700 + n)),
                          [1] * n, max_molecules=400, precision=A.FP32)
        ch.run(10000)
        if name == "learned":
            P = A.Proposal(seed=3)
            P.fit_at_loading(ch, ff, p, fw.lattice, guest, T, chain_ids=range(4), n_samples=1 << 16,
                             rounds=2, epochs=15, cells=32)
            lp = P.log_density(PO.cell_centres(32))
            assert abs(np.exp(lp).mean() - 1.0) <= 1e-9
            ch.set_proposal(P)
        ch.run(10000)
        before = [ch.info(c)["sum_molecules"] for c in range(n)]
        steps = 30000
        ch.run(steps)
        out[name] = np.array([(ch.info(c)["sum_molecules"] - before[c]) / steps for c in range(n)])
    mu, ml = out["uniform"], out["learned"]
    se = np.hypot(mu.std(ddof=1), ml.std(ddof=1)) / np.sqrt(n)
    assert mu.mean() > 0.5
    assert abs(ml.mean() - mu.mean()) <= 3 * se, (ml.mean(), mu.mean(), se)


def test_ideal_gas_mixture_poisson_with_biased_proposal(lib):
    """Two ideal-gas species (CH4 and a 3-site CO2, every epsilon and charge
    zero) with identity swaps and a strongly non-uniform insertion density:
    each species' count stays Poisson with mean f_k V / T (means within 3
    standard errors over independent chains, variances within 10 %)."""
    A, _ = lib
    fw = W.cubic_framework(seed=11)
    eps = np.zeros_like(fw.eps)
    ff = A.LennardJones(eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData(fw.x, fw.y, fw.z, None, fw.species)
    guests = [W.ch4_guest(fw), dict(W.co2_guest(fw), charge=[0.0, 0.0, 0.0])]
    V = abs(np.linalg.det(np.asarray(fw.lattice).reshape(3, 3)))
    lams = [8.0, 5.0]
    fugs = [lam * T / V / O.PASCAL_TO_INTERNAL for lam in lams]
    n = 128
    chains = A.GcmcChains(ff, p, fw.lattice, guests, T, [fugs] * n, list(range(300, 300 + n)),
                          [0] * n, max_molecules=200)
    P = A.Proposal(seed=23)
    rng = np.random.default_rng(7)
    w = P.get_params()
    P.set_params((rng.normal(0, 1, w.size) * 0.25).astype(np.float32))
    P.tabulate(16, 0.1)
    lp = P.log_density(PO.cell_centres(16))
    assert np.exp(lp).max() / np.exp(lp).min() > 8.0
    chains.set_proposal(P)
    chains.run(10000)
    snaps = []
    for _ in range(100):
        chains.run(500)
        snaps.append([chains.info(c)["species_molecules"][:2] for c in range(n)])
    counts = np.array(snaps, dtype=np.float64)  # snapshots x chains x species
    info = chains.info(0)
    assert info["accepted"][4] > 0  # swaps happened
    for k, lam in enumerate(lams):
        per_chain = counts[:, :, k].mean(axis=0)
        se = per_chain.std(ddof=1) / np.sqrt(n)
        assert abs(per_chain.mean() - lam) <= 3 * se + 1e-9, (k, per_chain.mean(), lam, se)
        var = counts[:, :, k].var()
        assert abs(var / lam - 1) <= 0.10, (k, var, lam)
