"""GCMC chains on the GPU against the oracle's restatement of
MonteCarloEngine::run (itself bit-exact to the reference engine, see
tests/test_oracle_gcmc.py): the same Philox stream drives both, so the move
sequence, acceptances, molecule counts and particle order must agree;
positions and the committed Ewald energy within FP64 rounding (1e-9 Å and
1e-10 relative; the GPU sums pair energies in a tree order)."""
import numpy as np
import pytest

import oracle as O
from aleator_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _pair(A, orc, fw, guest, ewald, fug, seed, stream, T=298.0):
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    ew = A.Ewald(ewald["alpha"], ewald["rc"], ewald["kmax"]) if ewald else None
    gpu = A.GcmcChains(ff, p, fw.lattice, guest, T, [fug], [seed], [stream], ewald=ew)
    od = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    cpu = orc.gcmc(od, ewald, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guest, T, fug,
                   seed, stream)
    return gpu, cpu


def _compare(gpu, cpu, chain=0, charged=False):
    info = gpu.info(chain)
    assert info["molecules"] == cpu.molecules()
    assert info["call_index"] == cpu.calls()
    ctr = cpu.counters()
    n = len(info["attempted"])  # the oracle's counters: attempted[5], accepted[5]
    assert list(info["attempted"]) == [int(v) for v in ctr[:n]]
    assert list(info["accepted"]) == [int(v) for v in ctr[5:5 + n]]
    pg, pc = gpu.positions(chain), cpu.positions()
    assert pg.shape == pc.shape
    assert np.abs(pg - pc).max() <= 1e-9
    if charged:
        eg, ec = gpu.ewald_energy(chain), cpu.ewald_energy()
        assert abs(eg - ec) <= 1e-10 * max(1.0, abs(ec))


def test_ch4_chain_matches_oracle(lib, orc):
    A, _ = lib
    fw = W.cubic_framework(seed=11)
    fug = orc.pr_fugacity(*W.METHANE_CRITICAL, 298.0, 5e6)
    gpu, cpu = _pair(A, orc, fw, W.ch4_guest(fw), None, fug, 5, 1)
    for _ in range(4):
        gpu.run(400)
        cpu.run(400)
        _compare(gpu, cpu)
    assert gpu.info()["accepted"][2] > 0


def test_co2_charged_chain_with_resync(lib, orc):
    A, _ = lib
    fw = W.cubic_framework(seed=12, charged=True)
    fw.charge = fw.charge * 0.15  # weaker framework field: many accepted moves, several resyncs
    ew = dict(alpha=0.31, rc=12.0, kmax=5)
    fug = orc.pr_fugacity(*W.CO2_CRITICAL, 298.0, 1e6)
    gpu, cpu = _pair(A, orc, fw, W.co2_guest(fw), ew, fug, 3, 7)
    for _ in range(6):
        gpu.run(500)
        cpu.run(500)
        _compare(gpu, cpu, charged=True)
    assert gpu.info()["resyncs"] >= 1


def test_many_chains_independent(lib, orc):
    A, _ = lib
    fw = W.cubic_framework(seed=13, charged=True)
    fw.charge = fw.charge * 0.15
    ew = dict(alpha=0.31, rc=12.0, kmax=4)
    pressures = [1e4, 1e5, 1e6, 3e6]
    fugs = [orc.pr_fugacity(*W.CO2_CRITICAL, 298.0, P) for P in pressures]
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    chains = A.GcmcChains(ff, p, fw.lattice, W.co2_guest(fw), 298.0, fugs, [21] * 4,
                          [0, 1, 2, 3], ewald=A.Ewald(0.31, 12.0, 4))
    chains.run(600)
    od = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    for c in range(4):
        cpu = orc.gcmc(od, ew, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species,
                       W.co2_guest(fw), 298.0, fugs[c], 21, c)
        cpu.run(600)
        _compare(chains, cpu, chain=c, charged=True)


def test_capacity_is_reported(lib):
    A, _ = lib
    fw = W.cubic_framework(seed=14)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    chains = A.GcmcChains(ff, A.ParticleData.from_framework(fw), fw.lattice, W.ch4_guest(fw), 298.0,
                          [1e9], [1], [0], max_molecules=2)
    with pytest.raises(A.AleatorError) as e:
        chains.run(2000)
    assert e.value.status == 6


@pytest.mark.parametrize("charged", [False, True])
def test_chain_with_energy_grid_matches_oracle(lib, orc, charged):
    """The engine with its frameworkEnergyGrid (monte_carlo_engine.cc:341-374):
    the GPU chain reads a GPU-built FP64 grid (within 1e-10 of the reference's
    tables), the oracle the oracle's grid (bit-identical to the reference's,
    tests/test_oracle_gcmc.py); same moves and decisions, positions within
    1e-9 Å."""
    A, _ = lib
    fw = W.cubic_framework(seed=21, charged=charged)
    if charged:
        fw.charge = fw.charge * 0.15
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    ewd = dict(alpha=0.31, rc=12.0, kmax=5) if charged else None
    ew = A.Ewald(0.31, 12.0, 5) if charged else None
    guest = W.co2_guest(fw) if charged else W.ch4_guest(fw)
    fug = orc.pr_fugacity(*(W.CO2_CRITICAL if charged else W.METHANE_CRITICAL), 298.0, 1e6)
    species = sorted(set(int(s) for s in guest["lj_species"]))
    grid = A.FrameworkEnergyGrid(ff, p, fw.lattice, species, 0.5, A.FP64)
    od = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    tables = {s: orc.grid_build(od, fw.lattice, fw.x, fw.y, fw.z, fw.species, s, 0.5, threads=8)
              for s in species}
    gpu = A.GcmcChains(ff, p, fw.lattice, guest, 298.0, [fug], [9], [4], ewald=ew)
    gpu.set_grid(grid)
    cpu = orc.gcmc(od, ewd, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guest, 298.0, fug,
                   9, 4, grid={"counts": grid.point_counts(), "tables": tables})
    for _ in range(4):
        gpu.run(300)
        cpu.run(300)
        _compare(gpu, cpu, charged=charged)
    assert gpu.molecules() > 0


def test_energy_grid_guards(lib):
    A, _ = lib
    fw = W.cubic_framework(seed=21)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    guest = W.ch4_guest(fw)
    chains = A.GcmcChains(ff, p, fw.lattice, guest, 298.0, [1e5], [1], [0])
    # a grid without the guest's species: out_of_range, as interpolate
    g_wrong = A.FrameworkEnergyGrid(ff, p, fw.lattice, [fw.guest_species["CO2_C"]], 2.0, A.FP64)
    with pytest.raises(IndexError):
        chains.set_grid(g_wrong)
    # a grid on another cell: invalid_argument
    m2 = np.asarray(fw.lattice, dtype=float) * 1.01
    g_cell = A.FrameworkEnergyGrid(ff, p, m2, [guest["lj_species"][0]], 2.0, A.FP64)
    with pytest.raises(ValueError):
        chains.set_grid(g_cell)
    chains.set_grid(None)
    chains.run(10)


def test_large_kmax_chain_matches_oracle(lib, orc):
    """kMax 24 (a cell of about 100 A needs about 35 for Ewald 1e-6): the phase
    tables beyond the old limit of 20; same moves as the oracle."""
    A, _ = lib
    fw = W.cubic_framework(seed=12, charged=True)
    fw.charge = fw.charge * 0.15
    ew = dict(alpha=0.31, rc=12.0, kmax=24)
    fug = orc.pr_fugacity(*W.CO2_CRITICAL, 298.0, 1e6)
    gpu, cpu = _pair(A, orc, fw, W.co2_guest(fw), ew, fug, 3, 7)
    for _ in range(3):
        gpu.run(300)
        cpu.run(300)
        _compare(gpu, cpu, charged=True)
    with pytest.raises(ValueError):
        _pair(A, orc, fw, W.co2_guest(fw), dict(alpha=0.31, rc=12.0, kmax=65), fug, 3, 7)


@pytest.mark.parametrize("charged", [False, True])
def test_mixture_chain_matches_oracle(lib, orc, charged):
    """Two species (CH4 and CO2; the mixture constructor, monte_carlo_engine.hpp:
    143-151): 20 % each of translate, rotate, insert, delete and identity swap.
    Same moves, decisions, per-species counts and particle order as the oracle
    (itself bit-identical to the reference's mixture engine)."""
    A, _ = lib
    fw = W.cubic_framework(seed=21, charged=charged)
    if charged:
        fw.charge = fw.charge * 0.15
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    ewd = dict(alpha=0.31, rc=12.0, kmax=5) if charged else None
    ew = A.Ewald(0.31, 12.0, 5) if charged else None
    ch4 = dict(W.ch4_guest(fw), charge=[0.0])
    guests = [W.co2_guest(fw), ch4] if charged else [ch4, dict(W.co2_guest(fw), charge=[0.0] * 3)]
    fugs = [orc.pr_fugacity(*W.CO2_CRITICAL, 298.0, 5e5), orc.pr_fugacity(*W.METHANE_CRITICAL, 298.0, 2e6)]
    if not charged:
        fugs = fugs[::-1]
    gpu = A.GcmcChains(ff, p, fw.lattice, guests, 298.0, [fugs], [9], [4], ewald=ew)
    od = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    cpu = orc.gcmc_mixture(od, ewd, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guests,
                           298.0, fugs, 9, 4)
    for _ in range(5):
        gpu.run(400)
        cpu.run(400)
        _compare(gpu, cpu, charged=charged)
        assert gpu.info()["species_molecules"][:2] == [cpu.molecules_of(k) for k in range(2)]
    assert gpu.info()["accepted"][4] > 0  # swaps accepted


def test_mixture_with_energy_grid_matches_oracle(lib, orc):
    """CH4 + charged CO2 with the engine's energy grid (one table per guest LJ
    species: CH4, CO2's O and C): the same moves, decisions and positions as
    the oracle's mixture engine with the same tables."""
    A, _ = lib
    fw = W.cubic_framework(seed=23, charged=True)
    fw.charge = fw.charge * 0.15
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    ewd = dict(alpha=0.31, rc=12.0, kmax=5)
    ew = A.Ewald(0.31, 12.0, 5)
    guests = [W.co2_guest(fw), W.ch4_guest(fw)]
    species = sorted({int(s) for g in guests for s in g["lj_species"]})
    grid = A.FrameworkEnergyGrid(ff, p, fw.lattice, species, 0.5, A.FP64)
    od = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    tables = {s: orc.grid_build(od, fw.lattice, fw.x, fw.y, fw.z, fw.species, s, 0.5, threads=8)
              for s in species}
    fugs = [orc.pr_fugacity(*W.CO2_CRITICAL, 298.0, 5e5), orc.pr_fugacity(*W.METHANE_CRITICAL, 298.0, 2e6)]
    gpu = A.GcmcChains(ff, p, fw.lattice, guests, 298.0, [fugs], [13], [2], ewald=ew)
    gpu.set_grid(grid)
    cpu = orc.gcmc_mixture(od, ewd, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guests,
                           298.0, fugs, 13, 2, grid={"counts": grid.point_counts(), "tables": tables})
    for _ in range(4):
        gpu.run(300)
        cpu.run(300)
        _compare(gpu, cpu, charged=True)
        assert gpu.info()["species_molecules"][:2] == [cpu.molecules_of(k) for k in range(2)]
    assert gpu.molecules() > 0
