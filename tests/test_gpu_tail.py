"""The opt-in LJ tail correction of particle-number moves (no counterpart in
the reference engine, whose moves leave tailEnergyCorrection out): with it on,
an insertion, deletion or identity swap adds U_tail(after) - U_tail(before),
U_tail being tailEnergyCorrection (lennard_jones.cc:246-257) over every
particle. The oracle computes that change as two tailEnergyCorrection
evaluations per move; the GPU from per-species constants of the same
quadratic form. Trajectories are compared move for move (counts, particle
order, positions to 1e-9 Å, the Ewald energy to 1e-10)."""
import numpy as np
import pytest

import oracle as O
from aleator_gb300 import workloads as W
from test_gpu_gcmc import _compare

pytestmark = pytest.mark.gpu


def test_gcmc_tail_single_species_matches_oracle(lib, orc):
    A, _ = lib
    fw = W.cubic_framework(seed=11)
    fug = orc.pr_fugacity(*W.METHANE_CRITICAL, 298.0, 5e6)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    od = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    guest = W.ch4_guest(fw)
    gpu = A.GcmcChains(ff, p, fw.lattice, guest, 298.0, [fug], [5], [1])
    gpu.set_tail_correction(True)
    cpu = orc.gcmc(od, None, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guest, 298.0,
                   fug, 5, 1)
    cpu.set_tail(True)
    plain = orc.gcmc(od, None, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guest, 298.0,
                     fug, 5, 1)
    for _ in range(4):
        gpu.run(400)
        cpu.run(400)
        plain.run(400)
        _compare(gpu, cpu)
    # the correction changes decisions (about -40 K per CH4 insertion here)
    assert list(cpu.counters()) != list(plain.counters())


def test_gcmc_tail_mixture_matches_oracle(lib, orc):
    """CH4 + charged CO2: insertions, deletions and identity swaps each carry
    their own tail change (swaps change the site species counts too)."""
    A, _ = lib
    fw = W.cubic_framework(seed=21, charged=True)
    fw.charge = fw.charge * 0.15
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    ewd = dict(alpha=0.31, rc=12.0, kmax=5)
    guests = [W.co2_guest(fw), dict(W.ch4_guest(fw), charge=[0.0])]
    fugs = [orc.pr_fugacity(*W.CO2_CRITICAL, 298.0, 5e5),
            orc.pr_fugacity(*W.METHANE_CRITICAL, 298.0, 2e6)]
    gpu = A.GcmcChains(ff, p, fw.lattice, guests, 298.0, [fugs], [9], [4],
                       ewald=A.Ewald(0.31, 12.0, 5))
    gpu.set_tail_correction(True)
    od = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    cpu = orc.gcmc_mixture(od, ewd, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guests,
                           298.0, fugs, 9, 4)
    cpu.set_tail(True)
    for _ in range(5):
        gpu.run(400)
        cpu.run(400)
        _compare(gpu, cpu, charged=True)
        assert gpu.info()["species_molecules"][:2] == [cpu.molecules_of(k) for k in range(2)]
    assert gpu.info()["accepted"][4] > 0  # swaps accepted


def test_gcmc_tail_off_is_the_reference(lib, orc):
    """Switching it on and off again leaves the reference engine's moves."""
    A, _ = lib
    fw = W.cubic_framework(seed=11)
    fug = orc.pr_fugacity(*W.METHANE_CRITICAL, 298.0, 5e6)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    od = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    gpu = A.GcmcChains(ff, p, fw.lattice, W.ch4_guest(fw), 298.0, [fug], [5], [1])
    gpu.set_tail_correction(True)
    gpu.set_tail_correction(False)
    cpu = orc.gcmc(od, None, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, W.ch4_guest(fw),
                   298.0, fug, 5, 1)
    gpu.run(800)
    cpu.run(800)
    _compare(gpu, cpu)


@pytest.mark.parametrize("charged", [False, True])
def test_widom_tail_shift(lib, orc, charged):
    """Every trial's deltaU gains U_tail(framework + molecule) - U_tail(framework)
    (two tailEnergyCorrection evaluations in the oracle), and K_H is scaled by
    exp(-du_tail / T)."""
    A, _ = lib
    fw = W.cubic_framework(seed=3, charged=charged)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    guest = W.co2_guest(fw) if charged else W.ch4_guest(fw)
    ew = A.Ewald(0.31, 12.0, 5) if charged else None
    w = A.Widom(ff, p, fw.lattice, guest, 298.0, ewald=ew)
    r0, per0 = w.run(42, 0, 4096, per_trial=True)
    dut = w.set_tail_correction(True)
    r1, per1 = w.run(42, 0, 4096, per_trial=True)
    od = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    sp = np.asarray(fw.species, dtype=np.uint32)
    with_mol = np.concatenate([sp, np.asarray(guest["lj_species"], dtype=np.uint32)])
    want = orc.lj_tail(od, fw.lattice, with_mol) - orc.lj_tail(od, fw.lattice, sp)
    assert want < 0.0
    assert abs(dut - want) <= 1e-10 * abs(want)
    assert np.abs((per1 - per0) - want).max() <= 1e-10 * max(1.0, np.abs(per0).max())
    assert abs(r1["henry"] / r0["henry"] - np.exp(-want / 298.0)) <= 1e-12
    assert w.set_tail_correction(False) == dut
    r2 = w.run(42, 0, 4096)
    assert r2["henry"] == r0["henry"]
