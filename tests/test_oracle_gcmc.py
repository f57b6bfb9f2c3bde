"""The oracle's GCMC chain (oracle/aleator_oracle_gcmc.c) against the
reference's own MonteCarloEngine (oracle/_ref): bit-identical trajectories,
molecule counts and Ewald cache energies."""
import numpy as np
import pytest

import oracle as O
from aleator_gb300 import workloads as W


@pytest.mark.parametrize("charged", [False, True])
def test_chain_bit_identical_to_reference(orc, ref, charged):
    fw = W.cubic_framework(seed=21, charged=charged)
    if charged:
        fw.charge = fw.charge * 0.15
    ff = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    ew = dict(alpha=0.31, rc=12.0, kmax=5) if charged else None
    guest = W.co2_guest(fw) if charged else W.ch4_guest(fw)
    fug = ref.pr_fugacity(*(W.CO2_CRITICAL if charged else W.METHANE_CRITICAL), 298.0, 1e6)
    a = ref.gcmc(ff, ew, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guest, 298.0, fug, 9, 4)
    b = orc.gcmc(ff, ew, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guest, 298.0, fug, 9, 4)
    for _ in range(4):
        a.run(300)
        b.run(300)
        assert a.molecules() == b.molecules()
        assert np.array_equal(a.positions(), b.positions())
        assert a.ewald_energy() == b.ewald_energy()
