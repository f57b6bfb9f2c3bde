"""The FP32 form of the energy grid at the benchmark's own configuration: the
4x4x4 triclinic supercell (24 Å base cell, 70/80/100 degrees, 27 008 atoms),
0.2 Å spacing (457 x 437 x 437 nodes), the two LJ site types of CO2,
truncated-shifted at 12.8 Å (framework_energy_grid.cc:193-249).

* The FP64 form of the same grid against the oracle's restatement of the
  reference's loop on a strided sample of 2 048 nodes: 1e-10 relative with a
  1 K floor, as every FP64 grid test.
* Every node of the FP32 form against the FP64 form, by node class:
    - |E| >= kT (kT = 298 K): 1e-5 relative, |dE| <= 1e-5 |E|;
    - |E| < kT: |dE| <= 1e-5 kT. Such a node's energy is a sum of pair terms
      of up to ~1e3 K that cancel to below kT, so FP32 pair terms (~1e-7
      relative rounding each) cannot give it 1e-5 of its own size; the bound
      keeps the node's Boltzmann factor exp(-E/kT), the quantity Widom and
      GCMC use, within 1e-5 relative;
    - nodes at the 1e5 K cap in the FP64 form (about half the nodes of this
      dense framework) and nodes in (1e4, 1e5) K: 1e-5 relative (the FP32
      form's near-overlap pairs are double-float; a node just below the cap
      in FP32 is one whose exact energy lies just above it).
The measured figures (maximum pure relative error, maximum error against
max(kT, |E|), the count of nodes above 1e-5 pure relative, and the largest |E|
among them) are printed."""
import os

import numpy as np
import pytest

import oracle as O
from bench import fp32_error_stats

KT = 298.0

pytestmark = pytest.mark.gpu


def test_c5_fp32_grid_by_node_class(lib, orc):
    A, _ = lib
    from aleator_gb300 import workloads as W
    fw = W.triclinic_supercell(reps=4)
    assert fw.n_atoms == 27008
    guests = [fw.guest_species["CO2_C"], fw.guest_species["CO2_O"]]
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    g64 = A.FrameworkEnergyGrid(ff, p, fw.lattice, guests, 0.2, A.FP64)
    assert g64.point_counts() == (457, 437, 437)
    nodes = 457 * 437 * 437
    t64 = {s: g64.table(s) for s in guests}
    del g64
    # the FP64 form against the oracle on a strided sample (pins the FP64 form here)
    od = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    stride = nodes // 2048
    idx = np.arange(0, nodes, stride)[:2048]
    threads = os.cpu_count() or 4
    for s in guests:
        ref = _sample(orc, od, fw, s, idx, threads)
        err = np.abs(t64[s][idx] - ref) / np.maximum(1.0, np.abs(ref))
        assert err.max() <= 1e-10, (s, err.max())
    g32 = A.FrameworkEnergyGrid(ff, p, fw.lattice, guests, 0.2, A.FP32)
    for s in guests:
        t32 = g32.table(s)
        st = fp32_error_stats(t32, t64[s])
        print(f"\nC5 FP32 grid, guest species {s}: {st}")
        assert st["max_pure_rel_capped"] <= 1e-5, st
        assert st["max_pure_rel_1e4_to_1e5_K"] <= 1e-5, st
        assert st["max_rel_kT_floor"] <= 1e-5, st
        assert st["max_pure_rel_abs_E_ge_kT"] <= 1e-5, st
        assert st["max_abs_E_above_1e-5_pure_rel_K"] < KT, st


def _sample(orc, od, fw, s, idx, threads):
    """The oracle at the sampled nodes, split over host threads by node (the
    oracle's calls release the interpreter lock)."""
    from concurrent.futures import ThreadPoolExecutor

    def one(i):
        return orc.grid_build(od, fw.lattice, fw.x, fw.y, fw.z, fw.species, s, 0.2,
                              node_begin=int(i), node_end=int(i) + 1, threads=1)

    with ThreadPoolExecutor(max_workers=threads) as ex:
        return np.concatenate(list(ex.map(one, idx)))
