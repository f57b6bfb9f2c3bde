"""The reference's physics cross-checks of this path, run through the GPU
Widom and GCMC kernels (FP64, the parity form).

* Widom K_H against the slope of a low-pressure GCMC isotherm
  (test_gcmc_widom_henry.cc:66-157): 16 Å cubic cell with 8 LJ sites, a
  single-site adsorbate, 150 K; Widom with 2e6 trials (seed 1, stream 0), then
  six GCMC replicas (seed 1000, streams 0-5) at the fugacity that puts
  <N> = 0.3, 40 000 equilibration moves and 200 000 production moves sampled
  every 20; the implied K_H = <N>/(V f) within 2 % of Widom's.
* CH4 in the real IRMOF-1 cell (test_gcmc_ch4_irmof1_isotherm.cc:84-215):
  the structure as the reference's readCif reads it and the GenericMOFs LJ
  parameters of that test (tests/golden/irmof1.npz, made by
  tests/golden/make_golden.py from the reference's own files), rc 12 Å
  shifted, 298 K; Widom with 5e5 trials (seed 2026, stream 999), one GCMC
  chain at 0.1 bar (Peng-Robinson fugacity; seed 2026, stream 0), 30 000
  equilibration moves, 90 000 production moves in 10 blocks sampled every
  move; the implied K_H within 12 % of Widom's.
The chains run the reference engine's draw order, so they follow the same
trajectories as the reference's own tests (the move-for-move parity tests
show that)."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

K_PASCAL_TO_INTERNAL = 1.0 / (1.380649e-23 * 1.0e30)  # monte_carlo_engine.hpp:184


def test_widom_henry_matches_gcmc_slope(lib):
    A, _ = lib
    box = 16.0
    c = [box * 0.25, box * 0.75]
    pts = np.array([(x, y, z) for x in c for y in c for z in c])
    fw = A.ParticleData(pts[:, 0], pts[:, 1], pts[:, 2], None, np.zeros(8, dtype=np.uint32))
    lattice = np.eye(3) * box
    ff = A.LennardJones([100.0, 100.0], [3.0, 3.5], 6.0, A.SHIFTED)
    guest = dict(x=[0.0], y=[0.0], z=[0.0], lj_species=[1], charge=[0.0])
    T = 150.0
    kh = A.Widom(ff, fw, lattice, guest, T).run(1, 0, 2_000_000)["henry"]
    assert kh > 0.0
    volume = box ** 3
    f_internal = 0.3 / (kh * volume)
    f_pa = f_internal / K_PASCAL_TO_INTERNAL
    n_rep = 6
    chains = A.GcmcChains(ff, fw, lattice, guest, T, [f_pa] * n_rep, [1000] * n_rep,
                          list(range(n_rep)), max_molecules=64)
    chains.run(40_000)
    sums = np.zeros(n_rep)
    samples = 0
    for _ in range(0, 200_000, 20):
        chains.run(20)
        sums += [chains.info(r)["molecules"] for r in range(n_rep)]
        samples += 1
    loading = sums / samples / volume
    mean = loading.mean()
    se = loading.std(ddof=1) / np.sqrt(n_rep)
    implied = mean / f_internal
    rel = abs(implied - kh) / kh
    print(f"\nWidom K_H {kh:.6e}; GCMC-implied {implied:.6e} +/- {se / f_internal:.2e} "
          f"({100 * se / f_internal / kh:.2f} % s.e.); difference {100 * rel:.3f} %")
    assert rel < 0.02


def test_irmof1_ch4_widom_matches_gcmc_at_0p1_bar(lib):
    A, _ = lib
    g = golden("irmof1")
    fw = A.ParticleData(g["x"], g["y"], g["z"], g["charge"], g["species"])
    ff = A.LennardJones(g["eps"], g["sigma"], float(g["cutoff"]), A.SHIFTED)
    ch4 = len(g["eps"]) - 1
    guest = dict(x=[0.0], y=[0.0], z=[0.0], lj_species=[ch4], charge=[0.0])
    T = 298.0
    volume = abs(np.linalg.det(g["lattice"]))
    kh = A.Widom(ff, fw, g["lattice"], guest, T).run(2026, 999, 500_000)["henry"]
    assert kh > 0.0
    f_pa = A.peng_robinson_fugacity(190.6, 4.599e6, 0.011, T, 0.1e5)  # kMethane, 0.1 bar
    f_internal = f_pa * K_PASCAL_TO_INTERNAL
    ch = A.GcmcChains(ff, fw, g["lattice"], guest, T, [f_pa], [2026], [0], max_molecules=64)
    ch.run(30_000)
    prev = ch.info()["sum_molecules"]
    blocks = []
    for _ in range(10):
        ch.run(9_000)
        cur = ch.info()["sum_molecules"]
        blocks.append((cur - prev) / 9_000)
        prev = cur
    mean_n = float(np.mean(blocks))
    se_n = float(np.std(blocks, ddof=1) / np.sqrt(10))
    implied = mean_n / volume / f_internal
    rel = abs(implied - kh) / kh
    print(f"\nIRMOF-1 CH4 0.1 bar: <N> {mean_n:.4f} +/- {se_n:.4f}; implied K_H {implied:.6e}; "
          f"Widom {kh:.6e}; difference {100 * rel:.2f} % "
          f"({100 * se_n / volume / f_internal / kh:.2f} % s.e.)")
    assert rel < 0.12
