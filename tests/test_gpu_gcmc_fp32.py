"""The FP32 form of the GCMC chains (FP32 LJ and real-space pair terms after an
FP64 minimum image, FP32 S(k) phases; every sum, S(k), the self and exclusion
terms and the acceptance in FP64) against the FP64 form, which is move for
move equal to the oracle (test_gpu_gcmc.py).

Per move: from the same seeds both forms draw the same numbers and, while
their decisions agree, make the same moves. Each move's dU agrees within
1e-5 x max(kT, |dU|) for insertions and deletions (dU is then one molecule's
energy); a translation's or rotation's dU is a difference of two molecule
energies, so it agrees within 1e-5 x max(kT, |dU|, E), E the largest molecule
energy met in the run. Statistics: the mean loading of independent chains
within 3 combined standard errors of the FP64 form's."""
import numpy as np
import pytest

from aleator_gb300 import workloads as W

pytestmark = pytest.mark.gpu

KT = 298.0


def _chains(A, fw, guest, ew, fugs, seeds, streams, precision, max_molecules=256):
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    return A.GcmcChains(ff, p, fw.lattice, guest, KT, fugs, seeds, streams, ewald=ew,
                        max_molecules=max_molecules, precision=precision)


@pytest.mark.parametrize("charge_scale,kmax", [(1.0, None), (0.15, None), (0.15, 36)])
def test_fp32_move_energies_track_fp64(lib, orc, charge_scale, kmax):
    """kmax None: the 1e-6 rule (10 here); 36: the FP32 form forms the
    (n0, n1) phase products per term (its table would not fit)."""
    A, _ = lib
    fw = W.cubic_framework(seed=12, charged=True)
    fw.charge = fw.charge * charge_scale
    alpha, k_rule = W.ewald_parameters(fw.lattice, 12.0)
    ew = A.Ewald(alpha, 12.0, k_rule if kmax is None else kmax)
    fug = orc.pr_fugacity(*W.CO2_CRITICAL, KT, 1e6)
    guest = W.co2_guest(fw)
    c64 = _chains(A, fw, guest, ew, [fug], [3], [7], A.FP64)
    c32 = _chains(A, fw, guest, ew, [fug], [3], [7], A.FP32)
    compared = {0: 0, 1: 0, 2: 0, 3: 0}
    e_scale = 0.0
    prev = c64.info()["attempted"]
    for _ in range(1000):
        c64.run(1)
        c32.run(1)
        i64, i32 = c64.info(), c32.info()
        if i64["call_index"] != i32["call_index"] or i64["molecules"] != i32["molecules"]:
            break  # a decision differed: the trajectories part here
        step = np.array(i64["attempted"]) - np.array(prev)
        prev = i64["attempted"]
        if step.sum() == 0:
            continue  # nothing to act on: no energy evaluated
        move = int(np.argmax(step))
        if i64["attempted"] == i32["attempted"] and np.isfinite(i64["last_du"]):
            d64, d32 = i64["last_du"], i32["last_du"]
            if abs(d64) > 1e5:  # overlapping trial: both reject, the size is irrelevant
                continue
            if move >= 2:
                e_scale = max(e_scale, abs(d64))
                assert abs(d32 - d64) <= 1e-5 * max(KT, abs(d64)), (move, d32, d64)
            else:
                assert abs(d32 - d64) <= 1e-5 * max(KT, abs(d64), e_scale), (move, d32, d64, e_scale)
            compared[move] += 1
    assert sum(compared.values()) >= 300, compared
    assert compared[2] >= 50, compared
    assert compared[0] + compared[1] >= 50, compared


def test_fp32_loading_statistics_match_fp64(lib, orc):
    A, _ = lib
    n = 64
    # CH4, LJ only
    fw = W.cubic_framework(seed=11)
    fug = orc.pr_fugacity(*W.METHANE_CRITICAL, KT, 5e6)
    out = {}
    for prec in (A.FP64, A.FP32):
        ch = _chains(A, fw, W.ch4_guest(fw), None, [fug] * n, list(range(40, 40 + n)), [1] * n, prec)
        ch.run(5000)
        before = [ch.info(c)["sum_molecules"] for c in range(n)]
        ch.run(10000)
        out[prec] = np.array([(ch.info(c)["sum_molecules"] - before[c]) / 10000 for c in range(n)])
    m64, m32 = out[A.FP64], out[A.FP32]
    se = np.hypot(m64.std(ddof=1), m32.std(ddof=1)) / np.sqrt(n)
    assert m64.mean() > 1.0
    assert abs(m32.mean() - m64.mean()) <= 3 * se, (m32.mean(), m64.mean(), se)
    # charged CO2 in a weakened field (equilibrates within the run)
    fw = W.cubic_framework(seed=13, charged=True)
    fw.charge = fw.charge * 0.15
    ew = A.Ewald(0.31, 12.0, 6)
    fug = orc.pr_fugacity(*W.CO2_CRITICAL, KT, 1e6)
    for prec in (A.FP64, A.FP32):
        ch = _chains(A, fw, W.co2_guest(fw), ew, [fug] * n, list(range(80, 80 + n)), [2] * n, prec)
        ch.run(3000)
        before = [ch.info(c)["sum_molecules"] for c in range(n)]
        ch.run(6000)
        out[prec] = np.array([(ch.info(c)["sum_molecules"] - before[c]) / 6000 for c in range(n)])
    m64, m32 = out[A.FP64], out[A.FP32]
    se = np.hypot(m64.std(ddof=1), m32.std(ddof=1)) / np.sqrt(n)
    assert m64.mean() > 1.0
    assert abs(m32.mean() - m64.mean()) <= 3 * se, (m32.mean(), m64.mean(), se)


def test_fp32_with_energy_grid_matches_fp64_loading(lib, orc):
    """Both forms reading an energy grid (FP32-form grid for the FP32 chains,
    FP64-form grid for the FP64 chains): equal mean loadings."""
    A, _ = lib
    n = 64
    fw = W.cubic_framework(seed=11)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    guest = W.ch4_guest(fw)
    fug = orc.pr_fugacity(*W.METHANE_CRITICAL, KT, 5e6)
    out = {}
    for prec in (A.FP64, A.FP32):
        grid = A.FrameworkEnergyGrid(ff, p, fw.lattice, [guest["lj_species"][0]], 0.3, prec)
        ch = _chains(A, fw, guest, None, [fug] * n, list(range(40, 40 + n)), [3] * n, prec)
        ch.set_grid(grid)
        ch.run(5000)
        before = [ch.info(c)["sum_molecules"] for c in range(n)]
        ch.run(10000)
        out[prec] = np.array([(ch.info(c)["sum_molecules"] - before[c]) / 10000 for c in range(n)])
    m64, m32 = out[A.FP64], out[A.FP32]
    se = np.hypot(m64.std(ddof=1), m32.std(ddof=1)) / np.sqrt(n)
    assert m64.mean() > 1.0
    assert abs(m32.mean() - m64.mean()) <= 3 * se, (m32.mean(), m64.mean(), se)


def test_fp32_mixture_loading_matches_fp64(lib, orc):
    """CH4 + charged CO2 (field weakened to 0.15) with identity swaps: per
    species, the mean loading of the FP32 chains within 3 combined standard
    errors of the FP64 chains'."""
    A, _ = lib
    n = 64
    fw = W.cubic_framework(seed=13, charged=True)
    fw.charge = fw.charge * 0.15
    ew = A.Ewald(0.31, 12.0, 6)
    guests = [W.co2_guest(fw), W.ch4_guest(fw)]
    fugs = [orc.pr_fugacity(*W.CO2_CRITICAL, KT, 5e5), orc.pr_fugacity(*W.METHANE_CRITICAL, KT, 2e6)]
    out = {}
    for prec in (A.FP64, A.FP32):
        ch = _chains(A, fw, guests, ew, [fugs] * n, list(range(200, 200 + n)), [5] * n, prec)
        ch.run(3000)
        snaps = []
        for _ in range(12):
            ch.run(500)
            snaps.append([ch.info(c)["species_molecules"][:2] for c in range(n)])
        out[prec] = np.array(snaps, dtype=np.float64).mean(axis=0)  # chains x species
        info = ch.info(0)
        assert info["attempted"][4] > 0 and info["accepted"][4] > 0
    for k in range(2):
        m64, m32 = out[A.FP64][:, k], out[A.FP32][:, k]
        se = np.hypot(m64.std(ddof=1), m32.std(ddof=1)) / np.sqrt(n)
        assert m64.mean() > 0.5, (k, m64.mean())
        assert abs(m32.mean() - m64.mean()) <= 3 * se, (k, m32.mean(), m64.mean(), se)


def test_fp32_far_pairs_in_fixed_point_large_cell(lib, orc):
    """A cell above 100 x the 6 A near sphere (the 2x2x2 triclinic supercell,
    3 376 charged atoms): far pairs take the fixed-point FP32 displacement,
    near ones double-float. Move energies as in the small-cell test: insertion
    and deletion dU within 1e-5 x max(kT, |dU|) of the FP64 form."""
    A, _ = lib
    fw = W.triclinic_supercell(reps=2)
    assert abs(np.linalg.det(np.asarray(fw.lattice))) > 100 * 4 / 3 * np.pi * 6 ** 3
    fw.charge = fw.charge * 0.15
    alpha, _ = W.ewald_parameters(fw.lattice, 12.0)
    ew = A.Ewald(alpha, 12.0, 8)
    fug = orc.pr_fugacity(*W.CO2_CRITICAL, KT, 1e6)
    guest = W.co2_guest(fw)
    c64 = _chains(A, fw, guest, ew, [fug], [5], [3], A.FP64)
    c32 = _chains(A, fw, guest, ew, [fug], [5], [3], A.FP32)
    compared = {0: 0, 1: 0, 2: 0, 3: 0}
    e_scale = 0.0
    prev = c64.info()["attempted"]
    for _ in range(900):
        c64.run(1)
        c32.run(1)
        i64, i32 = c64.info(), c32.info()
        if i64["call_index"] != i32["call_index"] or i64["molecules"] != i32["molecules"]:
            break
        step = np.array(i64["attempted"]) - np.array(prev)
        prev = i64["attempted"]
        if step.sum() == 0:
            continue
        move = int(np.argmax(step))
        if i64["attempted"] == i32["attempted"] and np.isfinite(i64["last_du"]):
            d64, d32 = i64["last_du"], i32["last_du"]
            if abs(d64) > 1e5:
                continue
            if move >= 2:
                e_scale = max(e_scale, abs(d64))
                assert abs(d32 - d64) <= 1e-5 * max(KT, abs(d64)), (move, d32, d64)
            else:
                assert abs(d32 - d64) <= 1e-5 * max(KT, abs(d64), e_scale), (move, d32, d64, e_scale)
            compared[move] += 1
    assert sum(compared.values()) >= 150, compared
    assert compared[2] >= 20, compared
