"""The C ABI library: it loads, exports every entry point include/aleator_gb300.h
declares, and reports the reference's error behaviour (status codes mapped to
invalid_argument / out_of_range) for host-side checks, with no GPU needed."""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "aleator_gb300.h"


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(alea_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def so():
    from aleator_gb300.build import LIB, build

    if not LIB.exists():
        build()
    return LIB


def test_exports_every_declared_symbol(so):
    out = subprocess.run(["nm", "-D", "--defined-only", str(so)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\sT\s(alea_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    assert len(declared_symbols()) >= 40


def test_library_loads_and_reports(so):
    import aleator_gb300 as A

    lib = A.load_library()
    assert lib.alea_status_string(1) == b"invalid argument"
    ma, mi, arch = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    assert lib.alea_version(ctypes.byref(ma), ctypes.byref(mi), ctypes.byref(arch)) == 0
    assert arch.value == 103


def _fw():
    from aleator_gb300 import workloads as W
    return W.cubic_framework(seed=5)


def W_ch4(fw):
    from aleator_gb300 import workloads as W
    return W.ch4_guest(fw)


def test_host_side_errors_match_reference_exceptions(so):
    import aleator_gb300 as A

    fw = _fw()
    p = A.ParticleData.from_framework(fw)
    lj = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    # framework_energy_grid.cc:199-201: spacing must be positive -> invalid_argument
    with pytest.raises(ValueError, match="spacingAngstrom must be positive"):
        A.FrameworkEnergyGrid(lj, p, fw.lattice, [4], 0.0)
    # Lattice::validateCutoff message shape (the engines check it; the grid
    # constructor does not, as the reference's)
    big = A.LennardJones(fw.eps, fw.sigma, 13.5, A.SHIFTED)
    with pytest.raises(ValueError, match="exceeds half the perpendicular width"):
        A.Widom(big, p, fw.lattice, W_ch4(fw), 298.0)
    with pytest.raises(IndexError):
        A.FrameworkEnergyGrid(lj, p, fw.lattice, [99], 0.5)
    with pytest.raises(ValueError, match="alpha must be positive"):
        A.EwaldIncrementalState(A.Ewald(0.0, 12.0, 5), p, fw.lattice)
    with pytest.raises(ValueError, match="kMax must be at least 1"):
        A.ewald_reciprocal_terms(fw.lattice, 0.3, 0)
    with pytest.raises(ValueError, match="degenerate"):
        A.ewald_reciprocal_terms(np.zeros((3, 3)), 0.3, 4)
    q = np.ones(len(p))
    with pytest.raises(ValueError, match="not charge-neutral"):
        A.ewald_energy_breakdown(A.Ewald(0.3, 12.0, 4), A.ParticleData(fw.x, fw.y, fw.z, q), fw.lattice)


def test_host_side_formulas(so, orc):
    """Host-only entry points (k-term enumeration, acceptance ratios, EOS)."""
    import aleator_gb300 as A
    from aleator_gb300 import workloads as W

    fw = _fw()
    k, w = A.ewald_reciprocal_terms(fw.lattice, 0.31, 10)
    ko, wo = orc.ewald_terms(fw.lattice, 0.31, 10)
    assert np.array_equal(k, ko) and np.array_equal(w, wo)
    lib = A.load_library()
    f, v, T = 3.1e-5, 17000.0, 298.0
    for n, du in [(0, -500.0), (3, 120.0), (10, 0.0)]:
        r_ins = lib.alea_insertion_ratio(f, v, n, T, du)
        r_del = lib.alea_deletion_ratio(f, v, n + 1, T, -du)
        assert abs(r_ins * r_del - 1.0) < 1e-12  # test_gcmc_detailed_balance.cc identity
    assert abs(lib.alea_swap_ratio(1.0, 2.0, 3, 4, T, 50.0) *
               lib.alea_swap_ratio(2.0, 1.0, 5, 2, T, -50.0) - 1.0) < 1e-12
    for P in (1e4, 1e6):
        assert abs(A.peng_robinson_fugacity(*W.CO2_CRITICAL, 298.0, P) /
                   orc.pr_fugacity(*W.CO2_CRITICAL, 298.0, P) - 1) < 1e-13


def test_no_device_is_reported_not_faked(so):
    """Without a GPU the device paths fail with ALEA_ERR_NO_DEVICE instead of
    computing anything on the host."""
    import aleator_gb300 as A
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(A.AleatorError) as e:
        A.philox_u64(1, 2, 3, 8)
    assert e.value.status == 5
    fw = _fw()
    with pytest.raises(A.AleatorError) as e:
        A.FrameworkEnergyGrid(A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED),
                              A.ParticleData.from_framework(fw), fw.lattice, [4], 2.0)
    assert e.value.status == 5


def test_peng_robinson_mixture(so):
    """alea_peng_robinson_mixture (a host call) against the reference's values,
    its identities (test_peng_robinson.cc:147-210) and its argument errors."""
    import aleator_gb300 as A
    from aleator_gb300 import workloads as W
    from tests.test_oracle_golden import _pr_mixture_cases

    g, cases = _pr_mixture_cases()
    for row in g["rows"]:
        n, subs, kij = cases[int(row[0])]
        z, f = A.peng_robinson_mixture(subs, row[1], row[2], row[3:3 + n], kij)
        assert z == row[6]
        assert np.array_equal(f, row[7:7 + n])
    for row in g["fails"]:  # where the reference's Newton solve gives up, so does this one
        n, subs, kij = cases[int(row[0])]
        with pytest.raises(RuntimeError, match="did not converge"):
            A.peng_robinson_mixture(subs, row[1], row[2], row[3:3 + n], kij)
    # two identical components: the pure substance split by mole fraction
    ch4 = W.METHANE_CRITICAL
    for t, p in [(298.15, 1e5), (298.15, 1e7), (350.0, 5e6)]:
        fp = A.peng_robinson_fugacity(*ch4, t, p)
        for x0 in (0.5, 0.1, 0.999):
            _, f = A.peng_robinson_mixture([ch4, ch4], t, p, [x0, 1 - x0])
            assert abs(f[0] - x0 * fp) <= 1e-10 * fp and abs(f[1] - (1 - x0) * fp) <= 1e-10 * fp
    # ideal-gas limit
    _, f = A.peng_robinson_mixture([W.CO2_CRITICAL, (126.19, 3.3958e6, 0.0372)], 298.15, 1.0, [0.3, 0.7])
    assert abs(f[0] / 0.3 - 1) < 1e-6 and abs(f[1] / 0.7 - 1) < 1e-6
    bad = [
        (([ch4], 298.0, 1e5, [1.0], None), "needs at least 2 substances"),
        (([ch4, (0.0, 1e6, 0.0)], 298.0, 1e5, [0.5, 0.5], None), "criticalTemperatureKelvin must be positive"),
        (([ch4, ch4], 298.0, 1e5, [0.5, 0.5], [[0.1, 0.0], [0.0, 0.0]]), "diagonal must be zero"),
        (([ch4, ch4], 298.0, 1e5, [0.5, 0.5], [[0.0, 0.1], [0.2, 0.0]]), "must be symmetric"),
        (([ch4, ch4], 298.0, 1e5, [0.5, 0.5], [[0.0]]), "must be substances.size"),
        (([ch4, ch4], 298.0, 1e5, [1.0], None), "moleFractions.size"),
        (([ch4, ch4], 298.0, 1e5, [1.2, -0.2], None), "every mole fraction must be >= 0"),
        (([ch4, ch4], 298.0, 1e5, [0.5, 0.6], None), "must sum to 1"),
        (([ch4, ch4], -1.0, 1e5, [0.5, 0.5], None), "temperatureKelvin must be positive"),
        (([ch4, ch4], 298.0, 0.0, [0.5, 0.5], None), "totalPressurePascal must be positive"),
    ]
    for args, msg in bad:
        with pytest.raises(ValueError, match=msg):
            A.peng_robinson_mixture(*args)


def test_build_to_host_checks_before_device(so):
    """alea_grid_build_to_host: a null host array and the grid's own argument
    errors are reported before any device work; without a GPU a valid call
    reports ALEA_ERR_NO_DEVICE rather than building anything on the host."""
    import ctypes
    import torch
    import aleator_gb300 as A

    fw = _fw()
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    with pytest.raises(ValueError, match="host_tables"):
        A.FrameworkEnergyGrid.build_to_host(ff, p, fw.lattice, [4], 2.0, A.FP32, [0])
    buf = np.zeros(10)
    with pytest.raises(ValueError, match="spacingAngstrom must be positive"):
        A.FrameworkEnergyGrid.build_to_host(ff, p, fw.lattice, [4], -1.0, A.FP32,
                                            [buf.ctypes.data])
    if not torch.cuda.is_available():
        with pytest.raises(A.AleatorError) as e:
            A.FrameworkEnergyGrid.build_to_host(ff, p, fw.lattice, [4], 2.0, A.FP32,
                                                [buf.ctypes.data], keep=False)
        assert e.value.status == 5
        assert not buf.any()


C_PROGRAM = r"""
#include <stdio.h>
#include "aleator_gb300.h"
int main(int argc, char** argv) {
    alea_structure* s = NULL;
    if (argc < 2 || alea_read_cif(argv[1], &s) != ALEA_OK) return 2;
    uint64_t n = 0; uint32_t ns = 0;
    alea_structure_sizes(s, &n, &ns);
    double m[9];
    alea_structure_lattice(s, m);
    char sym[16];
    alea_structure_species_symbol(s, 0, sym, sizeof sym);
    alea_structure_destroy(s);
    const double tc[2] = {304.1282, 190.564}, pc[2] = {7.3773e6, 4.5992e6}, om[2] = {0.22394, 0.01142};
    const double x[2] = {0.4, 0.6};
    double z = 0.0, f[2];
    if (alea_peng_robinson_mixture(2, tc, pc, om, NULL, 298.0, 1e6, x, &z, f) != ALEA_OK) return 3;
    char msg[256];
    int bad = alea_read_cif("does/not/exist.cif", &s) == ALEA_ERR_RUNTIME;
    alea_last_error(msg, sizeof msg);
    printf("%llu %u %.3f %s %.6f %d %s\n", (unsigned long long)n, ns, m[0], sym, z, bad, msg);
    return 0;
}
"""


def test_plain_c_program_links_and_runs(so, tmp_path):
    """The header is C (C99, -pedantic) and a C program linked against the
    library runs its host entry points: the CIF reader, the Peng-Robinson
    mixture and the error channel."""
    import shutil
    import aleator_gb300 as A
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "prog.c"
    src.write_text(C_PROGRAM)
    exe = tmp_path / "prog"
    libdir = str(Path(so).parent)
    inc = str(Path(__file__).resolve().parents[1] / "include")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", inc,
                        str(src), "-o", str(exe), "-L", libdir, "-laleator_gb300",
                        f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    cif = Path(__file__).resolve().parent / "golden" / "cif" / "triclinic_symops.cif"
    out = subprocess.run([str(exe), str(cif)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    n, ns, a, sym, z, bad, *msg = out.stdout.split()
    s = A.read_cif(cif)
    assert int(n) == len(s.particles) and int(ns) == len(s.species_symbols) and sym == "Cu"
    assert float(a) == pytest.approx(9.10)
    z_py, _ = A.peng_robinson_mixture([(304.1282, 7.3773e6, 0.22394), (190.564, 4.5992e6, 0.01142)],
                                      298.0, 1e6, [0.4, 0.6])
    assert float(z) == pytest.approx(z_py, abs=1e-6)
    assert bad == "1" and "could not open file" in " ".join(msg)


def test_neutrality_errors_match_reference_text(so):
    """The engine constructor's neutrality checks (monte_carlo_engine.cc:273-293)
    with the reference's message text, before any device work: a non-neutral
    mixture species (GCMC), a non-neutral probe (Widom), a non-neutral framework."""
    import aleator_gb300 as A
    from aleator_gb300 import workloads as W

    fw = W.cubic_framework(seed=5, charged=True)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    ew = A.Ewald(0.31, 12.0, 5)
    bad = dict(W.co2_guest(fw), charge=[-0.35, 0.70, -0.30])  # +0.05 e
    tail = ("; every insertion/deletion/swap would drift the system away from neutrality, which "
            "electrostatics requires")
    msg = "MonteCarloEngine: GCMC species 1 is not individually charge-neutral (total site charge = "
    with pytest.raises(ValueError) as e:
        A.GcmcChains(ff, p, fw.lattice, [W.ch4_guest(fw), bad], 298.0, [[1e5, 1e5]], [1], [1], ewald=ew)
    qsum = 0.0
    for c in bad["charge"]:  # summed in site order, formatted as std::to_string (%f)
        qsum += c
    assert str(e.value) == msg + f"{qsum:f} e)" + tail
    with pytest.raises(ValueError) as e:
        A.Widom(ff, p, fw.lattice, bad, 298.0, ewald=ew)
    assert str(e.value).startswith("MonteCarloEngine: GCMC species 0 is not individually charge-neutral")
    assert str(e.value).endswith(tail)
    q = fw.charge.copy()
    q[0] += 0.5
    p2 = A.ParticleData(fw.x, fw.y, fw.z, q, fw.species)
    for make in (lambda: A.Widom(ff, p2, fw.lattice, W.co2_guest(fw), 298.0, ewald=ew),
                 lambda: A.GcmcChains(ff, p2, fw.lattice, W.co2_guest(fw), 298.0, [1e5], [1], [1],
                                      ewald=ew)):
        with pytest.raises(ValueError, match=r"^MonteCarloEngine: framework is not charge-neutral "
                                             r"\(total charge = 0\.5\d* e\)$"):
            make()


def test_block_cache_keying(so):
    """The device block cache hands a kept block only to a request of the same
    size on the same device (fake pointers, no device call); with no device
    nothing is kept and the trim call frees nothing."""
    import aleator_gb300 as A

    lib = A.load_library()
    assert lib.alea_test_block_cache() == 0
    n = ctypes.c_uint64(7)
    assert lib.alea_cached_bytes(ctypes.byref(n)) == 0 and n.value == 0
    assert lib.alea_release_cached(ctypes.byref(n)) == 0 and n.value == 0
    assert lib.alea_release_cached(None) == 0


def test_no_alloc_site_counts_cannot_wrap(so):
    """alea_ewald_propose_no_alloc checks each site count on its own, so a sum
    that wraps around 2^64 is rejected before any site is copied."""
    import aleator_gb300 as A
    from aleator_gb300._lib import _lattice, _D

    lib = A.load_library()
    lat = _lattice(np.eye(3) * 30.0)
    add = np.zeros(8)
    for n_removed, n_added in ((2 ** 64 - 1, 2), (65, 0), (0, 65), (40, 25), (2, 2 ** 64 - 1)):
        status = lib.alea_ewald_propose_no_alloc(None, None, None, None, 0, 0.3,
                                                 ctypes.byref(lat), add.ctypes.data_as(_D),
                                                 n_removed, add.ctypes.data_as(_D), n_added, 1,
                                                 None)
        assert status == 1, (n_removed, n_added)
        buf = ctypes.create_string_buffer(256)
        lib.alea_last_error(buf, 256)
        assert b"at most 64 removed + added sites" in buf.value
