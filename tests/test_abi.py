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


def test_host_side_errors_match_reference_exceptions(so):
    import aleator_gb300 as A

    fw = _fw()
    p = A.ParticleData.from_framework(fw)
    lj = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    # framework_energy_grid.cc:199-201: spacing must be positive -> invalid_argument
    with pytest.raises(ValueError, match="spacingAngstrom must be positive"):
        A.FrameworkEnergyGrid(lj, p, fw.lattice, [4], 0.0)
    # Lattice::validateCutoff message shape
    with pytest.raises(ValueError, match="exceeds half the perpendicular width"):
        A.FrameworkEnergyGrid(A.LennardJones(fw.eps, fw.sigma, 13.5, A.SHIFTED), p, fw.lattice, [4], 0.5)
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
