"""The CIF structure reader (alea_read_cif) against the reference's readCif
(io/structure_io.cc:177-245): bit-identical particles, cell, masses,
occupancies, species symbols and labels, and the same CifParseError messages.

Inputs: the synthetic CIF files in tests/golden/cif (written for these tests:
P1 with charges, esd suffixes and ?/. placeholders; a triclinic cell with
symmetry operations and atoms on special positions; a hexagonal cell through
_space_group_symop_operation_xyz with upper-case tags, a text field, tabs, a
row split over lines and a second data block; fourteen malformed files) against
the fixture the reference produced from them, and, where the reference tree is
present, the reference's own structure files read by both readers."""
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from conftest import golden

CIF_DIR = Path(__file__).resolve().parent / "golden" / "cif"


@pytest.fixture(scope="module")
def A():
    import aleator_gb300 as A
    from aleator_gb300.build import LIB, build

    if not LIB.exists():
        build()
    return A


def _same(s, r):
    assert np.array_equal(s.lattice, r["lattice"])
    for k in ("x", "y", "z", "charge", "species"):
        assert np.array_equal(getattr(s.particles, k), r[k]), k
    assert np.array_equal(s.mass, r["mass"])
    assert np.array_equal(s.occupancy, r["occupancy"])
    assert list(s.species_symbols) == [str(v) for v in r["symbols"]]
    assert list(s.source_label) == [str(v) for v in r["labels"]]


def test_reader_matches_reference_fixture(A):
    g = golden("cif_structures")
    files = sorted(CIF_DIR.glob("*.cif"))
    assert len(files) >= 17
    for f in files:
        if f"{f.stem}__error" in g:
            with pytest.raises(RuntimeError) as e:
                A.read_cif(f)
            assert str(e.value) == str(g[f"{f.stem}__error"]), f.name
            continue
        s = A.read_cif(f)
        _same(s, {k: g[f"{f.stem}__{k}"] for k in ("lattice", "x", "y", "z", "charge", "mass",
                                                    "species", "occupancy", "symbols", "labels")})


def test_expansion_and_species(A):
    """Orbits: four operations on the triclinic cell give 4 images of a general
    position and 2 of an inversion centre; species numbered by first
    appearance; charges and occupancies default to 0 and 1."""
    s = A.read_cif(CIF_DIR / "triclinic_symops.cif")
    labels = s.source_label
    assert labels.count("Cu2+") == 2 and labels.count("C12A") == 4
    assert s.species_symbols == ["Cu", "Cl", "C", "O", "Si", "N", "P"]
    assert (s.particles.charge == 0).all() and (s.occupancy == 1).all()
    p = A.read_cif(CIF_DIR / "p1_charged.cif")
    assert p.species_symbols == ["Zn", "O", "C", "H"]
    assert list(p.occupancy) == [1.0, 1.0, 0.5, 1.0, 0.95, 1.0]
    assert p.particles.charge[1] == -0.6718 and p.particles.charge[3] == 0.0
    # every atom inside the cell: fractional coordinates in [0, 1)
    f = np.stack([p.particles.x, p.particles.y, p.particles.z], 1) @ np.linalg.inv(p.lattice)
    assert (f > -1e-12).all() and (f < 1 + 1e-12).all()


def test_missing_file(A, ref):
    path = str(CIF_DIR / "does_not_exist.cif")
    with pytest.raises(RuntimeError) as mine:
        A.read_cif(path)
    with pytest.raises(RuntimeError) as theirs:
        ref.read_cif(path)
    assert str(mine.value) == str(theirs.value) == "could not open file: " + path


def test_reference_structures_read_identically(A, ref):
    """The reference's own structure files (MOF and zeolite cells, 30 to 576
    atoms after expansion) through both readers."""
    files = sorted((O.REFERENCE_ROOT / "tests").rglob("*.cif"))
    if not files:
        pytest.skip("the reference's structure files are not present")
    for f in files:
        _same(A.read_cif(f), ref.read_cif(f))
