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
        assert np.array_equal(getattr(s.particles, k), r[k], equal_nan=k != "species"), k
    assert np.array_equal(s.mass, r["mass"])
    assert np.array_equal(s.occupancy, r["occupancy"], equal_nan=True)
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
    files = sorted((O.REFERENCE_ROOT / "tests").rglob("*.cif")) if O.REFERENCE_ROOT else []
    if not files:
        pytest.skip("the reference's structure files are not present")
    for f in files:
        _same(A.read_cif(f), ref.read_cif(f))


def _cif_text(ops, coords, cell=("10.0", "11.0", "12.0", "90", "95.5", "100")):
    lines = ["data_fuzz",
             f"_cell_length_a {cell[0]}", f"_cell_length_b {cell[1]}", f"_cell_length_c {cell[2]}",
             f"_cell_angle_alpha {cell[3]}", f"_cell_angle_beta {cell[4]}",
             f"_cell_angle_gamma {cell[5]}", "loop_", "_symmetry_equiv_pos_as_xyz"]
    lines += [f"'{op}'" for op in ops]
    lines += ["loop_", "_atom_site_label", "_atom_site_fract_x", "_atom_site_fract_y",
              "_atom_site_fract_z", "_atom_site_charge"]
    for i, (x, y, z, q) in enumerate(coords):
        lines.append(f"C{i} {x} {y} {z} {q}")
    return "\n".join(lines) + "\n"


def test_reader_fuzzed_against_reference(A, ref, tmp_path):
    """Generated symmetry operations (signed terms, fractions, decimals, stray
    characters) and coordinate tokens (esd suffixes, placeholders, exponents,
    garbage): the library and the reference read the same particles or fail
    with the same message. One pass draws from the valid grammar (most files
    parse, so the particles are compared), one from anything."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    def ops_of(signs, numbers, variables, sizes):
        term = st.builds(lambda a, b, c: a + b + c, st.sampled_from(signs), st.sampled_from(numbers),
                         st.sampled_from(variables))
        comp = st.lists(term, min_size=1, max_size=3).map("".join)
        return st.lists(st.lists(comp, min_size=sizes[0], max_size=sizes[1]).map(",".join),
                        min_size=1, max_size=4)

    valid_ops = ops_of(["", "+", "-"], ["", "1", "1/2", "1/3", "2/3", "0.5", "3/4"],
                       ["x", "y", "z", "X"], (3, 3))
    any_ops = ops_of(["", "+", "-"], ["", "1", "2", "1/2", "0.5", "1/", ".25", "3/"],
                     ["x", "y", "z", "", "w", "Y"], (1, 4))
    valid_num = st.sampled_from(["0.1", "0.25(3)", "1e-3", ".5", "5.", "-0.75", "1.5", "0.333333",
                                 "0.0", "1.0", "2(1)"])
    any_num = st.sampled_from(["0.1", "?", ".", "abc", "nan", "1e400", "0.2(", "-"])
    case = {"n": 0, "ok": 0}

    def compare(ops, coords):
        case["n"] += 1
        f = tmp_path / f"f{case['n']}.cif"
        f.write_text(_cif_text(ops, coords))
        try:
            r, rerr = ref.read_cif(f), None
        except RuntimeError as e:
            r, rerr = None, str(e)
        try:
            s, serr = A.read_cif(f), None
        except RuntimeError as e:
            s, serr = None, str(e)
        assert rerr == serr, (ops, coords, rerr, serr)
        if r is not None:
            _same(s, r)
            case["ok"] += 1

    settings = hyp.settings(max_examples=150, deadline=None, database=None, derandomize=True)

    @settings
    @hyp.given(ops=valid_ops, coords=st.lists(st.tuples(valid_num, valid_num, valid_num, valid_num),
                                              min_size=1, max_size=3))
    def valid(ops, coords):
        compare(ops, coords)

    @settings
    @hyp.given(ops=any_ops, coords=st.lists(st.tuples(any_num, valid_num, any_num, any_num),
                                            min_size=1, max_size=3))
    def anything(ops, coords):
        compare(ops, coords)

    valid()
    assert case["ok"] >= 100, case  # the valid grammar parses: particles compared
    anything()


def test_document_grammar_fuzzed_against_reference(A, ref, tmp_path):
    """Random constructs between the sections of a valid file: comments, blank
    lines, tags with bare, quoted and text-field values, extra loops whose rows
    span lines (or fall short), unterminated quotes and text fields, stray
    words, a second data block. Same particles or the same message (with the
    same line number) from both readers."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies
    noise = st.sampled_from([
        "# a comment line", "", "   ", "\t# indented comment",
        "_extra_tag value", "_extra_tag 'two words'", '_extra_tag "it\'s quoted"',
        "_extra_tag\n;\nfree text\nover lines\n;", "_extra_tag\n; one-liner\n;",
        "_extra_tag\nnext_line_value", "_UPPER_Tag 3.5(2)",
        "loop_\n_l_a\n_l_b\n1 2\n3\n4", "loop_\n_l_a\n_l_b\n'x y' \"z\"\n# c\n5 6",
        "loop_\n_l_a\n_l_b\n1 2 3",                      # a short row
        "loop_\n# no columns", "_bad_tag 'unterminated", "_text\n; never closed",
        "stray words here", "data_second\n_cell_length_a 1", "_tag_at_end",
    ])
    head = ["data_grammar", "_cell_length_a 9.5", "_cell_length_b 10.5", "_cell_length_c 11.5",
            "_cell_angle_alpha 88", "_cell_angle_beta 92", "_cell_angle_gamma 101"]
    sym = ["loop_", "_symmetry_equiv_pos_as_xyz", "'x,y,z'", "'-x,-y,-z'"]
    atoms = ["loop_", "_atom_site_label", "_atom_site_type_symbol", "_atom_site_fract_x",
             "_atom_site_fract_y", "_atom_site_fract_z", "O1 O 0.1 0.2 0.3", "Si1 Si 0.5 0.5",
             "0.5", "C2 C 0.0 0.0 0.0"]
    sections = [head, sym, atoms]
    case = {"n": 0, "ok": 0}

    @hyp.settings(max_examples=200, deadline=None, database=None, derandomize=True)
    @hyp.given(inserts=st.lists(st.lists(noise, max_size=2), min_size=4, max_size=4))
    def check(inserts):
        case["n"] += 1
        parts = []
        for k in range(3):
            parts += inserts[k]
            parts += sections[k]
        parts += inserts[3]
        f = tmp_path / f"g{case['n']}.cif"
        f.write_text("\n".join(parts) + "\n")
        try:
            r, rerr = ref.read_cif(f), None
        except RuntimeError as e:
            r, rerr = None, str(e)
        try:
            s, serr = A.read_cif(f), None
        except RuntimeError as e:
            s, serr = None, str(e)
        assert rerr == serr, (inserts, rerr, serr)
        if r is not None:
            _same(s, r)
            case["ok"] += 1

    check()
    assert case["ok"] >= 30, case


def test_irmof1_fixture_is_the_readers_output(A):
    """tests/golden/irmof1.npz (the real IRMOF-1 cell the GPU physics test
    runs) equals this library's reader on the reference's IRMOF-1.cif, where
    the reference tree is present."""
    g = golden("irmof1")
    if O.REFERENCE_ROOT is None:
        pytest.skip("the reference tree is not present")
    f = O.REFERENCE_ROOT / "tests/validation/data/irmof1/IRMOF-1.cif"
    if not f.exists():
        pytest.skip("the reference's IRMOF-1.cif is not present")
    s = A.read_cif(f)
    assert np.array_equal(np.asarray(s.lattice), g["lattice"])
    for k in ("x", "y", "z", "species"):
        assert np.array_equal(getattr(s.particles, k), g[k])
    assert list(s.species_symbols) == [str(v) for v in g["symbols"]]
    assert len(g["eps"]) == len(s.species_symbols) + 1
