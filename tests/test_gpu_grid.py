"""Framework energy grid on the GPU against the reference (golden cache files,
interpolations) and the oracle.

Tolerances: FP64 form 1e-10 relative per node with a 1 K floor
(|dE| <= 1e-10 * max(1 K, |E|)). FP32 form 1e-5 relative with a kT floor,
|dE| <= 1e-5 * max(kT, |E|) with kT = 298 K (the workload temperature): an
FP32 term carries ~1e-6 relative rounding, so a node whose large repulsive and
attractive terms cancel keeps ~1e-2 K of absolute error, negligible against the
Boltzmann scale kT; checked on nodes below 1e4 K (deeper in the repulsive core
the FP32 terms are clamped and such nodes end at the 1e5 K cap in both forms).
Interpolation on identical tables is bit-exact."""
import os
import tempfile
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from conftest import golden, rel_err
from test_oracle_golden import _cache_tables

KT = 298.0

pytestmark = pytest.mark.gpu


def _gc():
    return golden("grid_cubic")


def _build(A, g, spacing, precision, cutoff=None, guests=None):
    ff = A.LennardJones(g["eps"], g["sigma"], float(g["cutoff"]) if cutoff is None else cutoff,
                        A.SHIFTED)
    p = A.ParticleData(g["x"], g["y"], g["z"], g["charge"], g["species"])
    gg = [int(v) for v in g["guests"]] if guests is None else guests
    return A.FrameworkEnergyGrid(ff, p, g["lattice"], gg, spacing, precision), ff, p


def test_fp64_grid_matches_reference_tables(lib):
    A, _ = lib
    g = _gc()
    grid, ff, p = _build(A, g, float(g["spacing"]), A.FP64)
    counts, tables = _cache_tables(g["cache_file"])
    assert grid.point_counts() == counts
    assert grid.species() == sorted(tables)
    for sid, ref_table in tables.items():
        assert rel_err(grid.table(sid), ref_table).max() <= 1e-10


def test_fp32_grid_within_1e5(lib):
    A, _ = lib
    g = _gc()
    grid, ff, p = _build(A, g, float(g["spacing"]), A.FP32)
    counts, tables = _cache_tables(g["cache_file"])
    for sid, ref_table in tables.items():
        mine = grid.table(sid)
        keep = ref_table <= 1e4
        assert keep.sum() > 500
        assert rel_err(mine[keep], ref_table[keep], floor=KT).max() <= 1e-5
        assert (mine[ref_table >= 1e5] >= 1e4).all()


def test_interpolation_bit_exact(lib):
    A, _ = lib
    g = _gc()
    grid, ff, p = _build(A, g, float(g["spacing"]), A.FP64)
    counts, tables = _cache_tables(g["cache_file"])
    # identical tables -> identical interpolation: load the reference's file
    with tempfile.TemporaryDirectory() as td:
        (Path(td) / str(g["cache_name"])).write_bytes(g["cache_file"].tobytes())
        loaded = A.FrameworkEnergyGrid.load_from_cache(td, ff, p, g["lattice"],
                                                       [int(v) for v in g["guests"]],
                                                       float(g["spacing"]))
    assert loaded is not None
    for i, sid in enumerate(g["guests"]):
        assert np.array_equal(loaded.interpolate(int(sid), g["points"]), g["interp"][i])
        # and the GPU-built tables interpolate to within the FP64 tolerance
        assert rel_err(grid.interpolate(int(sid), g["points"]), g["interp"][i]).max() <= 1e-10
    with pytest.raises(IndexError):
        grid.interpolate(0, g["points"][:4])


def test_fp32_form_interpolation_vs_oracle(lib, orc):
    """Grids built in the FP32 form interpolate in double-float on the FP32
    pipe (position and corners split into hi + lo by integer operations,
    ~48 bits): within 1e-9 x max(kT, |E|) of the oracle's reference-order
    interpolation of the same table, for points within a few cells of the
    origin, on nodes, on cell faces and at zero. The kT floor is the FP32
    form's; the worst case is a cell whose corners span the 1e5 K cap, where
    ~1e-14 of position rounding and 48-bit lerps leave ~3e-8 K. Far images
    (1e6 A: any form carries ~1e-10 A of rounding there, 1e-4 K on a steep
    wall) within 1e-6 x max(kT, |E|); operands outside the split's range
    (1e-30 A, 2e30 A, 3e8 A) are answered in FP64."""
    A, _ = lib
    from aleator_gb300 import workloads as W
    fw = W.triclinic_supercell(reps=1)
    ff = A.LennardJones(fw.eps, fw.sigma, 10.0, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    sid = fw.guest_species["CH4"]
    g32 = A.FrameworkEnergyGrid(ff, p, fw.lattice, [sid], 0.7, A.FP32)
    m = np.asarray(fw.lattice).reshape(3, 3)
    rng = np.random.default_rng(3)
    f = np.concatenate([rng.uniform(-1.5, 2.5, (4000, 3)),
                        np.floor(rng.uniform(0, 8, (200, 3))) / np.array(g32.point_counts())])
    near = np.concatenate([f @ m, [[0.0, 0.0, 0.0], [-0.0, 1e-30, 0.0], [1e-30, 5.0, -7.0],
                                   [2e30, 1.0, 2.0], [-3e8, 2.0, 2.0]]])
    far = np.array([[1e6, -1e6, 3.5e5], [1e6, 0.5, 0.25], [-7e5, 3e5, 1e6]]) + near[:3]
    for xyz, tol in ((near, 1e-9), (far, 1e-6)):
        ref = orc.grid_interpolate(m, g32.point_counts(), g32.table(sid), xyz)
        got = g32.interpolate(sid, xyz)
        assert np.isfinite(got).all()
        assert rel_err(got, ref, floor=KT).max() <= tol


def test_cache_file_byte_identical_and_guards(lib):
    """framework_energy_grid.cc:290-409 and test_framework_energy_grid_cache.cc:
    the written file equals the reference's bytes (tables from the reference's
    own file, so the comparison is of the format), names match, and a foreign
    file at the hashed path is a hard error."""
    A, _ = lib
    g = _gc()
    ff = A.LennardJones(g["eps"], g["sigma"], float(g["cutoff"]), A.SHIFTED)
    p = A.ParticleData(g["x"], g["y"], g["z"], g["charge"], g["species"])
    guests = [int(v) for v in g["guests"]]
    name = A.FrameworkEnergyGrid.cache_file_name(ff, p, g["lattice"], guests, float(g["spacing"]))
    assert name == str(g["cache_name"])
    with tempfile.TemporaryDirectory() as td:
        (Path(td) / name).write_bytes(g["cache_file"].tobytes())
        loaded = A.FrameworkEnergyGrid.load_from_cache(td, ff, p, g["lattice"], guests,
                                                       float(g["spacing"]))
        out = Path(td) / "again.bin"
        loaded.serialize(out)
        assert out.read_bytes() == g["cache_file"].tobytes()
        # miss -> None
        assert A.FrameworkEnergyGrid.load_from_cache(td, ff, p, g["lattice"], guests, 1.0) is None
        # version mismatch -> hard error
        bad = bytearray(g["cache_file"].tobytes())
        bad[0] = 2
        (Path(td) / name).write_bytes(bytes(bad))
        with pytest.raises(RuntimeError, match="format version"):
            A.FrameworkEnergyGrid.load_from_cache(td, ff, p, g["lattice"], guests, float(g["spacing"]))
        # truncated -> hard error
        (Path(td) / name).write_bytes(g["cache_file"].tobytes()[:5000])
        with pytest.raises(RuntimeError, match="truncated or corrupt"):
            A.FrameworkEnergyGrid.load_from_cache(td, ff, p, g["lattice"], guests, float(g["spacing"]))
        # GPU-built grid round-trips bit-identically through its own file
        grid, _, _ = _build(A, g, float(g["spacing"]), A.FP64)
        grid.serialize(Path(td) / name)
        back = A.FrameworkEnergyGrid.load_from_cache(td, ff, p, g["lattice"], guests, float(g["spacing"]))
        for sid in guests:
            assert np.array_equal(back.table(sid), grid.table(sid))


def test_triclinic_fp64(lib):
    A, _ = lib
    t = golden("triclinic")
    counts, tables = _cache_tables(t["cache_file"])
    sid = list(tables)[0]
    ff = A.LennardJones(t["eps"], t["sigma"], 10.0, A.SHIFTED)
    p = A.ParticleData(t["x"], t["y"], t["z"], t["charge"], t["species"])
    grid = A.FrameworkEnergyGrid(ff, p, t["lattice"], [sid], 1.0, A.FP64)
    assert grid.point_counts() == counts
    assert rel_err(grid.table(sid), tables[sid]).max() <= 1e-10
    g32 = A.FrameworkEnergyGrid(ff, p, t["lattice"], [sid], 1.0, A.FP32)
    keep = tables[sid] <= 1e4
    assert rel_err(g32.table(sid)[keep], tables[sid][keep], floor=KT).max() <= 1e-5


@pytest.mark.parametrize("trunc", [0, 2])
def test_truncations_vs_oracle(lib, orc, trunc):
    A, _ = lib
    from aleator_gb300 import workloads as W
    fw = W.cubic_framework(seed=7)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.0, trunc)
    p = A.ParticleData.from_framework(fw)
    grid = A.FrameworkEnergyGrid(ff, p, fw.lattice, [4, 6], 1.7, A.FP64)
    for sid in (4, 6):
        ref = orc.grid_build(dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.0, truncation=trunc),
                             fw.lattice, fw.x, fw.y, fw.z, fw.species, sid, 1.7, threads=8)
        assert rel_err(grid.table(sid), ref).max() <= 1e-10


@pytest.mark.parametrize("trunc", [0, 1, 2])
def test_fp32_truncations_vs_oracle(lib, orc, trunc):
    """The FP32 sweep in every truncation, two guests, at a coarse spacing
    (every node) and a fine one (a strided sample): the atoms of a warp's
    tile take the clamp-free, cutoff-clamped and close-pair paths."""
    A, _ = lib
    from aleator_gb300 import workloads as W
    fw = W.cubic_framework(seed=7)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.0, trunc)
    p = A.ParticleData.from_framework(fw)
    odict = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.0, truncation=trunc)
    for spacing, stride in ((1.7, 1), (0.45, 131)):
        grid = A.FrameworkEnergyGrid(ff, p, fw.lattice, [4, 6], spacing, A.FP32)
        nodes = int(np.prod(grid.point_counts()))
        idx = np.arange(0, nodes, stride)
        for sid in (4, 6):
            if stride == 1:
                ref = orc.grid_build(odict, fw.lattice, fw.x, fw.y, fw.z, fw.species, sid, spacing,
                                     threads=8)
            else:
                ref = np.concatenate([orc.grid_build(odict, fw.lattice, fw.x, fw.y, fw.z, fw.species,
                                                     sid, spacing, node_begin=int(i),
                                                     node_end=int(i) + 1) for i in idx])
            mine = grid.table(sid)[idx]
            keep = ref <= 1e4
            assert keep.sum() > 100
            assert rel_err(mine[keep], ref[keep], floor=KT).max() <= 1e-5
            assert (mine[ref >= 1e5] >= 1e4).all()


@pytest.mark.parametrize("trunc", [0, 1, 2])
def test_fp32_every_node_vs_fp64(lib, trunc):
    """Every node of a fine grid (0.3 Å, 636k nodes, the CO2 site guests) in
    FP32 against the FP64 form (itself within 1e-10 of the oracle): the nodes
    whose close pairs take the double-float correction are among them."""
    A, _ = lib
    from aleator_gb300 import workloads as W
    fw = W.cubic_framework(seed=13)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, trunc)
    p = A.ParticleData.from_framework(fw)
    guests = [fw.guest_species["CO2_C"], fw.guest_species["CO2_O"]]
    g64 = A.FrameworkEnergyGrid(ff, p, fw.lattice, guests, 0.3, A.FP64)
    g32 = A.FrameworkEnergyGrid(ff, p, fw.lattice, guests, 0.3, A.FP32)
    for sid in guests:
        t64, t32 = g64.table(sid), g32.table(sid)
        keep = t64 <= 1e4
        assert keep.sum() > 100000
        assert rel_err(t32[keep], t64[keep], floor=KT).max() <= 1e-5
        assert (t32[t64 >= 1e5] >= 1e4).all()


def test_full_c1_grid_vs_oracle_sample(lib, orc):
    """The 52^3 grid of the 424-atom cell at 0.5 Å: every node in FP64 and FP32
    against the oracle on a strided sample of nodes."""
    A, _ = lib
    from aleator_gb300 import workloads as W
    fw = W.cubic_framework()
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    g64 = A.FrameworkEnergyGrid(ff, p, fw.lattice, [4], 0.5, A.FP64)
    g32 = A.FrameworkEnergyGrid(ff, p, fw.lattice, [4], 0.5, A.FP32)
    assert g64.point_counts() == (52, 52, 52)
    t64, t32 = g64.table(4), g32.table(4)
    st = g64.stats()
    assert st["algorithmic_pairs"] == 52 ** 3 * 424
    odict = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    idx = np.arange(0, 52 ** 3, 97)
    ref = np.concatenate([orc.grid_build(odict, fw.lattice, fw.x, fw.y, fw.z, fw.species, 4, 0.5,
                                         node_begin=int(i), node_end=int(i) + 1) for i in idx])
    assert rel_err(t64[idx], ref).max() <= 1e-10
    keep = ref <= 1e4
    assert rel_err(t32[idx][keep], ref[keep], floor=KT).max() <= 1e-5


def test_supercell_invariance_at_scale(lib):
    """Size-independent property (test_supercell_energy_invariance.cc): the grid
    of a 2x2x2 supercell with node spacing L/n equals the base cell's grid tiled,
    node for node."""
    A, _ = lib
    from aleator_gb300 import workloads as W
    base = W.cubic_framework(seed=3)
    sup = W.replicate(base, (2, 2, 2))
    ff = A.LennardJones(base.eps, base.sigma, 12.8, A.SHIFTED)
    n = 40
    spacing = 25.832 / n
    gb = A.FrameworkEnergyGrid(ff, A.ParticleData.from_framework(base), base.lattice, [5], spacing, A.FP64)
    gs = A.FrameworkEnergyGrid(ff, A.ParticleData.from_framework(sup), sup.lattice, [5], spacing, A.FP64)
    assert gs.point_counts() == (2 * n, 2 * n, 2 * n)
    tb = gb.table(5).reshape(n, n, n)
    ts = gs.table(5).reshape(2 * n, 2 * n, 2 * n)
    tiled = np.tile(tb, (2, 2, 2))
    assert rel_err(ts, tiled).max() <= 1e-10
    for prec in (A.FP32,):
        g32 = A.FrameworkEnergyGrid(ff, A.ParticleData.from_framework(sup), sup.lattice, [5], spacing, prec)
        t32 = g32.table(5)
        keep = tiled.reshape(-1) <= 1e4
        assert rel_err(t32[keep], tiled.reshape(-1)[keep], floor=KT).max() <= 1e-5


def test_edge_cases(lib):
    A, _ = lib
    from aleator_gb300 import workloads as W
    fw = W.cubic_framework(seed=5)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.0, A.SHIFTED)
    # empty framework: every node is 0
    empty = A.ParticleData(np.zeros(0), np.zeros(0), np.zeros(0))
    g = A.FrameworkEnergyGrid(ff, empty, fw.lattice, [4], 3.0)
    assert (g.table(4) == 0).all()
    # one atom, grid coarser than one node per axis is clamped to 1
    one = A.ParticleData([1.0], [2.0], [3.0], None, [0])
    g1 = A.FrameworkEnergyGrid(ff, one, fw.lattice, [4, 4, 4], 100.0)
    assert g1.point_counts() == (1, 1, 1) and g1.species() == [4]
    d = np.sqrt(1 + 4 + 9)
    eps, sig = np.sqrt(fw.eps[4] * fw.eps[0]), 0.5 * (fw.sigma[4] + fw.sigma[0])
    raw = lambda r: 4 * eps * ((sig / r) ** 12 - (sig / r) ** 6)
    assert abs(g1.table(4)[0] - min(raw(d) - raw(12.0), 1e5)) <= 1e-10 * max(1, abs(raw(d)))


def test_grid_from_cif_structure(lib, orc):
    """A framework read from a CIF file (triclinic cell, symmetry-expanded),
    replicated until the cutoff fits, through the FP64 energy grid: within
    1e-10 of the oracle's grid on the same particles."""
    A, _ = lib
    from pathlib import Path
    from aleator_gb300 import workloads as W
    s = A.read_cif(Path(__file__).resolve().parent / "golden" / "cif" / "triclinic_symops.cif")
    ns = len(s.species_symbols)
    rng = np.random.default_rng(4)
    eps = np.concatenate([rng.uniform(20, 100, ns), [148.0]])   # framework types, then the probe
    sigma = np.concatenate([rng.uniform(2.5, 3.5, ns), [3.73]])
    # shifted off the nodes: the atoms on special positions (the origin among
    # them) would otherwise sit exactly on grid nodes, where r = 0
    fw = W.Framework(lattice=np.asarray(s.lattice), x=s.particles.x + 0.0123,
                     y=s.particles.y + 0.0456, z=s.particles.z + 0.0789,
                     species=s.particles.species, charge=s.particles.charge, eps=eps, sigma=sigma)
    fw = W.replicate(fw, W.minimum_replication(fw.lattice, 9.0))
    ff = A.LennardJones(fw.eps, fw.sigma, 9.0, A.SHIFTED)
    grid = A.FrameworkEnergyGrid(ff, A.ParticleData.from_framework(fw), fw.lattice, [ns], 1.0, A.FP64)
    od = dict(eps=fw.eps, sigma=fw.sigma, cutoff=9.0, truncation=O.SHIFTED)
    want = orc.grid_build(od, fw.lattice, fw.x, fw.y, fw.z, fw.species, ns, 1.0, threads=8)
    assert rel_err(grid.table(ns), want).max() <= 1e-10


def test_build_to_host_equals_build(lib):
    """alea_grid_build_to_host (slab-pipelined build with the copies overlapped)
    hands back exactly the tables of a plain build, both forms, a species listed
    twice included."""
    A, _ = lib
    import torch
    from aleator_gb300 import workloads as W
    fw = W.triclinic_supercell(reps=1)
    ff = A.LennardJones(fw.eps, fw.sigma, 10.0, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    guests = [fw.guest_species["CO2_O"], fw.guest_species["CO2_C"], fw.guest_species["CO2_O"]]
    for prec in (A.FP64, A.FP32):
        ref = A.FrameworkEnergyGrid(ff, p, fw.lattice, guests, 0.4, prec)
        nodes = int(np.prod(ref.point_counts()))
        outs = [torch.full((nodes,), np.nan, dtype=torch.float64, pin_memory=True) for _ in guests]
        g = A.FrameworkEnergyGrid.build_to_host(ff, p, fw.lattice, guests, 0.4, prec,
                                                [o.data_ptr() for o in outs])
        for s, o in zip(guests, outs):
            assert np.array_equal(o.numpy(), ref.table(s))
            assert np.array_equal(g.table(s), ref.table(s))
        plain = np.full(nodes, np.nan)  # pageable memory and no grid kept
        assert A.FrameworkEnergyGrid.build_to_host(ff, p, fw.lattice, guests[:1], 0.4, prec,
                                                   [plain.ctypes.data], keep=False) is None
        assert np.array_equal(plain, ref.table(guests[0]))


def test_bounded_tile_wait_gives_up_and_recovers(lib):
    """The FP64 build's tile waits (TMA copies on an mbarrier) are bounded:
    with the test knob the next build's waits give up at the first poll (no
    fault, no hang: each CTA still waits, bounded, for the copies it has in
    flight, then returns). The build reports ALEA_ERR_DEVICE_CHECK ("wait"),
    the knob is spent, and the next build on the same context returns the
    normal tables. An FP32 build is not affected by the knob."""
    A, _ = lib
    from aleator_gb300 import workloads as W
    fw = W.cubic_framework(seed=5)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.0, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    grid = A.FrameworkEnergyGrid(ff, p, fw.lattice, [4, 6], 0.8, A.FP64)
    want = {s: grid.table(s) for s in (4, 6)}
    lib_ = A.load_library()
    assert lib_.alea_test_grid_tile_wait_limit(0) == 0
    with pytest.raises(A.AleatorError) as e:
        grid.rebuild()
    assert e.value.status == 6 and "wait" in str(e.value)
    grid.rebuild()  # the knob was consumed by the failed build
    for s in (4, 6):
        assert np.array_equal(grid.table(s), want[s])
    again = A.FrameworkEnergyGrid(ff, p, fw.lattice, [4, 6], 0.8, A.FP64)
    for s in (4, 6):
        assert np.array_equal(again.table(s), want[s])
    # the FP32 build leaves a pending knob alone; the next FP64 build takes it
    f32 = A.FrameworkEnergyGrid(ff, p, fw.lattice, [4, 6], 0.8, A.FP32)
    assert lib_.alea_test_grid_tile_wait_limit(0) == 0
    f32.rebuild()
    with pytest.raises(A.AleatorError):
        grid.rebuild()
    grid.rebuild()


@pytest.mark.parametrize("cell", ["cubic", "triclinic"])
def test_cutoff_beyond_half_width_is_the_reference_minimum_image(lib, orc, cell):
    """rc > L_perp/2, which the reference's grid constructor accepts: one
    minimum image per atom (lattice.cc:185-255), as the oracle computes it,
    within 1e-10 (1 K floor); a request for the FP32 form gets the same FP64
    tables."""
    A, _ = lib
    from aleator_gb300 import workloads as W
    if cell == "cubic":
        fw, rc = W.cubic_framework(seed=99, charged=True), 13.5
    else:
        fw, rc = W.triclinic_supercell(reps=1, seed=31), 11.5
    ff = A.LennardJones(fw.eps, fw.sigma, rc, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    sid = fw.guest_species["CH4"]
    od = dict(eps=fw.eps, sigma=fw.sigma, cutoff=rc, truncation=O.SHIFTED)
    want = orc.grid_build(od, fw.lattice, fw.x, fw.y, fw.z, fw.species, sid, 1.0, threads=8)
    for prec in (A.FP64, A.FP32):
        g = A.FrameworkEnergyGrid(ff, p, fw.lattice, [sid], 1.0, prec)
        assert rel_err(g.table(sid), want).max() <= 1e-10
