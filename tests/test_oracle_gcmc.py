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


@pytest.mark.parametrize("charged", [False, True])
def test_chain_with_energy_grid_bit_identical_to_reference(orc, ref, charged):
    """The engine with its shared FrameworkEnergyGrid (monte_carlo_engine.cc:353-372):
    a site's dispersion is the grid's interpolation plus the guests' LJ. The
    oracle is given the oracle's own grid tables (bit-identical to the
    reference's, test_oracle_vs_reference.py)."""
    fw = W.cubic_framework(seed=21, charged=charged)
    if charged:
        fw.charge = fw.charge * 0.15
    ff = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    ew = dict(alpha=0.31, rc=12.0, kmax=5) if charged else None
    guest = W.co2_guest(fw) if charged else W.ch4_guest(fw)
    fug = ref.pr_fugacity(*(W.CO2_CRITICAL if charged else W.METHANE_CRITICAL), 298.0, 1e6)
    species = sorted(set(int(s) for s in guest["lj_species"]))
    spacing = 0.5
    tables = {s: orc.grid_build(ff, fw.lattice, fw.x, fw.y, fw.z, fw.species, s, spacing, threads=8)
              for s in species}
    counts = orc.grid_point_counts(fw.lattice, spacing)
    a = ref.gcmc(ff, ew, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guest, 298.0, fug, 9, 4,
                 grid={"spacing": spacing, "species": species})
    b = orc.gcmc(ff, ew, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guest, 298.0, fug, 9, 4,
                 grid={"counts": counts, "tables": tables})
    for _ in range(4):
        a.run(300)
        b.run(300)
        assert a.molecules() == b.molecules()
        assert np.array_equal(a.positions(), b.positions())
        assert a.ewald_energy() == b.ewald_energy()
    assert a.molecules() > 0


@pytest.mark.parametrize("charged", [False, True])
def test_mixture_chain_bit_identical_to_reference(orc, ref, charged):
    """The mixture constructor (monte_carlo_engine.hpp:143-151): CH4 and CO2,
    20 % each of translate, rotate, insert, delete and identity swap
    (monte_carlo_engine.cc:405-439, 673-792); bit-identical trajectories,
    per-species counts and Ewald cache energies."""
    fw = W.cubic_framework(seed=21, charged=charged)
    if charged:
        fw.charge = fw.charge * 0.15
    ff = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    ew = dict(alpha=0.31, rc=12.0, kmax=5) if charged else None
    ch4 = W.ch4_guest(fw)
    ch4 = dict(ch4, charge=[0.0])
    guests = [W.co2_guest(fw), ch4] if charged else [ch4, dict(W.co2_guest(fw), charge=[0.0] * 3)]
    fugs = [ref.pr_fugacity(*W.CO2_CRITICAL, 298.0, 5e5), ref.pr_fugacity(*W.METHANE_CRITICAL, 298.0, 2e6)]
    if not charged:
        fugs = fugs[::-1]
    a = ref.gcmc_mixture(ff, ew, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guests, 298.0,
                         fugs, 9, 4)
    b = orc.gcmc_mixture(ff, ew, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guests, 298.0,
                         fugs, 9, 4)
    for _ in range(5):
        a.run(400)
        b.run(400)
        assert a.molecules() == b.molecules()
        assert [a.molecules_of(k) for k in range(2)] == [b.molecules_of(k) for k in range(2)]
        assert np.array_equal(a.positions(), b.positions())
        assert a.ewald_energy() == b.ewald_energy()
    ctr = b.counters()
    assert ctr[9] > 0, ctr  # swaps accepted
    assert min(a.molecules_of(k) for k in range(2)) > 0


def test_peng_robinson_mixture_errors_match_reference(ref):
    """The library's argument errors carry the reference's own exception text."""
    import aleator_gb300 as A
    from aleator_gb300.build import LIB, build

    if not LIB.exists():
        build()
    ch4 = W.METHANE_CRITICAL
    cases = [
        ([ch4, (0.0, 1e6, 0.0)], 298.0, 1e5, [0.5, 0.5], None),
        ([ch4, ch4], 298.0, 1e5, [0.5, 0.5], [[0.1, 0.0], [0.0, 0.0]]),
        ([ch4, ch4], 298.0, 1e5, [0.5, 0.5], [[0.0, 0.1], [0.2, 0.0]]),
        ([ch4, ch4], 298.0, 1e5, [1.2, -0.2], None),
        ([ch4, ch4], 298.0, 1e5, [0.5, 0.6], None),
        ([ch4, ch4], -1.0, 1e5, [0.5, 0.5], None),
        ([ch4, ch4], 298.0, 0.0, [0.5, 0.5], None),
    ]
    for args in cases:
        with pytest.raises(ValueError) as mine:
            A.peng_robinson_mixture(*args)
        with pytest.raises(ValueError) as theirs:
            ref.pr_mixture(*args)
        assert str(mine.value) == str(theirs.value)


def test_mixture_with_grid_bit_identical_to_reference(ref, orc):
    """Mixture (charged CO2 + CH4, identity swaps) with the engine's energy grid:
    the oracle (tables from its own grid restatement) against the reference
    engine with the FrameworkEnergyGrid it builds itself: identical positions,
    per-species counts and Ewald energy."""
    fw = W.cubic_framework(seed=23, charged=True)
    fw.charge = fw.charge * 0.15
    ff = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    ew = dict(alpha=0.31, rc=12.0, kmax=5)
    guests = [W.co2_guest(fw), W.ch4_guest(fw)]
    species = sorted({int(s) for g in guests for s in g["lj_species"]})
    spacing = 0.5
    tables = {s: orc.grid_build(ff, fw.lattice, fw.x, fw.y, fw.z, fw.species, s, spacing, threads=8)
              for s in species}
    counts = orc.grid_point_counts(fw.lattice, spacing)
    fugs = [ref.pr_fugacity(*W.CO2_CRITICAL, 298.0, 5e5), ref.pr_fugacity(*W.METHANE_CRITICAL, 298.0, 2e6)]
    a = ref.gcmc_mixture(ff, ew, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guests, 298.0,
                         fugs, 13, 2, grid={"spacing": spacing, "species": species})
    b = orc.gcmc_mixture(ff, ew, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guests, 298.0,
                         fugs, 13, 2, grid={"counts": counts, "tables": tables})
    for _ in range(4):
        a.run(300)
        b.run(300)
        assert a.molecules() == b.molecules()
        assert [a.molecules_of(k) for k in range(2)] == [b.molecules_of(k) for k in range(2)]
        assert np.array_equal(a.positions(), b.positions())
        assert a.ewald_energy() == b.ewald_energy()
    assert a.molecules() > 0


def test_peng_robinson_mixture_fuzzed_against_reference(ref):
    """Random substances (2-4), compositions, temperatures, pressures and k_ij:
    the library's Z and partial fugacities equal the reference's bit for bit,
    or both reject the input with the same message."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies
    import aleator_gb300 as A
    from aleator_gb300.build import LIB, build

    if not LIB.exists():
        build()
    sub = st.tuples(st.floats(80.0, 700.0), st.floats(1e6, 8e6), st.floats(-0.2, 0.6))

    @hyp.settings(max_examples=200, deadline=None, database=None, derandomize=True)
    @hyp.given(subs=st.lists(sub, min_size=2, max_size=4), t=st.floats(150.0, 600.0),
               p=st.sampled_from([1.0, 1e3, 1e5, 1e6, 5e6, 2e7]),
               w=st.lists(st.floats(0.0, 1.0), min_size=4, max_size=4), k=st.floats(-0.1, 0.2),
               use_k=st.booleans())
    def check(subs, t, p, w, k, use_k):
        n = len(subs)
        tot = sum(w[:n]) or 1.0
        x = [v / tot for v in w[:n]]
        kij = None
        if use_k:
            kij = [[0.0 if i == j else k for j in range(n)] for i in range(n)]
        try:
            zr, fr = ref.pr_mixture(subs, t, p, x, kij)
            rerr = None
        except ValueError as e:
            rerr = str(e)
        try:
            zs, fs = A.peng_robinson_mixture(subs, t, p, x, kij)
            serr = None
        except (ValueError, RuntimeError) as e:
            serr = str(e)
        assert rerr == serr, (subs, t, p, x, kij, rerr, serr)
        if rerr is None:
            assert zs == zr and np.array_equal(fs, fr)

    check()


def test_gcmc_oracle_fuzzed_against_reference(ref, orc):
    """Random engines: seed and stream, pressure, CH4 / CO2 / their mixture,
    charged or not, with or without the energy grid. The oracle's trajectory is
    the reference engine's, bit for bit (positions, counts, Ewald energy)."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies
    fw = W.cubic_framework(seed=31, charged=True)
    fw.charge = fw.charge * 0.15
    ff = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    ew = dict(alpha=0.31, rc=12.0, kmax=4)
    spacing = 1.0
    all_species = sorted({int(s) for g in (W.co2_guest(fw), W.ch4_guest(fw)) for s in g["lj_species"]})
    tables = {s: orc.grid_build(ff, fw.lattice, fw.x, fw.y, fw.z, fw.species, s, spacing, threads=8)
              for s in all_species}
    counts = orc.grid_point_counts(fw.lattice, spacing)

    @hyp.settings(max_examples=12, deadline=None, database=None, derandomize=True)
    @hyp.given(seed=st.integers(0, 2 ** 40), stream=st.integers(0, 1000),
               bar=st.sampled_from([0.5, 5.0, 30.0]), kind=st.sampled_from(["ch4", "co2", "mix"]),
               charged=st.booleans(), grid=st.booleans())
    def check(seed, stream, bar, kind, charged, grid):
        co2 = W.co2_guest(fw) if charged else dict(W.co2_guest(fw), charge=[0.0, 0.0, 0.0])
        guests = {"ch4": [W.ch4_guest(fw)], "co2": [co2], "mix": [co2, W.ch4_guest(fw)]}[kind]
        crit = {"ch4": [W.METHANE_CRITICAL], "co2": [W.CO2_CRITICAL],
                "mix": [W.CO2_CRITICAL, W.METHANE_CRITICAL]}[kind]
        fugs = [ref.pr_fugacity(*c, 298.0, bar * 1e5) for c in crit]
        ewd = ew if charged else None
        species = sorted({int(s) for g in guests for s in g["lj_species"]})
        rg = {"spacing": spacing, "species": species} if grid else None
        og = {"counts": counts, "tables": {s: tables[s] for s in species}} if grid else None
        if kind == "mix":
            a = ref.gcmc_mixture(ff, ewd, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guests,
                                 298.0, fugs, seed, stream, grid=rg)
            b = orc.gcmc_mixture(ff, ewd, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guests,
                                 298.0, fugs, seed, stream, grid=og)
        else:
            a = ref.gcmc(ff, ewd, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guests[0], 298.0,
                         fugs[0], seed, stream, grid=rg)
            b = orc.gcmc(ff, ewd, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guests[0], 298.0,
                         fugs[0], seed, stream, grid=og)
        for _ in range(2):
            a.run(250)
            b.run(250)
            assert a.molecules() == b.molecules()
            assert np.array_equal(a.positions(), b.positions())
            assert a.ewald_energy() == b.ewald_energy()
        if kind == "mix":
            assert [a.molecules_of(k) for k in range(2)] == [b.molecules_of(k) for k in range(2)]

    check()


def test_widom_oracle_fuzzed_against_reference(ref, orc):
    """Random Widom runs (seed, stream, CH4 or CO2, charged or not, cubic or
    triclinic cell, every truncation): the oracle's per-trial energies and K_H
    equal the reference engine's."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies
    cells = {"cubic": W.cubic_framework(seed=41, charged=True),
             "triclinic": W.triclinic_supercell(reps=1)}

    @hyp.settings(max_examples=12, deadline=None, database=None, derandomize=True)
    @hyp.given(seed=st.integers(0, 2 ** 40), stream=st.integers(0, 1000),
               co2=st.booleans(), charged=st.booleans(), cell=st.sampled_from(["cubic", "triclinic"]),
               trunc=st.sampled_from([O.TRUNCATED, O.SHIFTED, O.LINEAR_FORCE_SHIFTED]))
    def check(seed, stream, co2, charged, cell, trunc):
        fw = cells[cell]
        rc = 12.8 if cell == "cubic" else 10.0
        ff = dict(eps=fw.eps, sigma=fw.sigma, cutoff=rc, truncation=trunc)
        ew = dict(alpha=0.33, rc=min(rc, 10.0), kmax=4) if charged else None
        guest = W.co2_guest(fw) if co2 else W.ch4_guest(fw)
        q = fw.charge if charged else None
        kr, pr = ref.widom(ff, ew, fw.lattice, fw.x, fw.y, fw.z, q, fw.species, guest, 298.0, seed,
                           stream, 150, per_trial=True)
        ko, po = orc.widom(ff, ew, fw.lattice, fw.x, fw.y, fw.z, q, fw.species, guest, 298.0, seed,
                           stream, 150, per_trial=True)
        assert np.array_equal(pr, po)
        assert kr[0] == ko

    check()


def test_grid_oracle_fuzzed_against_reference(ref, orc, tmp_path):
    """Random triclinic frameworks (50-300 atoms, replicated to fit the cutoff),
    spacings and truncations: the oracle's grid tables equal the reference's
    FrameworkEnergyGrid (read back from its own cache file) node for node."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies
    from test_oracle_golden import _cache_tables

    @hyp.settings(max_examples=6, deadline=None, database=None, derandomize=True)
    @hyp.given(seed=st.integers(1, 10 ** 6), spacing=st.sampled_from([1.7, 2.3, 3.1]),
               trunc=st.sampled_from([O.TRUNCATED, O.SHIFTED, O.LINEAR_FORCE_SHIFTED]))
    def check(seed, spacing, trunc):
        fw = W.random_triclinic_frameworks(1, seed=seed, cutoff=9.0, max_atoms=300)[0]
        ff = dict(eps=fw.eps, sigma=fw.sigma, cutoff=9.0, truncation=trunc)
        guest = fw.guest_species["CH4"]
        g = ref.grid(ff, fw.lattice, fw.x, fw.y, fw.z, fw.species, [guest], spacing)
        f = tmp_path / f"g{seed}.bin"
        g.serialize(f)
        _, tables = _cache_tables(np.frombuffer(f.read_bytes(), np.uint8))
        mine = orc.grid_build(ff, fw.lattice, fw.x, fw.y, fw.z, fw.species, guest, spacing, threads=8)
        assert np.array_equal(mine, tables[guest])

    check()


def test_ewald_state_fuzzed_against_reference(ref, orc):
    """Random propose/commit sequences on the EwaldIncrementalState (insertions,
    deletions and moves of 1- to 3-site molecules at random charges, proposals
    left uncommitted, cubic or triclinic cell, random alpha and kMax): the
    oracle's deltas, energies and raw S(k) equal the reference's."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies
    cells = {"cubic": W.cubic_framework(seed=51, charged=True), "triclinic": W.triclinic_supercell(reps=1)}

    @hyp.settings(max_examples=10, deadline=None, database=None, derandomize=True)
    @hyp.given(seed=st.integers(0, 2 ** 31), cell=st.sampled_from(["cubic", "triclinic"]),
               alpha=st.sampled_from([0.22, 0.3, 0.41]), kmax=st.integers(2, 6))
    def check(seed, cell, alpha, kmax):
        fw = cells[cell]
        a = ref.ewald_state(fw.lattice, fw.x, fw.y, fw.z, fw.charge, alpha, kmax)
        b = orc.ewald_state(fw.lattice, fw.x, fw.y, fw.z, fw.charge, alpha, kmax)
        rng = np.random.default_rng(seed)
        span = float(np.abs(np.asarray(fw.lattice)).sum(axis=0).max())
        mols = []
        for _ in range(40):
            ns = int(rng.integers(1, 4))
            q = rng.uniform(-1, 1, ns)
            q -= q.mean()
            new = np.column_stack([rng.uniform(-0.2 * span, 1.2 * span, (ns, 3)), q])
            pick = rng.uniform()
            if mols and pick < 0.35:
                rem, add = mols[-1], np.zeros((0, 4))
            elif mols and pick < 0.6:
                rem = mols[-1]
                add = rem.copy()
                add[:, :3] += rng.uniform(-2, 2, 3)
            else:
                rem, add = np.zeros((0, 4)), new
            assert a.propose(rem, add) == b.propose(rem, add)
            if rng.uniform() < 0.7:
                a.commit(rem, add)
                b.commit(rem, add)
                if len(rem) and len(add):
                    mols[-1] = add
                elif len(rem):
                    mols.pop()
                else:
                    mols.append(add)
            assert a.energy() == b.energy()
        assert np.array_equal(a.raw(), b.raw())

    check()


def test_philox_fuzzed_against_reference(ref, orc):
    """Philox4x32-10 streams for arbitrary 64-bit seeds and streams and call
    offsets up to 1e5 (the reference's generator reaches an offset by drawing;
    the 2^32 word boundary of the call counter is pinned by the golden
    fixture): the oracle's u64 and uniform draws equal the reference's."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies
    u64 = st.integers(0, 2 ** 64 - 1)

    @hyp.settings(max_examples=40, deadline=None, database=None, derandomize=True)
    @hyp.given(seed=u64, stream=u64, first=st.integers(0, 100_000))
    def check(seed, stream, first):
        assert np.array_equal(orc.philox_u64(seed, stream, first, 64),
                              ref.philox_u64(seed, stream, first, 64))
        assert np.array_equal(orc.philox_uniform(seed, stream, first, 64),
                              ref.philox_uniform(seed, stream, first, 64))

    check()
