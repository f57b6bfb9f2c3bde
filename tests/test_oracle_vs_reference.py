"""The C restatement against the reference's own code (oracle/_ref) on fresh
random inputs: bit-exact where the operation sequence is the same. Skipped
where the reference tree was not available to build oracle/_ref."""
import numpy as np
import pytest

import oracle as O
from aleator_gb300 import workloads as W


@pytest.fixture(scope="module")
def fw():
    return W.cubic_framework(seed=99, charged=True)


def test_philox_bit_exact(orc, ref):
    for seed, stream, first in [(1, 0, 0), (2**63 + 5, 2**40 + 3, 2**32 - 4), (42, 999, 123456)]:
        assert np.array_equal(orc.philox_u64(seed, stream, first, 512), ref.philox_u64(seed, stream, first, 512))


def test_min_image_bit_exact(orc, ref):
    rng = np.random.default_rng(11)
    for angles in [(90, 90, 90), (60, 60, 60), (70, 80, 100), (89.5, 90, 90), (100, 110, 95)]:
        m = W.lattice_from_parameters(17.0, 19.0, 23.0, *angles)
        a = rng.uniform(-50, 50, (200, 3))
        b = rng.uniform(-50, 50, (200, 3))
        assert np.array_equal(orc.min_image(m, a, b), ref.min_image(m, a, b))


@pytest.mark.parametrize("trunc", [O.TRUNCATED, O.SHIFTED, O.LINEAR_FORCE_SHIFTED])
def test_grid_bit_exact(orc, ref, fw, trunc):
    ff = dict(eps=fw.eps, sigma=fw.sigma, cutoff=11.0, truncation=trunc)
    g = ref.grid(ff, fw.lattice, fw.x, fw.y, fw.z, fw.species, [4], 2.5)
    pts = np.random.default_rng(3).uniform(0, 26, (64, 3))
    mine_table = orc.grid_build(ff, fw.lattice, fw.x, fw.y, fw.z, fw.species, 4, 2.5, threads=4)
    assert np.array_equal(orc.grid_interpolate(fw.lattice, g.counts, mine_table, pts),
                          g.interpolate(4, pts))


def test_widom_bit_exact(orc, ref, fw):
    ff = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED)
    ew = dict(alpha=0.3, rc=12.0, kmax=5)
    for guest, e in ((W.ch4_guest(fw), None), (W.co2_guest(fw), ew)):
        for order in (O.DRAWS_RIGHT_TO_LEFT,):
            kr, pr = ref.widom(ff, e, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guest,
                               298.0, 5, 7, 200, draw_order=order, per_trial=True)
            ko, po = orc.widom(ff, e, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species, guest,
                               298.0, 5, 7, 200, draw_order=order, per_trial=True)
            assert kr[0] == kr[1] == ko
            assert np.array_equal(pr, po)


def test_ewald_state_bit_exact(orc, ref, fw):
    a, b = ref.ewald_state(fw.lattice, fw.x, fw.y, fw.z, fw.charge, 0.3, 5), \
        orc.ewald_state(fw.lattice, fw.x, fw.y, fw.z, fw.charge, 0.3, 5)
    rng = np.random.default_rng(1)
    sites = np.array([[0, 0, -1.16, -0.35], [0, 0, 0, 0.7], [0, 0, 1.16, -0.35]])
    mols = []
    for step in range(40):
        new = sites.copy()
        new[:, :3] += rng.uniform(0, 25, 3)
        if mols and rng.uniform() < 0.5:
            rem, add = mols.pop(), np.zeros((0, 4))
        else:
            rem, add = np.zeros((0, 4)), new
            mols.append(new)
        assert a.propose(rem, add) == b.propose(rem, add)
        a.commit(rem, add)
        b.commit(rem, add)
        assert a.energy() == b.energy()
    assert np.array_equal(a.raw(), b.raw())


@pytest.mark.parametrize("cell", ["cubic", "triclinic"])
def test_grid_bit_exact_beyond_half_width(orc, ref, fw, cell):
    """The reference's constructor takes a cutoff above L_perp/2 and sums one
    minimum image per atom; the restatement does the same (bit-exact
    interpolations of its tables)."""
    if cell == "cubic":
        f, rc = fw, 13.5  # L/2 = 12.916
    else:
        f, rc = W.triclinic_supercell(reps=1, seed=31), 11.5  # L_perp/2 ~ 10.9
    ff = dict(eps=f.eps, sigma=f.sigma, cutoff=rc, truncation=O.SHIFTED)
    sid = f.guest_species["CH4"]
    g = ref.grid(ff, f.lattice, f.x, f.y, f.z, f.species, [sid], 2.0)
    pts = np.random.default_rng(4).uniform(0, 24, (64, 3))
    mine = orc.grid_build(ff, f.lattice, f.x, f.y, f.z, f.species, sid, 2.0, threads=4)
    assert np.array_equal(orc.grid_interpolate(f.lattice, g.counts, mine, pts), g.interpolate(sid, pts))
