"""Seeded synthetic workloads: deterministic, with the configured shapes."""
import numpy as np

from aleator_gb300 import workloads as W


def test_cubic_framework_shape():
    fw = W.cubic_framework(charged=True)
    assert fw.n_atoms == 424
    assert np.bincount(fw.species).tolist() == [32, 104, 192, 96]
    assert abs(fw.charge.sum()) < 1e-10 and np.abs(fw.charge).max() <= 2.4
    assert (fw.sigma[:4] >= 2.5).all() and (fw.sigma[:4] <= 3.5).all()
    assert (fw.eps[:4] >= 20).all() and (fw.eps[:4] <= 100).all()
    # 1.0 Å minimum-image separation
    pos = np.stack([fw.x, fw.y, fw.z], 1)
    d = pos[:, None, :] - pos[None, :, :]
    d -= 25.832 * np.rint(d / 25.832)
    r = np.sqrt((d ** 2).sum(-1)) + np.eye(len(pos)) * 100
    assert r.min() >= 1.0
    again = W.cubic_framework(charged=True)
    assert np.array_equal(again.x, fw.x) and np.array_equal(again.charge, fw.charge)


def test_triclinic_supercell_shape():
    fw = W.triclinic_supercell(reps=2)
    assert fw.n_atoms == 8 * 422
    w = W.perpendicular_widths(fw.lattice)
    assert np.allclose(w / 2, [22.87, 21.83, 21.83], atol=0.02)
    assert W.minimum_replication(W.lattice_from_parameters(24, 24, 24, 70, 80, 100), 12.8) == (2, 2, 2)


def test_ewald_parameters():
    fw = W.cubic_framework()
    alpha, kmax = W.ewald_parameters(fw.lattice, 12.0)
    assert abs(alpha - 0.3097) < 1e-3 and kmax == 10


def test_random_triclinic_frameworks_shape():
    """The screening set's frameworks. Base cells (a cutoff small enough that
    nothing is replicated): a, b, c in 10-40 A, angles in 60-120 degrees, 50-2000
    atoms (fewer only where 8 A^3 per atom caps a small cell), framework types
    0-3 plus the CH4 probe. At the 12.8 A cutoff every perpendicular width
    exceeds 2 rc after replication (the reference's buildSupercell rule). The same
    seed gives the same frameworks."""
    for fw in W.random_triclinic_frameworks(12, seed=77, cutoff=1.0):
        m = np.asarray(fw.lattice)
        lengths = np.linalg.norm(m, axis=1)
        assert ((lengths >= 10.0) & (lengths <= 40.0)).all(), lengths
        cos = [m[1] @ m[2] / (lengths[1] * lengths[2]), m[0] @ m[2] / (lengths[0] * lengths[2]),
               m[0] @ m[1] / (lengths[0] * lengths[1])]
        ang = np.degrees(np.arccos(cos))
        assert ((ang >= 60 - 1e-9) & (ang <= 120 + 1e-9)).all(), ang
        vol = abs(np.linalg.det(m))
        assert min(50, int(vol / 8.0)) <= fw.n_atoms <= 2000
        assert fw.species.max() <= 3 and fw.guest_species == {"CH4": 4}
    fws = W.random_triclinic_frameworks(12, seed=77)
    for fw in fws:
        assert (W.perpendicular_widths(np.asarray(fw.lattice)) > 2 * 12.8).all()
    again = W.random_triclinic_frameworks(12, seed=77)
    assert all(np.array_equal(a.x, b.x) and np.array_equal(a.lattice, b.lattice)
               for a, b in zip(fws, again))
