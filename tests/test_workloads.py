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
