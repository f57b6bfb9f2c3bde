"""Per-particle LJ energies on the GPU (LennardJones::computeParticleEnergy)
against the reference on the NIST SRSW configurations: total U_pair =
half the sum of the per-particle energies, 1e-10 relative against the
reference's own value and 5e-5 against NIST's published digits."""
import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu


def test_nist_lj_configs(lib):
    A, _ = lib
    n = golden("nist_lj")
    for cfg in ("lj_sample_config_periodic1", "lj_sample_config_periodic2",
                "lj_sample_config_periodic3", "lj_sample_config_periodic4"):
        box, xyz = n[cfg + "_box"], n[cfg + "_xyz"]
        p = A.ParticleData(xyz[:, 0], xyz[:, 1], xyz[:, 2])
        for row in n[cfg + "_rows"]:
            rc, trunc, upair, wpair, ulrc, tail, r_u, r_w, r_lrc = row
            ff = A.LennardJones([1.0], [1.0], rc, int(trunc))
            per = A.lj_particle_energy(ff, p, np.diag(box), np.arange(len(xyz)))
            u = 0.5 * per.sum()
            assert abs(u - r_u) <= 1e-10 * abs(r_u)
            assert abs(u - upair) <= 5e-5 * abs(upair)
            if tail:
                lrc = A.lj_tail_correction(ff, p, np.diag(box))
                assert abs(lrc - r_lrc) <= 1e-12 * abs(r_lrc)


def test_move_energy_with_exclusions(lib, orc):
    A, _ = lib
    g = golden("grid_cubic")
    x = np.concatenate([g["x"], [5.0, 5.0, 5.0]])
    y = np.concatenate([g["y"], [6.0, 6.0, 6.0]])
    z = np.concatenate([g["z"], [7.0 - 1.16, 7.0, 7.0 + 1.16]])
    sp = np.concatenate([g["species"], [6, 5, 6]]).astype(np.uint32)
    ff = A.LennardJones(g["eps"], g["sigma"], 12.8, A.SHIFTED)
    p = A.ParticleData(x, y, z, None, sp)
    sites = [424, 425, 426]
    got = A.lj_particle_energy(ff, p, g["lattice"], sites, sites)
    od = dict(eps=g["eps"], sigma=g["sigma"], cutoff=12.8, truncation=1)
    want = [orc.lj_particle_energy(od, g["lattice"], x, y, z, sp, s, sites) for s in sites]
    assert rel_err(got, want).max() <= 1e-10
