"""Ewald on the GPU: reciprocal terms, the incremental S(k) cache (the
reference's drift, negation and rollback gates, test_ewald_incremental_state.cc)
and the full breakdown against NIST SPC/E and the NaCl Madelung constant.
FP64 throughout: 1e-10 relative (1 K floor) against the reference."""
import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu


def _cube_state(A, e):
    box = float(e["box"])
    fx = e["framework"]
    p = A.ParticleData(fx[:, 0], fx[:, 1], fx[:, 2], e["framework_q"])
    return A.EwaldIncrementalState(A.Ewald(float(e["alpha"]), 9.0, int(e["kmax"])), p,
                                   np.diag([box] * 3)), p


def test_incremental_sequence_matches_reference(lib):
    A, _ = lib
    e = golden("ewald_state")
    st, _ = _cube_state(A, e)
    off = 0
    for i in range(len(e["op_delta"])):
        nr, na = int(e["op_removed"][i]), int(e["op_added"][i])
        rem = e["op_sites"][off:off + nr]
        add = e["op_sites"][off + nr:off + nr + na]
        off += nr + na
        d = st.propose(rem, add)
        assert abs(d - e["op_delta"][i]) <= 1e-10 * max(1.0, abs(e["op_delta"][i]))
        if e["op_commit"][i]:
            st.commit(rem, add)
        en = st.committed_energy()
        assert abs(en - e["op_energy"][i]) <= 1e-10 * max(1.0, abs(e["op_energy"][i]))
    assert rel_err(st.raw_state_for_testing(), e["raw_final"]).max() <= 1e-10


def _co2(c):
    return np.array([[c[0], c[1], c[2] - 1.16, -0.35], [c[0], c[1], c[2], 0.7],
                     [c[0], c[1], c[2] + 1.16, -0.35]])


def test_drift_gate_every_step(lib):
    """test_ewald_incremental_state.cc:137-222: after every step the committed
    energy equals a from-scratch recomputation to 1e-10."""
    A, _ = lib
    e = golden("ewald_state")
    st, fw = _cube_state(A, e)
    rng = np.random.default_rng(7)
    box = float(e["box"])
    mols = []
    for step in range(300):
        pick = rng.uniform()
        c = rng.uniform(0, box, 3)
        if pick < 0.4 or not mols:
            rem, add = np.zeros((0, 4)), _co2(c)
        elif pick < 0.7:
            rem, add = mols[-1], np.zeros((0, 4))
        else:
            rem = mols[-1]
            add = rem.copy()
            add[:, :3] += rng.uniform(-1.5, 1.5, 3)
        st.propose(rem, add)
        if rng.uniform() < 0.5:
            st.commit(rem, add)
            if len(rem) == 0:
                mols.append(add)
            elif len(add) == 0:
                mols.pop()
            else:
                mols[-1] = add
        allx = np.concatenate([np.stack([fw.x, fw.y, fw.z, fw.charge], 1)] + mols)
        p = A.ParticleData(allx[:, 0], allx[:, 1], allx[:, 2], allx[:, 3])
        molecules = [list(range(8 + 3 * k, 8 + 3 * k + 3)) for k in range(len(mols))]
        fresh = st.recompute_from_scratch(p, molecules)
        assert abs(fresh - st.committed_energy()) <= 1e-10 * max(1.0, abs(fresh))
    # resync reproduces the recomputation
    st.resync(p, molecules)
    assert abs(st.committed_energy() - fresh) <= 1e-10 * max(1.0, abs(fresh))


def test_negation_and_rollback(lib):
    """Insertion/deletion deltas are exact negatives (1e-9, :342-387) and a
    rejected trial leaves the committed cache bit-identical (:389-430)."""
    A, _ = lib
    e = golden("ewald_state")
    st, _ = _cube_state(A, e)
    rng = np.random.default_rng(99)
    for _ in range(50):
        s = _co2(rng.uniform(0, 20.0, 3))
        di = st.propose_insertion(s)
        st.commit_insertion(s)
        dd = st.propose_deletion(s)
        assert abs(di + dd) <= 1e-9 * max(1.0, abs(di))
        st.commit_deletion(s)
    committed = _co2((10.0, 10.0, 10.0))
    st.commit_insertion(committed)
    before = st.raw_state_for_testing()
    st.propose_insertion(_co2((3.0, 3.0, 3.0)))
    st.propose_deletion(committed)
    moved = committed.copy()
    moved[:, 0] += 5.0
    st.propose_move(committed, moved)
    assert np.array_equal(before, st.raw_state_for_testing())


def test_terms_and_breakdown(lib):
    A, _ = lib
    t = golden("ewald_terms")
    g = golden("grid_cubic")
    k, w = A.ewald_reciprocal_terms(g["lattice"], float(t["alpha"]), int(t["kmax"]))
    assert np.array_equal(k, t["k"]) and rel_err(w, t["w"], floor=1e-300).max() <= 1e-14
    b = golden("ewald_breakdown_cubic")
    p = A.ParticleData(g["x"], g["y"], g["z"], g["charge"], g["species"])
    mine = A.ewald_energy_breakdown(A.Ewald(float(b["alpha"]), float(b["rc"]), int(b["kmax"])), p,
                                    g["lattice"])
    assert rel_err(mine, b["breakdown"]).max() <= 1e-10
    st = A.EwaldIncrementalState(A.Ewald(float(b["alpha"]), float(b["rc"]), int(b["kmax"])), p, g["lattice"])
    assert abs(st.committed_energy() - (mine[1] + mine[2])) <= 1e-10 * abs(mine[1] + mine[2])


def test_madelung_and_nist_spce(lib):
    A, _ = lib
    m = golden("madelung")
    xyz = m["xyz"]
    p = A.ParticleData(xyz[:, 0], xyz[:, 1], xyz[:, 2], m["q"])
    b = A.ewald_energy_breakdown(A.Ewald(float(m["alpha"]), float(m["rc"]), int(m["kmax"])), p,
                                 np.diag(m["box"]))
    assert rel_err(b, m["breakdown"]).max() <= 1e-10
    mad = -b[:4].sum() / 167100.9468982874 / float(m["formula_units"])
    assert abs(mad - float(m["published"])) <= 1e-6 * float(m["published"])
    s = golden("nist_spce1")
    xyz = s["xyz"]
    p = A.ParticleData(xyz[:, 0], xyz[:, 1], xyz[:, 2], s["q"])
    b = A.ewald_energy_breakdown(A.Ewald(float(s["alpha"]), float(s["rc"]), int(s["kmax"])), p,
                                 np.diag(s["box"]), s["exclusions"])
    assert rel_err(b, s["breakdown"]).max() <= 1e-10
    assert (rel_err(b[:4], s["published"]) <= 5e-4).all()


def test_real_space_particle_energy(lib, orc):
    A, _ = lib
    g = golden("grid_cubic")
    p = A.ParticleData(g["x"], g["y"], g["z"], g["charge"], g["species"])
    q = np.arange(0, 424, 7)
    ex = [1, 2, 3]
    got = A.ewald_real_space_particle_energy(A.Ewald(0.31, 12.0, 5), p, g["lattice"], q, ex)
    want = [orc.ewald_real_space_particle_energy(g["lattice"], g["x"], g["y"], g["z"], g["charge"],
                                                 0.31, 12.0, int(i), ex) for i in q]
    assert rel_err(got, want).max() <= 1e-10
