"""The C restatement (oracle/) against the golden vectors made by the
reference itself (tests/golden/make_golden.py) and the known-answer tests the
reference's own test suite holds. Runs on any CPU host.

Tolerances: integer work is bit-exact; FP64 energies 1e-12 relative (the
fixtures were made on another host whose libm may differ in the last bit)."""
import numpy as np
import pytest

import oracle as O
from conftest import golden, rel_err

# Random123 known-answer vectors as listed in the reference's
# tests/validation/test_philox_random123_vectors.cc:22-44.
KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


@pytest.mark.parametrize("ctr,key,expected", KAT)
def test_philox_kat(orc, ctr, key, expected):
    assert list(orc.philox4x32_10(ctr, key)) == expected


def test_philox_streams(orc):
    g = golden("philox")
    assert np.array_equal(orc.philox_u64(42, 0, 0, 4096), g["u64_42_0"])
    assert np.array_equal(orc.philox_u64(7, 3, 1000, 1024), g["u64_7_3_skip1000"])
    assert np.array_equal(orc.philox_u64(0xDEADBEEFCAFEF00D, 0x0123456789ABCDEF, (1 << 32) - 8, 64),
                          g["u64_big"])
    assert np.array_equal(orc.philox_uniform(42, 0, 0, 4096), g["uniform_42_0"])
    assert np.array_equal(orc.philox_uniform(2026, 999, 0, 1024), g["uniform_2026_999"])
    u = orc.philox_uniform(7, 3, 0, 100000)
    assert (u >= 0).all() and (u < 1).all()
    assert abs(u.mean() - 0.5) < 5 * 9.13e-4  # test_philox_random123_vectors.cc:75-94


def test_host_philox_matches(orc):
    from aleator_gb300 import philox_np

    assert np.array_equal(philox_np.u64(42, 0, 0, 2048), orc.philox_u64(42, 0, 0, 2048))
    big = (1 << 32) - 3
    assert np.array_equal(philox_np.u64(5, (1 << 40) + 7, big, 16), orc.philox_u64(5, (1 << 40) + 7, big, 16))


def _cache_tables(cache_bytes):
    import struct
    b = cache_bytes.tobytes()
    off = 4
    for _ in range(3):
        n, = struct.unpack_from("<Q", b, off)
        off += 8 + 8 * n
    n, = struct.unpack_from("<Q", b, off)
    off += 8 + 4 * n + 72
    ns, = struct.unpack_from("<Q", b, off)
    off += 8 + 16 * ns + 9
    n, = struct.unpack_from("<Q", b, off)
    off += 8 + 4 * n + 16
    counts = struct.unpack_from("<3i", b, off)
    off += 12
    nt, = struct.unpack_from("<Q", b, off)
    off += 8
    tables = {}
    for _ in range(nt):
        sid, = struct.unpack_from("<I", b, off)
        n, = struct.unpack_from("<Q", b, off + 4)
        tables[sid] = np.frombuffer(b, dtype=np.float64, count=n, offset=off + 12).copy()
        off += 12 + 8 * n
    return counts, tables


def test_grid_nodes_match_reference(orc):
    g = golden("grid_cubic")
    ff = dict(eps=g["eps"], sigma=g["sigma"], cutoff=float(g["cutoff"]), truncation=O.SHIFTED)
    counts, tables = _cache_tables(g["cache_file"])
    assert counts == tuple(g["counts"])
    assert orc.grid_point_counts(g["lattice"], float(g["spacing"])) == counts
    for sid, table in tables.items():
        mine = orc.grid_build(ff, g["lattice"], g["x"], g["y"], g["z"], g["species"], sid,
                              float(g["spacing"]), threads=4)
        assert rel_err(mine, table).max() <= 1e-12
    # trilinear interpolation on the reference's tables
    for i, sid in enumerate(g["guests"]):
        got = orc.grid_interpolate(g["lattice"], counts, tables[int(sid)], g["points"])
        assert rel_err(got, g["interp"][i]).max() <= 1e-12


def test_triclinic_grid_and_min_image(orc):
    t = golden("triclinic")
    mi = orc.min_image(t["lattice"], t["min_image_a"], t["min_image_b"])
    assert np.abs(mi - t["min_image"]).max() <= 1e-12
    ff = dict(eps=t["eps"], sigma=t["sigma"], cutoff=10.0, truncation=O.SHIFTED)
    counts, tables = _cache_tables(t["cache_file"])
    sid = list(tables)[0]
    mine = orc.grid_build(ff, t["lattice"], t["x"], t["y"], t["z"], t["species"], sid, 1.0,
                          threads=4)
    assert rel_err(mine, tables[sid]).max() <= 1e-12


def test_widom_per_trial(orc):
    gc = golden("grid_cubic")
    ff = dict(eps=gc["eps"], sigma=gc["sigma"], cutoff=12.8, truncation=O.SHIFTED)
    from aleator_gb300 import workloads as W

    class FW:
        guest_species = {"CH4": 4, "CO2_C": 5, "CO2_O": 6}
    w = golden("widom_ch4")
    kh, per = orc.widom(ff, None, gc["lattice"], gc["x"], gc["y"], gc["z"], None, gc["species"],
                        W.ch4_guest(FW), 298.0, 42, 0, len(w["per_trial"]), per_trial=True)
    assert rel_err(per, w["per_trial"]).max() <= 1e-12
    assert abs(kh / float(w["kh"]) - 1) <= 1e-12
    c = golden("widom_co2")
    ew = dict(alpha=float(c["alpha"]), rc=12.0, kmax=int(c["kmax"]))
    kh, per = orc.widom(ff, ew, gc["lattice"], gc["x"], gc["y"], gc["z"], gc["charge"],
                        gc["species"], W.co2_guest(FW), 298.0, 42, 0, len(c["per_trial"]),
                        per_trial=True)
    assert rel_err(per, c["per_trial"]).max() <= 1e-12
    assert abs(kh / float(c["kh"]) - 1) <= 1e-11


def test_ewald_terms_and_breakdown(orc):
    t = golden("ewald_terms")
    gc = golden("grid_cubic")
    k, w = orc.ewald_terms(gc["lattice"], float(t["alpha"]), int(t["kmax"]))
    assert len(w) == 4336 and np.abs(k - t["k"]).max() == 0.0
    assert rel_err(w, t["w"], floor=1e-300).max() <= 1e-14
    b = golden("ewald_breakdown_cubic")
    mine = orc.ewald_breakdown(gc["lattice"], gc["x"], gc["y"], gc["z"], gc["charge"],
                               float(b["alpha"]), float(b["rc"]), int(b["kmax"]))
    assert rel_err(mine, b["breakdown"]).max() <= 1e-12


def test_ewald_incremental_sequence(orc):
    e = golden("ewald_state")
    box = float(e["box"])
    fx = e["framework"]
    st = orc.ewald_state(np.diag([box] * 3), fx[:, 0], fx[:, 1], fx[:, 2], e["framework_q"],
                         float(e["alpha"]), int(e["kmax"]))
    off = 0
    for i in range(len(e["op_delta"])):
        nr, na = int(e["op_removed"][i]), int(e["op_added"][i])
        rem = e["op_sites"][off:off + nr]
        add = e["op_sites"][off + nr:off + nr + na]
        off += nr + na
        d = st.propose(rem, add)
        assert abs(d - e["op_delta"][i]) <= 1e-12 * max(1.0, abs(e["op_delta"][i]))
        if e["op_commit"][i]:
            st.commit(rem, add)
        assert abs(st.energy() - e["op_energy"][i]) <= 1e-12 * max(1.0, abs(e["op_energy"][i]))
    raw = st.raw()
    assert rel_err(raw, e["raw_final"]).max() <= 1e-12


def test_nist_lj(orc):
    n = golden("nist_lj")
    for cfg in ("lj_sample_config_periodic1", "lj_sample_config_periodic2",
                "lj_sample_config_periodic3", "lj_sample_config_periodic4"):
        box = n[cfg + "_box"]
        xyz = n[cfg + "_xyz"]
        m = np.diag(box)
        for row in n[cfg + "_rows"]:
            rc, trunc, upair, wpair, ulrc, tail, r_u, r_w, r_lrc = row
            ff = dict(eps=[1.0], sigma=[1.0], cutoff=rc, truncation=int(trunc))
            sp = np.zeros(len(xyz), np.uint32)
            per = [orc.lj_particle_energy(ff, m, xyz[:, 0], xyz[:, 1], xyz[:, 2], sp, i)
                   for i in range(len(xyz))]
            u = 0.5 * sum(per)
            assert abs(u - r_u) <= 1e-10 * abs(r_u)            # vs the reference's own value
            assert abs(u - upair) <= 5e-5 * abs(upair)          # vs NIST (5 significant figures)
            if tail:
                lrc = orc.lj_tail(ff, m, sp)
                assert abs(lrc - r_lrc) <= 1e-12 * abs(r_lrc)
                assert abs(lrc - ulrc) <= 5e-5 * abs(ulrc)


def test_madelung_and_spce(orc):
    m = golden("madelung")
    box = m["box"]
    xyz = m["xyz"]
    b = orc.ewald_breakdown(np.diag(box), xyz[:, 0], xyz[:, 1], xyz[:, 2], m["q"],
                            float(m["alpha"]), float(m["rc"]), int(m["kmax"]))
    mad = -b[:4].sum() / O.COULOMB_K * 1.0 / float(m["formula_units"])
    assert abs(mad - float(m["published"])) <= 1e-6 * float(m["published"])
    s = golden("nist_spce1")
    xyz = s["xyz"]
    b = orc.ewald_breakdown(np.diag(s["box"]), xyz[:, 0], xyz[:, 1], xyz[:, 2], s["q"],
                            float(s["alpha"]), float(s["rc"]), int(s["kmax"]), s["exclusions"])
    assert rel_err(b, s["breakdown"]).max() <= 1e-10
    assert (rel_err(b[:4], s["published"]) <= 5e-4).all()


def test_peng_robinson(orc):
    from aleator_gb300 import workloads as W
    p = golden("peng_robinson")
    for i, P in enumerate(p["pressures"]):
        assert abs(orc.pr_fugacity(*W.CO2_CRITICAL, 298.0, P) / p["co2"][i] - 1) <= 1e-13
        assert abs(orc.pr_fugacity(*W.METHANE_CRITICAL, 298.0, P) / p["ch4"][i] - 1) <= 1e-13


def _pr_mixture_cases():
    g = golden("peng_robinson_mixture")
    cases = []
    for ci in range(len(g["n"])):
        n = int(g["n"][ci])
        subs = [(g["tc"][ci][i], g["pc"][ci][i], g["omega"][ci][i]) for i in range(n)]
        kij = g["kij"][ci][:n, :n] if g["has_kij"][ci] else None
        cases.append((n, subs, kij))
    return g, cases


def test_peng_robinson_mixture(orc):
    """The oracle's PengRobinsonMixture against the reference's Z and partial
    fugacities (two and three components, k_ij = 0 and 0.09)."""
    g, cases = _pr_mixture_cases()
    for row in g["rows"]:
        n, subs, kij = cases[int(row[0])]
        z, f = orc.pr_mixture(subs, row[1], row[2], row[3:3 + n], kij)
        assert z == row[6]
        assert np.array_equal(f, row[7:7 + n])
