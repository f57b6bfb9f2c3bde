"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run where the reference tree is present, naming its root as the argument or
in ALEA_REFERENCE_ROOT:

    python tests/golden/make_golden.py [REFERENCE_ROOT] [--only=irmof1]

It builds oracle/_ref (the reference's hot-path sources compiled by
oracle/build_ref.sh), runs the reference code on seeded synthetic inputs and
on the reference's own test data (NIST SRSW LJ and SPC/E configurations, read
from the reference's tests/validation/data/), and writes compact .npz
fixtures. The published NIST reference numbers are read from the reference's
test sources (tests/validation/test_lennard_jones_nist.cc:122-162,
test_ewald_spce_water.cc:134-147). Nothing here runs at test time.
"""
from __future__ import annotations

import json
import os
import re
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle as O  # noqa: E402
from aleator_gb300 import workloads as W  # noqa: E402

OUT = Path(__file__).resolve().parent


def parse_nist_lj_reference(text: str):
    """{config file: [(label, cutoff, truncation, upair, wpair, ulrc, tail)]}"""
    out = {}
    blocks = re.split(r'\{"(lj_sample_config_periodic\d\.txt)"', text)
    for name, body in zip(blocks[1::2], blocks[2::2]):
        rows = re.findall(r'\{"(L\w+ rc\*=[\d.]+)",\s*([\d.]+),\s*LennardJonesTruncation::(\w+),'
                          r'\s*([-\d.eE+]+),\s*([-\d.eE+]+),\s*([-\d.eE+]+),\s*(true|false)\}', body)
        out[name] = [[r[0], float(r[1]), r[2], float(r[3]), float(r[4]), float(r[5]),
                      r[6] == "true"] for r in rows]
    return out


def parse_nist_spce_reference(text: str):
    rows = re.findall(r'\{"(spce_sample_config_periodic\d\.txt)",\s*(\d+),\s*([-\d.eE+]+),\s*'
                      r'([-\d.eE+]+),\s*([-\d.eE+]+),\s*\n?\s*([-\d.eE+]+)\}', text)
    return {r[0]: [int(r[1])] + [float(v) for v in r[2:]] for r in rows}


def load_xyz(path: Path, with_type=False):
    tok = path.read_text().split()
    lx, ly, lz = (float(v) for v in tok[:3])
    n = int(tok[3])
    stride = 5 if with_type else 4
    count = 3 * n if with_type else n
    body = tok[4:4 + stride * count]
    xyz = np.array([[float(body[stride * i + 1 + c]) for c in range(3)] for i in range(count)])
    types = [body[stride * i + 4] for i in range(count)] if with_type else None
    return np.diag([lx, ly, lz]), xyz, types


def irmof1_fixture(refroot: Path, ref) -> dict:
    """The real IRMOF-1 cell as the reference's readCif reads it
    (tests/validation/data/irmof1/IRMOF-1.cif), with the force field of the
    reference's CH4/IRMOF-1 validation test: the UFF-derived GenericMOFs
    parameters per element and the CH4 site, parsed from that test's source
    (test_gcmc_ch4_irmof1_isotherm.cc:61-76, 98-101)."""
    r = ref.read_cif(refroot / "tests/validation/data/irmof1/IRMOF-1.cif")
    src = (refroot / "tests/validation/test_gcmc_ch4_irmof1_isotherm.cc").read_text()
    table = dict((m[0], (float(m[1]), float(m[2]))) for m in
                 re.findall(r'\{"(\w+)",\s*\{([\d.]+),\s*([\d.]+)\}\}', src))
    ch4 = re.search(r"ljParameters\.push_back\(\{([\d.]+),\s*([\d.]+)\}\);\s*//\s*CH4", src)
    cutoff = re.search(r"const double cutoff = ([\d.]+);", src)
    eps = [table[s][0] for s in r["symbols"]] + [float(ch4.group(1))]
    sigma = [table[s][1] for s in r["symbols"]] + [float(ch4.group(2))]
    return dict(lattice=r["lattice"], x=r["x"], y=r["y"], z=r["z"], species=r["species"],
                charge=r["charge"], symbols=np.array(r["symbols"]), eps=np.array(eps),
                sigma=np.array(sigma), cutoff=np.array(float(cutoff.group(1))))


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--only=")]
    only = [a.split("=", 1)[1] for a in sys.argv[1:] if a.startswith("--only=")]
    root = args[0] if args else os.environ.get("ALEA_REFERENCE_ROOT")
    if not root:
        sys.exit("make_golden.py: name the reference root (argument or ALEA_REFERENCE_ROOT)")
    refroot = Path(root)
    O.build_reference(str(refroot))
    ref = O.Reference()
    if only == ["irmof1"]:  # regenerate this one fixture, keep the others
        data = irmof1_fixture(refroot, ref)
        np.savez_compressed(OUT / "irmof1.npz", **data)
        man = json.loads((OUT / "MANIFEST.json").read_text())
        man["irmof1"] = sorted(data.keys())
        (OUT / "MANIFEST.json").write_text(json.dumps(man, indent=1) + "\n")
        print("wrote irmof1 to", OUT)
        return
    fixtures = {}

    # ---- Philox streams (counter_based_rng.cc:56-79)
    fixtures["philox"] = dict(
        u64_42_0=ref.philox_u64(42, 0, 0, 4096),
        u64_7_3_skip1000=ref.philox_u64(7, 3, 1000, 1024),
        u64_big=ref.philox_u64(0xDEADBEEFCAFEF00D, 0x0123456789ABCDEF, (1 << 32) - 8, 64),
        uniform_42_0=ref.philox_uniform(42, 0, 0, 4096),
        uniform_2026_999=ref.philox_uniform(2026, 999, 0, 1024),
    )

    # ---- Cubic 424-atom framework: grid, interpolation, Widom
    fw = W.cubic_framework(charged=True)
    ff = dict(eps=fw.eps, sigma=fw.sigma, cutoff=12.8, truncation=O.SHIFTED,
              mixing=O.LORENTZ_BERTHELOT)
    ch4 = fw.guest_species["CH4"]
    guests = [ch4, fw.guest_species["CO2_C"], fw.guest_species["CO2_O"]]
    g = ref.grid(ff, fw.lattice, fw.x, fw.y, fw.z, fw.species, guests, 1.5)
    with tempfile.TemporaryDirectory() as td:
        p = Path(td) / "g.bin"
        g.serialize(p)
        cache_bytes = p.read_bytes()
    pts = np.random.default_rng(20260805).uniform(-10.0, 40.0, size=(2000, 3))
    interp = np.stack([g.interpolate(s, pts) for s in guests])
    fixtures["grid_cubic"] = dict(
        lattice=fw.lattice, x=fw.x, y=fw.y, z=fw.z, species=fw.species, charge=fw.charge,
        eps=fw.eps, sigma=fw.sigma, cutoff=12.8, spacing=1.5, guests=np.array(guests, np.uint32),
        counts=np.array(g.counts, np.int32), cache_file=np.frombuffer(cache_bytes, np.uint8),
        cache_name=np.array(g.cache_name()), points=pts, interp=interp)

    kh, per = ref.widom(ff, None, fw.lattice, fw.x, fw.y, fw.z, None, fw.species,
                        W.ch4_guest(fw), 298.0, 42, 0, 4000, per_trial=True)
    assert kh[0] == kh[1], "Widom replay diverged from MonteCarloEngine"
    fixtures["widom_ch4"] = dict(kh=kh[0], per_trial=per, seed=42, stream=0, temperature=298.0)

    alpha, kmax10 = W.ewald_parameters(fw.lattice, 12.0)
    ew = dict(alpha=alpha, rc=12.0, kmax=6)
    kh, per = ref.widom(ff, ew, fw.lattice, fw.x, fw.y, fw.z, fw.charge, fw.species,
                        W.co2_guest(fw), 298.0, 42, 0, 500, per_trial=True)
    assert kh[0] == kh[1]
    fixtures["widom_co2"] = dict(kh=kh[0], per_trial=per, alpha=alpha, ewald_rc=12.0, kmax=6,
                                 seed=42, stream=0, temperature=298.0)
    k, w = ref.ewald_terms(fw.lattice, alpha, kmax10)
    fixtures["ewald_terms"] = dict(alpha=alpha, kmax=kmax10, k=k, w=w)
    fixtures["ewald_breakdown_cubic"] = dict(
        alpha=alpha, rc=12.0, kmax=6,
        breakdown=ref.ewald_breakdown(fw.lattice, fw.x, fw.y, fw.z, fw.charge, alpha, 12.0, 6))

    # ---- Triclinic cell (70/80/100 degrees, one base cell, rc 10 < L_perp/2)
    tfw = W.triclinic_supercell(reps=1)
    tff = dict(eps=tfw.eps, sigma=tfw.sigma, cutoff=10.0, truncation=O.SHIFTED)
    tg = ref.grid(tff, tfw.lattice, tfw.x, tfw.y, tfw.z, tfw.species,
                  [tfw.guest_species["CO2_O"]], 1.0)
    with tempfile.TemporaryDirectory() as td:
        p = Path(td) / "g.bin"
        tg.serialize(p)
        tbytes = p.read_bytes()
    a = np.random.default_rng(5).uniform(-40, 40, size=(512, 3))
    b = np.random.default_rng(6).uniform(-40, 40, size=(512, 3))
    kh, per = ref.widom(tff, dict(alpha=0.35, rc=10.0, kmax=5), tfw.lattice, tfw.x, tfw.y, tfw.z,
                        tfw.charge, tfw.species, W.co2_guest(tfw), 298.0, 7, 3, 300,
                        per_trial=True)
    assert kh[0] == kh[1]
    fixtures["triclinic"] = dict(
        lattice=tfw.lattice, x=tfw.x, y=tfw.y, z=tfw.z, species=tfw.species, charge=tfw.charge,
        eps=tfw.eps, sigma=tfw.sigma, counts=np.array(tg.counts, np.int32),
        cache_file=np.frombuffer(tbytes, np.uint8), min_image_a=a, min_image_b=b,
        min_image=ref.min_image(tfw.lattice, a, b), widom_kh=kh[0], widom_per_trial=per)

    # ---- EwaldIncrementalState scripted sequence (test_ewald_incremental_state.cc:137-222)
    box = 20.0
    m = np.diag([box] * 3)
    cs = [box * 0.25, box * 0.75]
    fx = np.array([[x, y, z] for x in cs for y in cs for z in cs])
    fq = np.array([1.0 if i % 2 == 0 else -1.0 for i in range(8)])
    st = ref.ewald_state(m, fx[:, 0], fx[:, 1], fx[:, 2], fq, 0.25, 6)
    ops = []
    rng = np.random.default_rng(7)
    mols = []
    for step in range(300):
        pick = rng.uniform()
        c = rng.uniform(0, box, 3)
        sites = np.array([[c[0], c[1], c[2] - 1.16, -0.35], [c[0], c[1], c[2], 0.7],
                          [c[0], c[1], c[2] + 1.16, -0.35]])
        if pick < 0.4 or not mols:
            rem, add = np.zeros((0, 4)), sites
        elif pick < 0.7:
            rem, add = mols[-1], np.zeros((0, 4))
        else:
            rem = mols[-1]
            add = rem.copy()
            add[:, :3] += rng.uniform(-1.5, 1.5, 3)
        delta = st.propose(rem, add)
        commit = rng.uniform() < 0.5
        if commit:
            st.commit(rem, add)
            if len(rem) == 0:
                mols.append(add)
            elif len(add) == 0:
                mols.pop()
            else:
                mols[-1] = add
        ops.append((rem.copy(), add.copy(), delta, commit, st.energy()))
    fixtures["ewald_state"] = dict(
        box=box, framework=fx, framework_q=fq, alpha=0.25, kmax=6,
        op_removed=np.array([len(o[0]) for o in ops]),
        op_sites=np.concatenate([np.concatenate([o[0], o[1]]) for o in ops]),
        op_added=np.array([len(o[1]) for o in ops]), op_delta=np.array([o[2] for o in ops]),
        op_commit=np.array([o[3] for o in ops]), op_energy=np.array([o[4] for o in ops]),
        raw_final=st.raw())

    # ---- NIST SRSW LJ (tests/validation/test_lennard_jones_nist.cc)
    nist_txt = (refroot / "tests/validation/test_lennard_jones_nist.cc").read_text()
    table = parse_nist_lj_reference(nist_txt)
    nist = {}
    for name in sorted(table):
        mm, xyz, _ = load_xyz(refroot / "tests/validation/data/nist_lj" / name)
        rows = []
        for label, rc, trunc, upair, wpair, ulrc, tail in table[name]:
            tcode = {"Truncated": O.TRUNCATED, "Shifted": O.SHIFTED,
                     "LinearForceShifted": O.LINEAR_FORCE_SHIFTED}[trunc]
            mine = ref.lj_energy_virial(mm, xyz[:, 0], xyz[:, 1], xyz[:, 2], 1.0, 1.0, rc, tcode)
            rows.append([rc, tcode, upair, wpair, ulrc, float(tail), mine[0], mine[1], mine[2]])
        key = name.replace(".txt", "")
        nist[key + "_box"] = np.diag(mm)
        nist[key + "_xyz"] = xyz
        nist[key + "_rows"] = np.array(rows)
    fixtures["nist_lj"] = nist

    # ---- NIST SRSW SPC/E, first configuration (test_ewald_spce_water.cc:134-216)
    spce_txt = (refroot / "tests/validation/test_ewald_spce_water.cc").read_text()
    spce_ref = parse_nist_spce_reference(spce_txt)
    name = "spce_sample_config_periodic1.txt"
    mm, xyz, types = load_xyz(refroot / "tests/validation/data/nist_spce" / name, with_type=True)
    q = np.array([-2.0 * 0.42380 if t == "O" else 0.42380 for t in types])
    excl = []
    for k in range(len(types) // 3):
        excl += [(3 * k, 3 * k + 1), (3 * k, 3 * k + 2), (3 * k + 1, 3 * k + 2)]
    alpha_s = 5.6 / float(np.min(np.diag(mm)))
    bd = ref.ewald_breakdown(mm, xyz[:, 0], xyz[:, 1], xyz[:, 2], q, alpha_s, 10.0, 5,
                             np.array(excl, np.uint64), skin=0.1)
    fixtures["nist_spce1"] = dict(box=np.diag(mm), xyz=xyz, q=q, exclusions=np.array(excl),
                                  alpha=alpha_s, rc=10.0, kmax=5, breakdown=bd,
                                  published=np.array(spce_ref[name][1:]))

    # ---- NaCl Madelung (test_ewald_madelung.cc:41, 108-127)
    a, nrep = 1.0, 3
    na = [(0, 0, 0), (a, a, 0), (a, 0, a), (0, a, a)]
    cl = [(a, 0, 0), (0, a, 0), (0, 0, a), (a, a, a)]
    pos, qq = [], []
    for ox in range(nrep):
        for oy in range(nrep):
            for oz in range(nrep):
                d = np.array([ox, oy, oz]) * 2.0 * a
                pos += [np.array(s) + d for s in na]
                qq += [1.0] * 4
                pos += [np.array(s) + d for s in cl]
                qq += [-1.0] * 4
    pos = np.array(pos)
    mm = np.diag([2.0 * a * nrep] * 3)
    bd = ref.ewald_breakdown(mm, pos[:, 0], pos[:, 1], pos[:, 2], np.array(qq), 1.4, 2.9, 12)
    fixtures["madelung"] = dict(box=np.diag(mm), xyz=pos, q=np.array(qq), alpha=1.4, rc=2.9,
                                kmax=12, breakdown=bd, published=1.747564594633,
                                formula_units=4 * nrep ** 3)

    # ---- Peng-Robinson fugacities (CO2, CH4) at the workload pressures
    pressures = np.array([1e3, 1e4, 1e5, 1e6, 3e6, 5e6])
    fixtures["peng_robinson"] = dict(
        pressures=pressures,
        co2=np.array([ref.pr_fugacity(*W.CO2_CRITICAL, 298.0, p) for p in pressures]),
        ch4=np.array([ref.pr_fugacity(*W.METHANE_CRITICAL, 298.0, p) for p in pressures]))

    # ---- PengRobinsonMixture: CO2 + CH4 (k_ij 0 and 0.09), CO2 + N2 + CH4, over
    # pressures and compositions; critical constants as in the workloads
    n2 = (126.19, 3.3958e6, 0.0372)  # the reference's mixture test substance
    mix_cases = [([W.CO2_CRITICAL, W.METHANE_CRITICAL], None),
                 ([W.CO2_CRITICAL, W.METHANE_CRITICAL], [[0.0, 0.09], [0.09, 0.0]]),
                 ([W.CO2_CRITICAL, n2, W.METHANE_CRITICAL], None)]
    rows, fails = [], []
    for ci, (subs, kij) in enumerate(mix_cases):
        for t in (250.0, 298.0, 350.0):
            for p in (1e4, 1e6, 5e6):
                for x0 in (0.1, 0.5, 0.85):
                    x = [x0, 1.0 - x0] if len(subs) == 2 else [x0, (1.0 - x0) * 0.6, (1.0 - x0) * 0.4]
                    try:
                        z, f = ref.pr_mixture(subs, t, p, x, kij)
                    except ValueError:  # the reference's Newton solve gives up (near condensation)
                        fails.append([ci, t, p] + x + [0.0] * (3 - len(x)))
                        continue
                    rows.append([ci, t, p] + x + [0.0] * (3 - len(x)) + [z] + list(f) +
                                [0.0] * (3 - len(f)))
    fixtures["peng_robinson_mixture"] = dict(
        tc=np.array([[s[0] for s in c] + [0.0] * (3 - len(c)) for c, _ in mix_cases]),
        pc=np.array([[s[1] for s in c] + [1.0] * (3 - len(c)) for c, _ in mix_cases]),
        omega=np.array([[s[2] for s in c] + [0.0] * (3 - len(c)) for c, _ in mix_cases]),
        n=np.array([len(c) for c, _ in mix_cases]),
        kij=np.array([np.zeros((3, 3)) if k is None else np.pad(np.array(k), ((0, 1), (0, 1)))
                      for _, k in mix_cases]),
        has_kij=np.array([k is not None for _, k in mix_cases]),
        rows=np.array(rows),  # case, T, P, x0..x2, Z, f0..f2
        fails=np.array(fails).reshape(-1, 6))  # case, T, P, x0..x2: the solve does not converge

    # ---- readCif on the synthetic CIF files of tests/golden/cif (written for
    # these tests): the parsed structure, or the reference's error message
    cif = {}
    for f in sorted((OUT / "cif").glob("*.cif")):
        try:
            r = ref.read_cif(f)
        except RuntimeError as e:
            cif[f"{f.stem}__error"] = np.array(str(e))
            continue
        for k in ("lattice", "x", "y", "z", "charge", "mass", "species", "occupancy"):
            cif[f"{f.stem}__{k}"] = r[k]
        cif[f"{f.stem}__symbols"] = np.array(r["symbols"])
        cif[f"{f.stem}__labels"] = np.array(r["labels"])
    fixtures["cif_structures"] = cif
    fixtures["irmof1"] = irmof1_fixture(refroot, ref)

    for name, data in fixtures.items():
        np.savez_compressed(OUT / f"{name}.npz", **data)
    (OUT / "MANIFEST.json").write_text(json.dumps(
        {n: sorted(d.keys()) for n, d in fixtures.items()}, indent=1) + "\n")
    print("wrote", len(fixtures), "fixtures to", OUT)


if __name__ == "__main__":
    main()
