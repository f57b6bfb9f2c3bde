"""Seeded synthetic frameworks for the energy-grid / Widom / GCMC workloads.

The reference benchmarks its hot path on the real IRMOF-1 cell (cubic
25.832 Å, 424 atoms; benchmarks/bench_gcmc_ch4_irmof1.cc:55-57). The
workloads here imitate that shape with seeded synthetic inputs:

* ``cubic_framework``   — 25.832 Å cube, 424 atoms of 4 types (32/104/192/96),
  positions uniform with 1.0 Å minimum-image rejection, sigma 2.5-3.5 Å and
  eps/kB 20-100 K per type, optional charges uniform in [-1.2, 1.2] e shifted
  to net zero.
* ``triclinic_supercell`` — a 24 Å base cell with angles 70/80/100 degrees,
  ~422 atoms, replicated n x n x n (4x4x4 gives ~27 000 atoms).
* ``random_triclinic_frameworks`` — many cells with a, b, c in 10-40 Å,
  angles 60-120 degrees and 50-2000 atoms, replicated so that the cutoff fits
  (supercell.cc:7-20 rule n * L_perp > 2 rc).

All randomness comes from the Philox4x32-10 stream (seed, stream) of
``philox_np``, so a workload is bit-identical on every host.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .philox_np import uniforms

# united-atom CH4 probe and rigid CO2 (C between two O at 1.16 Å)
CH4_SIGMA, CH4_EPS = 3.73, 148.0
CO2_C = (2.80, 27.0, +0.70)
CO2_O = (3.05, 79.0, -0.35)
CO2_BOND = 1.16
CO2_CRITICAL = (304.1282, 7.3773e6, 0.22394)
METHANE_CRITICAL = (190.6, 4.599e6, 0.011)


@dataclass
class Framework:
    """A rigid framework: lattice rows a_i (Å) and SoA atoms."""

    lattice: np.ndarray  # (3, 3), row i = a_i
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    species: np.ndarray  # uint32 framework LJ type
    charge: np.ndarray
    eps: np.ndarray      # per LJ species (framework types first, then guest types)
    sigma: np.ndarray
    guest_species: dict = field(default_factory=dict)  # name -> LJ species id

    @property
    def n_atoms(self) -> int:
        return int(self.x.shape[0])


def lattice_from_parameters(a, b, c, alpha_deg, beta_deg, gamma_deg) -> np.ndarray:
    """Standard crystallographic cell -> row-vector matrix (a along x, b in xy)."""
    al, be, ga = (math.radians(v) for v in (alpha_deg, beta_deg, gamma_deg))
    ca, cb, cg, sg = math.cos(al), math.cos(be), math.cos(ga), math.sin(ga)
    cx = c * cb
    cy = c * (ca - cb * cg) / sg
    cz2 = 1.0 - ca * ca - cb * cb - cg * cg + 2.0 * ca * cb * cg
    if cz2 <= 0.0:
        raise ValueError("invalid cell angles")
    cz = c * math.sqrt(cz2) / sg
    return np.array([[a, 0.0, 0.0], [b * cg, b * sg, 0.0], [cx, cy, cz]], dtype=np.float64)


def perpendicular_widths(m: np.ndarray) -> np.ndarray:
    vol = abs(float(np.dot(m[0], np.cross(m[1], m[2]))))
    return np.array([vol / np.linalg.norm(np.cross(m[(i + 1) % 3], m[(i + 2) % 3]))
                     for i in range(3)])


_IMAGE_SHIFTS = np.array([n for n in np.array(np.meshgrid([-1, 0, 1], [-1, 0, 1], [-1, 0, 1])).T.reshape(-1, 3)
                          if n.any()], dtype=np.float64)


def _min_image_dist2(m: np.ndarray, minv: np.ndarray, p: np.ndarray, pts: np.ndarray) -> np.ndarray:
    if pts.shape[0] == 0:
        return np.zeros(0)
    df = (pts - p) @ minv
    df -= np.rint(df)
    d = df @ m
    best = np.einsum("ij,ij->i", d, d)
    # small skewed cells: also look at the 26 neighbouring images
    dd = d[None, :, :] + (_IMAGE_SHIFTS @ m)[:, None, :]
    return np.minimum(best, np.einsum("kij,kij->ki", dd, dd).min(axis=0))


def _place_atoms(m: np.ndarray, n_atoms: int, seed: int, stream: int, min_sep: float = 1.0):
    """Uniform positions with minimum-image rejection below ``min_sep`` Å.

    Candidates are checked against the atoms of the 27 neighbouring fractional
    bins only: a bin is at least ``min_sep`` wide across, so every atom closer
    than that is among them and the decisions equal those of a full scan."""
    minv = np.linalg.inv(m)
    nb = np.maximum(1, np.floor(perpendicular_widths(m) / min_sep).astype(int))
    bins: dict = {}
    pos = np.zeros((n_atoms, 3))
    count = 0
    call = 0
    batch = 3 * 256
    while count < n_atoms:
        u = uniforms(seed, stream, call, batch).reshape(-1, 3)
        call += batch
        for f in u:
            p = f @ m
            b = [min(int(f[a] * nb[a]), nb[a] - 1) for a in range(3)]
            cand = []
            for i in {(b[0] + d) % nb[0] for d in (-1, 0, 1)}:
                for j in {(b[1] + d) % nb[1] for d in (-1, 0, 1)}:
                    for k in {(b[2] + d) % nb[2] for d in (-1, 0, 1)}:
                        cand.extend(bins.get((i, j, k), ()))
            if cand and _min_image_dist2(m, minv, p, pos[cand]).min() < min_sep * min_sep:
                continue
            pos[count] = p
            bins.setdefault((b[0], b[1], b[2]), []).append(count)
            count += 1
            if count == n_atoms:
                break
        if call > 3 * 10_000_000:
            raise RuntimeError("could not place atoms at the requested separation")
    return pos, call


def _type_parameters(n_types: int, seed: int, stream: int):
    u = uniforms(seed, stream, 0, 2 * n_types).reshape(n_types, 2)
    sigma = 2.5 + u[:, 0] * 1.0
    eps = 20.0 + u[:, 1] * 80.0
    return eps, sigma


def _charges(n: int, seed: int, stream: int, qmax: float = 1.2):
    q = -qmax + 2.0 * qmax * uniforms(seed, stream, 0, n)
    return q - q.sum() / n


def _with_guests(fw_eps, fw_sigma, guests):
    eps = list(fw_eps)
    sigma = list(fw_sigma)
    ids = {}
    for name, (s, e) in guests.items():
        ids[name] = len(eps)
        eps.append(e)
        sigma.append(s)
    return np.array(eps), np.array(sigma), ids


def cubic_framework(seed: int = 2026, charged: bool = False, length: float = 25.832,
                    counts=(32, 104, 192, 96)) -> Framework:
    """The 424-atom synthetic cubic cell (CH4 and CO2 guest types appended)."""
    m = np.diag([length] * 3).astype(np.float64)
    n = int(sum(counts))
    pos, _ = _place_atoms(m, n, seed, 1)
    species = np.concatenate([np.full(c, t, dtype=np.uint32) for t, c in enumerate(counts)])
    fw_eps, fw_sigma = _type_parameters(len(counts), seed, 2)
    q = _charges(n, seed, 3) if charged else np.zeros(n)
    eps, sigma, ids = _with_guests(fw_eps, fw_sigma, {
        "CH4": (CH4_SIGMA, CH4_EPS), "CO2_C": CO2_C[:2], "CO2_O": CO2_O[:2]})
    return Framework(m, pos[:, 0].copy(), pos[:, 1].copy(), pos[:, 2].copy(), species, q, eps,
                     sigma, ids)


def replicate(fw: Framework, n) -> Framework:
    """supercell.cc:22-59: exact integer lattice translations, cell order i, j, k."""
    nx, ny, nz = n
    m = fw.lattice
    xs, ys, zs, sp, qs = [], [], [], [], []
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                ox = i * m[0][0] + j * m[1][0] + k * m[2][0]
                oy = i * m[0][1] + j * m[1][1] + k * m[2][1]
                oz = i * m[0][2] + j * m[1][2] + k * m[2][2]
                xs.append(fw.x + ox)
                ys.append(fw.y + oy)
                zs.append(fw.z + oz)
                sp.append(fw.species)
                qs.append(fw.charge)
    newm = np.array([nx * m[0], ny * m[1], nz * m[2]])
    return Framework(newm, np.concatenate(xs), np.concatenate(ys), np.concatenate(zs),
                     np.concatenate(sp), np.concatenate(qs), fw.eps, fw.sigma,
                     dict(fw.guest_species))


def minimum_replication(m: np.ndarray, cutoff: float):
    """supercell.cc:7-20"""
    w = perpendicular_widths(m)
    out = []
    for axis in range(3):
        k = 1
        while k * w[axis] <= 2.0 * cutoff:
            k += 1
        out.append(k)
    return tuple(out)


def triclinic_supercell(seed: int = 2027, reps: int = 4, base_atoms: int = 422,
                        charged: bool = True) -> Framework:
    """24 Å base cell, angles 70/80/100 degrees, replicated reps^3 times."""
    m = lattice_from_parameters(24.0, 24.0, 24.0, 70.0, 80.0, 100.0)
    pos, _ = _place_atoms(m, base_atoms, seed, 1)
    counts = (32, 104, 190, base_atoms - 326)
    species = np.concatenate([np.full(c, t, dtype=np.uint32) for t, c in enumerate(counts)])
    fw_eps, fw_sigma = _type_parameters(4, seed, 2)
    q = _charges(base_atoms, seed, 3) if charged else np.zeros(base_atoms)
    eps, sigma, ids = _with_guests(fw_eps, fw_sigma, {
        "CH4": (CH4_SIGMA, CH4_EPS), "CO2_C": CO2_C[:2], "CO2_O": CO2_O[:2]})
    base = Framework(m, pos[:, 0].copy(), pos[:, 1].copy(), pos[:, 2].copy(), species, q, eps,
                     sigma, ids)
    return replicate(base, (reps, reps, reps)) if reps > 1 else base


def random_triclinic_frameworks(count: int, seed: int = 2028, cutoff: float = 12.8,
                                min_atoms: int = 50, max_atoms: int = 2000):
    """Uneven triclinic frameworks (each replicated so that the cutoff fits)."""
    out = []
    stream = 0
    while len(out) < count:
        u = uniforms(seed, 1000 + stream, 0, 8)
        stream += 1
        a, b, c = (10.0 + 30.0 * u[i] for i in range(3))
        al, be, ga = (60.0 + 60.0 * u[3 + i] for i in range(3))
        try:
            m = lattice_from_parameters(a, b, c, al, be, ga)
        except ValueError:
            continue
        vol = abs(float(np.linalg.det(m)))
        if vol < 0.3 * a * b * c:
            continue  # reject strongly degenerate cells
        n_atoms = min_atoms + int(u[6] * (max_atoms - min_atoms + 1))
        n_atoms = min(n_atoms, max(1, int(vol / 8.0)))  # keep the 1 Å separation feasible
        pos, _ = _place_atoms(m, n_atoms, seed, 2000 + stream)
        species = (uniforms(seed, 3000 + stream, 0, n_atoms) * 4).astype(np.uint32)
        fw_eps, fw_sigma = _type_parameters(4, seed, 4000 + stream)
        eps, sigma, ids = _with_guests(fw_eps, fw_sigma, {"CH4": (CH4_SIGMA, CH4_EPS)})
        fw = Framework(m, pos[:, 0].copy(), pos[:, 1].copy(), pos[:, 2].copy(), species,
                       np.zeros(n_atoms), eps, sigma, ids)
        reps = minimum_replication(m, cutoff)
        out.append(replicate(fw, reps) if reps != (1, 1, 1) else fw)
    return out


def ch4_guest(fw: Framework) -> dict:
    return {"x": [0.0], "y": [0.0], "z": [0.0], "lj_species": [fw.guest_species["CH4"]],
            "charge": [0.0]}


def co2_guest(fw: Framework) -> dict:
    """Site order O, C, O along z (bench_gcmc_co2_irmof1.cc:145-148)."""
    o, c = fw.guest_species["CO2_O"], fw.guest_species["CO2_C"]
    return {"x": [0.0, 0.0, 0.0], "y": [0.0, 0.0, 0.0], "z": [-CO2_BOND, 0.0, CO2_BOND],
            "lj_species": [o, c, o], "charge": [CO2_O[2], CO2_C[2], CO2_O[2]]}


def ewald_parameters(m: np.ndarray, rc: float, precision: float = 1e-6):
    """alpha and kMax for a target relative precision eps.

    alpha = sqrt(-ln eps) / rc makes the real-space tail erfc(alpha rc) ~ eps.
    The reciprocal truncation follows the same Gaussian: terms are dropped
    once exp(-k^2 / 4 alpha^2) < eps, i.e. k_max = 2 alpha sqrt(-ln eps), and
    kMax (an index radius) = ceil(k_max * L_max / 2 pi) over the longest
    perpendicular width. (Standard Ewald error estimates, e.g. Kolafa &
    Perram, Mol. Simul. 9 (1992) 351.)
    """
    s = math.sqrt(-math.log(precision))
    alpha = s / rc
    kcut = 2.0 * alpha * s
    lmax = float(perpendicular_widths(m).max())
    kmax = int(math.ceil(kcut * lmax / (2.0 * math.pi)))
    return alpha, kmax
