"""ORACLE — test infrastructure, not product code.

ctypes bindings for the two CPU checkers of the GCMC energy hot path:

* ``Oracle`` binds ``oracle/_build/liboracle.so``, the plain-C FP64
  restatement of the reference algorithms (``oracle/aleator_oracle.c``). It
  travels to every machine and is rebuilt there by ``build_oracle()``.
* ``Reference`` binds ``oracle/_ref/libaleator_ref.so``, the reference
  engine's own hot-path sources compiled by ``oracle/build_ref.sh`` together
  with ``oracle/ref_shim.cc``. It exists only where the reference tree is
  present and is used to pin the restatement and to make the golden fixtures.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this package.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
ORACLE_SO = BUILD / "liboracle.so"
REF_SO = HERE / "_ref" / "libaleator_ref.so"


def _reference_root() -> Path | None:
    """The reference source tree (its sources and test data), present only
    where it was checked out: ALEA_REFERENCE_ROOT, else the tree oracle/_ref
    was last built from (recorded by build_ref.sh); None when neither is set."""
    env = os.environ.get("ALEA_REFERENCE_ROOT")
    if env:
        return Path(env)
    rec = HERE / "_ref" / "source_root"
    if rec.exists():
        return Path(rec.read_text().strip())
    return None


REFERENCE_ROOT = _reference_root()

DRAWS_RIGHT_TO_LEFT = 0
DRAWS_LEFT_TO_RIGHT = 1
TRUNCATED, SHIFTED, LINEAR_FORCE_SHIFTED = 0, 1, 2
LORENTZ_BERTHELOT, GEOMETRIC = 0, 1
COULOMB_K = 167100.9468982874
PASCAL_TO_INTERNAL = 1.0 / (1.380649e-23 * 1.0e30)


def build_oracle(force: bool = False) -> Path:
    """Compile the C restatement (gcc, no FMA contraction, pthreads)."""
    srcs = [HERE / "aleator_oracle.c", HERE / "aleator_oracle_gcmc.c"]
    deps = srcs + [HERE / "aleator_oracle.h", HERE / "aleator_oracle_gcmc.h"]
    if ORACLE_SO.exists() and not force and all(
            ORACLE_SO.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return ORACLE_SO
    BUILD.mkdir(exist_ok=True)
    tmp = ORACLE_SO.with_suffix(f".so.{os.getpid()}")
    subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
                    "-o", str(tmp), *map(str, srcs), "-lm"], check=True)
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_reference(reference_root: str | None = None) -> Path | None:
    """Build oracle/_ref from the reference sources when they are present: the
    tree given, else ALEA_REFERENCE_ROOT, else build_ref.sh's own default."""
    global REFERENCE_ROOT
    root = reference_root or os.environ.get("ALEA_REFERENCE_ROOT")
    if root is not None and not Path(root, "src").is_dir():
        return REF_SO if REF_SO.exists() else None
    subprocess.run(["bash", str(HERE / "build_ref.sh"), *([root] if root else [])], check=True,
                   stdout=subprocess.DEVNULL)
    REFERENCE_ROOT = _reference_root()
    return REF_SO if REF_SO.exists() else None


_D = ctypes.POINTER(ctypes.c_double)
_U32 = ctypes.POINTER(ctypes.c_uint32)
_U64 = ctypes.POINTER(ctypes.c_uint64)
_I32 = ctypes.POINTER(ctypes.c_int)


def _dp(a):
    return None if a is None else a.ctypes.data_as(_D)


def _u32(a):
    return None if a is None else a.ctypes.data_as(_U32)


def _u64(a):
    return None if a is None else a.ctypes.data_as(_U64)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class _LJ(ctypes.Structure):
    _fields_ = [("n_species", ctypes.c_uint32), ("eps", _D), ("sigma", _D),
                ("cutoff", ctypes.c_double), ("truncation", ctypes.c_int), ("mixing", ctypes.c_int)]


class _Species(ctypes.Structure):
    _fields_ = [("n_sites", ctypes.c_uint32), ("x", _D), ("y", _D), ("z", _D),
                ("lj_species", _U32), ("charge", _D)]


class _EwaldParams(ctypes.Structure):
    _fields_ = [("alpha", ctypes.c_double), ("rc", ctypes.c_double), ("kmax", ctypes.c_int)]


class _EwaldState(ctypes.Structure):
    _fields_ = [("m", ctypes.c_double * 9), ("alpha", ctypes.c_double), ("volume", ctypes.c_double),
                ("nk", ctypes.c_uint64), ("k", _D), ("w", _D), ("sre", _D), ("sim", _D),
                ("self_energy", ctypes.c_double), ("exclusion_energy", ctypes.c_double)]


def _mat(m):
    return _f64(np.asarray(m, dtype=np.float64).reshape(9))


class Oracle:
    """The C restatement. Arrays are numpy; lattices are 3x3 row-vector matrices."""

    def __init__(self, path: Path | None = None):
        self.lib = ctypes.CDLL(str(path or build_oracle()))
        L = self.lib
        L.orc_philox_u64.restype = ctypes.c_uint64
        L.orc_philox_u64.argtypes = [ctypes.c_uint64] * 3
        L.orc_philox_uniform.restype = ctypes.c_double
        L.orc_philox_uniform.argtypes = [ctypes.c_uint64] * 3
        L.orc_philox_fill_u64.argtypes = [ctypes.c_uint64] * 4 + [_U64]
        L.orc_philox_fill_uniform.argtypes = [ctypes.c_uint64] * 4 + [_D]
        for name in ("orc_volume",):
            getattr(L, name).restype = ctypes.c_double
            getattr(L, name).argtypes = [_D]
        L.orc_perpendicular_width.restype = ctypes.c_double
        L.orc_perpendicular_width.argtypes = [_D, ctypes.c_int]
        L.orc_min_image.argtypes = [_D, _D, _D, _D]
        L.orc_grid_point_counts.argtypes = [_D, ctypes.c_double, _I32]
        L.orc_grid_build_nodes.argtypes = [ctypes.POINTER(_LJ), _D, ctypes.c_uint64, _D, _D, _D,
                                           _U32, ctypes.c_uint32, ctypes.c_double, ctypes.c_uint64,
                                           ctypes.c_uint64, ctypes.c_int, _D]
        L.orc_grid_interpolate.restype = ctypes.c_double
        L.orc_grid_interpolate.argtypes = [_D, _I32, _D, _D]
        L.orc_lj_particle_energy.restype = ctypes.c_double
        L.orc_lj_particle_energy.argtypes = [ctypes.POINTER(_LJ), _D, ctypes.c_uint64, _D, _D, _D,
                                             _U32, ctypes.c_uint64, _U64, ctypes.c_uint64]
        L.orc_lj_pair_energy.restype = ctypes.c_double
        L.orc_lj_pair_energy.argtypes = [ctypes.POINTER(_LJ), ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double]
        L.orc_lj_tail.restype = ctypes.c_double
        L.orc_lj_tail.argtypes = [ctypes.POINTER(_LJ), _D, ctypes.c_uint64, _U32]
        L.orc_ewald_terms.restype = ctypes.c_uint64
        L.orc_ewald_terms.argtypes = [_D, ctypes.c_double, ctypes.c_int, _D, _D, ctypes.c_uint64]
        L.orc_ewald_real_space_particle_energy.restype = ctypes.c_double
        L.orc_ewald_real_space_particle_energy.argtypes = [
            _D, ctypes.c_uint64, _D, _D, _D, _D, ctypes.c_double, ctypes.c_double,
            ctypes.c_uint64, _U64, ctypes.c_uint64]
        L.orc_ewald_breakdown.argtypes = [_D, ctypes.c_uint64, _D, _D, _D, _D, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_int, _U64, ctypes.c_uint64, _D]
        L.orc_ews_init.argtypes = [ctypes.POINTER(_EwaldState), _D, ctypes.c_double, ctypes.c_int,
                                   ctypes.c_uint64, _D, _D, _D, _D]
        L.orc_ews_free.argtypes = [ctypes.POINTER(_EwaldState)]
        L.orc_ews_energy.restype = ctypes.c_double
        L.orc_ews_energy.argtypes = [ctypes.POINTER(_EwaldState)]
        L.orc_ews_delta.restype = ctypes.c_double
        L.orc_ews_delta.argtypes = [ctypes.POINTER(_EwaldState), _D, ctypes.c_uint64, _D,
                                    ctypes.c_uint64, _D, _D, _D, _D]
        L.orc_ews_commit.argtypes = [ctypes.POINTER(_EwaldState), _D, ctypes.c_uint64, _D,
                                     ctypes.c_uint64]
        L.orc_ews_recompute.restype = ctypes.c_double
        L.orc_ews_recompute.argtypes = [ctypes.POINTER(_EwaldState), ctypes.c_uint64, _D, _D, _D,
                                        _D, ctypes.c_uint64, _U64, _U64]
        L.orc_ews_resync.argtypes = [ctypes.POINTER(_EwaldState), ctypes.c_uint64, _D, _D, _D, _D,
                                     ctypes.c_uint64, _U64, _U64]
        L.orc_widom.restype = ctypes.c_double
        L.orc_widom.argtypes = [ctypes.POINTER(_LJ), ctypes.POINTER(_EwaldParams), _D,
                                ctypes.c_uint64, _D, _D, _D, _D, _U32, ctypes.POINTER(_Species),
                                ctypes.c_double, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                ctypes.c_uint64, ctypes.c_int, ctypes.c_int, _D]
        L.orc_pr_fugacity.restype = ctypes.c_double
        L.orc_pr_fugacity.argtypes = [ctypes.c_double] * 5
        L.orc_pr_mixture.restype = ctypes.c_int
        L.orc_pr_mixture.argtypes = [ctypes.c_uint32, _D, _D, _D, _D, ctypes.c_double,
                                     ctypes.c_double, _D, _D, _D]
        L.orc_random_unit_quaternion.argtypes = [ctypes.c_double] * 3 + [_D]
        L.orc_rotate_by_quaternion.argtypes = [_D, _D, _D]
        self._keep = []

    # ---- Philox
    def philox4x32_10(self, ctr, key):
        c = np.asarray(ctr, dtype=np.uint32)
        k = np.asarray(key, dtype=np.uint32)
        out = np.zeros(4, np.uint32)
        self.lib.orc_philox4x32_10(_u32(c), _u32(k), _u32(out))
        return out

    def philox_u64(self, seed, stream, first, n):
        out = np.zeros(n, np.uint64)
        self.lib.orc_philox_fill_u64(seed, stream, first, n, _u64(out))
        return out

    def philox_uniform(self, seed, stream, first, n):
        out = np.zeros(n, np.float64)
        self.lib.orc_philox_fill_uniform(seed, stream, first, n, _dp(out))
        return out

    # ---- Lattice
    def volume(self, m):
        return self.lib.orc_volume(_dp(_mat(m)))

    def perpendicular_width(self, m, axis):
        return self.lib.orc_perpendicular_width(_dp(_mat(m)), axis)

    def min_image(self, m, a, b):
        mm = _mat(m)
        a = _f64(a).reshape(-1, 3)
        b = _f64(b).reshape(-1, 3)
        out = np.zeros_like(a)
        for i in range(a.shape[0]):
            o = np.zeros(3)
            self.lib.orc_min_image(_dp(mm), _dp(_f64(a[i])), _dp(_f64(b[i])), _dp(o))
            out[i] = o
        return out

    # ---- LJ
    def _lj(self, ff):
        eps = _f64(ff["eps"])
        sig = _f64(ff["sigma"])
        self._keep = [eps, sig]
        return _LJ(len(eps), _dp(eps), _dp(sig), ff["cutoff"], ff.get("truncation", SHIFTED),
                   ff.get("mixing", LORENTZ_BERTHELOT)), (eps, sig)

    def lj_pair_energy(self, ff, r, eps, sigma):
        lj, keep = self._lj(ff)
        return self.lib.orc_lj_pair_energy(ctypes.byref(lj), r, eps, sigma)

    def lj_particle_energy(self, ff, m, x, y, z, species, index, excluded=()):
        lj, keep = self._lj(ff)
        ex = np.asarray(excluded, dtype=np.uint64)
        x, y, z = _f64(x), _f64(y), _f64(z)
        sp = np.ascontiguousarray(species, dtype=np.uint32)
        return self.lib.orc_lj_particle_energy(ctypes.byref(lj), _dp(_mat(m)), len(x), _dp(x),
                                               _dp(y), _dp(z), _u32(sp), index, _u64(ex), len(ex))

    def lj_tail(self, ff, m, species):
        lj, keep = self._lj(ff)
        sp = np.ascontiguousarray(species, dtype=np.uint32)
        return self.lib.orc_lj_tail(ctypes.byref(lj), _dp(_mat(m)), len(sp), _u32(sp))

    # ---- Grid
    def grid_point_counts(self, m, spacing):
        out = np.zeros(3, np.int32)
        self.lib.orc_grid_point_counts(_dp(_mat(m)), spacing, out.ctypes.data_as(_I32))
        return tuple(int(v) for v in out)

    def grid_build(self, ff, m, x, y, z, species, guest, spacing, node_begin=0, node_end=None,
                   threads=1):
        lj, keep = self._lj(ff)
        counts = self.grid_point_counts(m, spacing)
        total = counts[0] * counts[1] * counts[2]
        node_end = total if node_end is None else node_end
        out = np.zeros(node_end - node_begin)
        x, y, z = _f64(x), _f64(y), _f64(z)
        sp = np.ascontiguousarray(species, dtype=np.uint32)
        self.lib.orc_grid_build_nodes(ctypes.byref(lj), _dp(_mat(m)), len(x), _dp(x), _dp(y),
                                      _dp(z), _u32(sp), guest, spacing, node_begin, node_end,
                                      threads, _dp(out))
        return out

    def grid_interpolate(self, m, counts, table, xyz):
        c = np.asarray(counts, dtype=np.int32)
        t = _f64(table)
        mm = _mat(m)
        xyz = _f64(xyz).reshape(-1, 3)
        return np.array([self.lib.orc_grid_interpolate(_dp(mm), c.ctypes.data_as(_I32), _dp(t),
                                                       _dp(_f64(p))) for p in xyz])

    # ---- Ewald
    def ewald_terms(self, m, alpha, kmax):
        mm = _mat(m)
        n = self.lib.orc_ewald_terms(_dp(mm), alpha, kmax, None, None, 0)
        k = np.zeros(3 * n)
        w = np.zeros(n)
        self.lib.orc_ewald_terms(_dp(mm), alpha, kmax, _dp(k), _dp(w), n)
        return k.reshape(n, 3), w

    def ewald_real_space_particle_energy(self, m, x, y, z, q, alpha, rc, index, excluded=()):
        ex = np.asarray(excluded, dtype=np.uint64)
        x, y, z, q = _f64(x), _f64(y), _f64(z), _f64(q)
        return self.lib.orc_ewald_real_space_particle_energy(_dp(_mat(m)), len(x), _dp(x), _dp(y),
                                                             _dp(z), _dp(q), alpha, rc, index,
                                                             _u64(ex), len(ex))

    def ewald_breakdown(self, m, x, y, z, q, alpha, rc, kmax, exclusions=()):
        ex = np.asarray(exclusions, dtype=np.uint64).reshape(-1)
        out = np.zeros(5)
        x, y, z, q = _f64(x), _f64(y), _f64(z), _f64(q)
        self.lib.orc_ewald_breakdown(_dp(_mat(m)), len(x), _dp(x), _dp(y), _dp(z), _dp(q), alpha,
                                     rc, kmax, _u64(ex), len(ex) // 2, _dp(out))
        return out

    def ewald_state(self, m, x, y, z, q, alpha, kmax):
        return OracleEwaldState(self, m, x, y, z, q, alpha, kmax)

    # ---- Widom
    def widom(self, ff, ewald, m, x, y, z, q, species, guest, temperature, seed, stream, n_trials,
              first_trial=0, draw_order=DRAWS_RIGHT_TO_LEFT, threads=1, per_trial=False):
        lj, keep = self._lj(ff)
        ew = _EwaldParams(ewald["alpha"], ewald["rc"], ewald["kmax"]) if ewald else _EwaldParams(0, 0, 0)
        gx, gy, gz = _f64(guest["x"]), _f64(guest["y"]), _f64(guest["z"])
        gs = np.ascontiguousarray(guest["lj_species"], dtype=np.uint32)
        gq = _f64(guest["charge"])
        sp = _Species(len(gx), _dp(gx), _dp(gy), _dp(gz), _u32(gs), _dp(gq))
        x, y, z = _f64(x), _f64(y), _f64(z)
        q = _f64(q if q is not None else np.zeros(len(x)))
        fs = np.ascontiguousarray(species, dtype=np.uint32)
        out = np.zeros(n_trials) if per_trial else None
        kh = self.lib.orc_widom(ctypes.byref(lj), ctypes.byref(ew), _dp(_mat(m)), len(x), _dp(x),
                                _dp(y), _dp(z), _dp(q), _u32(fs), ctypes.byref(sp), temperature,
                                seed, stream, first_trial, n_trials, draw_order, threads, _dp(out))
        return (kh, out) if per_trial else kh

    def pr_fugacity(self, tc, pc, omega, t, p):
        return self.lib.orc_pr_fugacity(tc, pc, omega, t, p)

    def pr_mixture(self, substances, t, p, x, kij=None):
        """(Z, [f_i]) of PengRobinsonMixture; substances = [(tc, pc, omega), ...]."""
        tc, pc, om = (np.ascontiguousarray([s[i] for s in substances], dtype=np.float64)
                      for i in range(3))
        xs = np.ascontiguousarray(x, dtype=np.float64)
        k = None if kij is None else np.ascontiguousarray(kij, dtype=np.float64)
        f = np.zeros(len(substances))
        z = ctypes.c_double()
        rc = self.lib.orc_pr_mixture(len(substances), _dp(tc), _dp(pc), _dp(om),
                                     None if k is None else _dp(k), t, p, _dp(xs),
                                     ctypes.byref(z), _dp(f))
        if rc != 0:
            raise ValueError("PengRobinsonMixture: invalid argument")
        return z.value, f

    def gcmc(self, ff, ewald, m, x, y, z, q, species, guest, temperature, fugacity_pa, seed,
             stream, max_translation=1.5, max_rotation=0.5, draw_order=DRAWS_RIGHT_TO_LEFT,
             grid=None):
        """grid: None, or {"counts": (nx, ny, nz), "tables": {species: table}}
        on this cell (the engine's frameworkEnergyGrid)."""
        return OracleGcmc(self, ff, ewald, m, x, y, z, q, species, guest, temperature,
                          fugacity_pa, seed, stream, max_translation, max_rotation, draw_order,
                          grid)

    def gcmc_mixture(self, ff, ewald, m, x, y, z, q, species, guests, temperature, fugacities_pa,
                     seed, stream, max_translation=1.5, max_rotation=0.5,
                     draw_order=DRAWS_RIGHT_TO_LEFT, grid=None):
        """Several rigid species (the engine's mixture constructor); grid as in gcmc()."""
        return OracleGcmc(self, ff, ewald, m, x, y, z, q, species, list(guests), temperature,
                          list(fugacities_pa), seed, stream, max_translation, max_rotation,
                          draw_order, grid)


class OracleGcmc:
    """Single-species GCMC chain (MonteCarloEngine::run restated in C)."""

    def __init__(self, orc, ff, ewald, m, x, y, z, q, species, guest, temperature, fugacity_pa,
                 seed, stream, max_translation, max_rotation, draw_order, grid=None):
        L = orc.lib
        self.L = L
        L.orc_gcmc_new.restype = ctypes.c_void_p
        L.orc_gcmc_new.argtypes = [ctypes.POINTER(_LJ), ctypes.POINTER(_EwaldParams), _D,
                                   ctypes.c_uint64, _D, _D, _D, _D, _U32, ctypes.POINTER(_Species),
                                   ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int]
        L.orc_gcmc_run.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.orc_gcmc_delete.argtypes = [ctypes.c_void_p]
        L.orc_gcmc_molecules.restype = ctypes.c_uint64
        L.orc_gcmc_molecules.argtypes = [ctypes.c_void_p]
        L.orc_gcmc_particles.restype = ctypes.c_uint64
        L.orc_gcmc_particles.argtypes = [ctypes.c_void_p, _D, ctypes.c_uint64]
        L.orc_gcmc_calls.restype = ctypes.c_uint64
        L.orc_gcmc_calls.argtypes = [ctypes.c_void_p]
        L.orc_gcmc_ewald_energy.restype = ctypes.c_double
        L.orc_gcmc_ewald_energy.argtypes = [ctypes.c_void_p]
        L.orc_gcmc_counters.argtypes = [ctypes.c_void_p, _U64]
        L.orc_gcmc_new_mixture.restype = ctypes.c_void_p
        L.orc_gcmc_new_mixture.argtypes = [ctypes.POINTER(_LJ), ctypes.POINTER(_EwaldParams), _D,
                                           ctypes.c_uint64, _D, _D, _D, _D, _U32, ctypes.c_uint32,
                                           ctypes.POINTER(_Species), ctypes.c_double, _D,
                                           ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                           ctypes.c_uint64, ctypes.c_int]
        lj, keep = orc._lj(ff)
        self._keep = keep
        ew = _EwaldParams(ewald["alpha"], ewald["rc"], ewald["kmax"]) if ewald else _EwaldParams(0, 0, 0)
        guests = guest if isinstance(guest, list) else [guest]
        self._gkeep = []
        sps = (_Species * len(guests))()
        for i, gd in enumerate(guests):
            g = {k: _f64(gd[k]) for k in ("x", "y", "z", "charge")}
            gs = np.ascontiguousarray(gd["lj_species"], dtype=np.uint32)
            self._gkeep.append((g, gs))
            sps[i] = _Species(len(g["x"]), _dp(g["x"]), _dp(g["y"]), _dp(g["z"]), _u32(gs),
                              _dp(g["charge"]))
        x, y, z = _f64(x), _f64(y), _f64(z)
        q = _f64(q if q is not None else np.zeros(len(x)))
        fs = np.ascontiguousarray(species, dtype=np.uint32)
        fug = _f64(np.atleast_1d(fugacity_pa))
        self._fug = fug
        self.h = L.orc_gcmc_new_mixture(ctypes.byref(lj), ctypes.byref(ew), _dp(_mat(m)), len(x),
                                        _dp(x), _dp(y), _dp(z), _dp(q), _u32(fs), len(guests), sps,
                                        temperature, _dp(fug), max_translation, max_rotation, seed,
                                        stream, draw_order)
        if grid is not None:
            L.orc_gcmc_set_grid.argtypes = [ctypes.c_void_p, _I32, ctypes.c_uint32, _U32,
                                            ctypes.POINTER(_D)]
            self._tables = [(int(s), _f64(t)) for s, t in grid["tables"].items()]
            ids = np.array([s for s, _ in self._tables], dtype=np.uint32)
            ptrs = (_D * len(self._tables))(*[_dp(t) for _, t in self._tables])
            counts = np.ascontiguousarray(grid["counts"], dtype=np.int32)
            self._grid_keep = (ids, ptrs, counts)
            L.orc_gcmc_set_grid(self.h, counts.ctypes.data_as(_I32), len(ids), _u32(ids), ptrs)

    def __del__(self):
        try:
            self.L.orc_gcmc_delete(self.h)
        except Exception:
            pass

    def run(self, steps):
        self.L.orc_gcmc_run(self.h, steps)

    def molecules(self):
        return int(self.L.orc_gcmc_molecules(self.h))

    def positions(self):
        n = self.L.orc_gcmc_particles(self.h, None, 0)
        out = np.zeros(3 * n)
        self.L.orc_gcmc_particles(self.h, _dp(out), n)
        return out.reshape(n, 3)

    def calls(self):
        return int(self.L.orc_gcmc_calls(self.h))

    def ewald_energy(self):
        return self.L.orc_gcmc_ewald_energy(self.h)

    def counters(self):
        """attempted[5] then accepted[5]: translate, rotate, insert, delete, swap"""
        out = np.zeros(10, np.uint64)
        self.L.orc_gcmc_counters(self.h, _u64(out))
        return out

    def set_tail(self, on=True):
        """Opt-in: insertions, deletions and swaps add U_tail(after) - U_tail(before)."""
        self.L.orc_gcmc_set_tail.argtypes = [ctypes.c_void_p, ctypes.c_int]
        self.L.orc_gcmc_set_tail(self.h, 1 if on else 0)

    def set_orientation_trials(self, k):
        """Opt-in: orientation-biased insertion and deletion with k trials, in
        the GPU chains' FP64 draw order (no reference counterpart)."""
        self.L.orc_gcmc_set_orientation_trials.argtypes = [ctypes.c_void_p, ctypes.c_int]
        self.L.orc_gcmc_set_orientation_trials(self.h, int(k))

    def molecules_of(self, species):
        self.L.orc_gcmc_molecules_of.restype = ctypes.c_uint64
        self.L.orc_gcmc_molecules_of.argtypes = [ctypes.c_void_p, ctypes.c_uint32]
        return int(self.L.orc_gcmc_molecules_of(self.h, species))


class OracleEwaldState:
    def __init__(self, orc: Oracle, m, x, y, z, q, alpha, kmax):
        self.orc = orc
        self.s = _EwaldState()
        x, y, z, q = _f64(x), _f64(y), _f64(z), _f64(q)
        orc.lib.orc_ews_init(ctypes.byref(self.s), _dp(_mat(m)), alpha, kmax, len(x), _dp(x),
                             _dp(y), _dp(z), _dp(q))

    def __del__(self):
        try:
            self.orc.lib.orc_ews_free(ctypes.byref(self.s))
        except Exception:
            pass

    @property
    def nk(self):
        return int(self.s.nk)

    def energy(self):
        return self.orc.lib.orc_ews_energy(ctypes.byref(self.s))

    def propose(self, removed, added):
        r = _f64(removed).reshape(-1)
        a = _f64(added).reshape(-1)
        return self.orc.lib.orc_ews_delta(ctypes.byref(self.s), _dp(r), len(r) // 4, _dp(a),
                                          len(a) // 4, None, None, None, None)

    def commit(self, removed, added):
        r = _f64(removed).reshape(-1)
        a = _f64(added).reshape(-1)
        self.orc.lib.orc_ews_commit(ctypes.byref(self.s), _dp(r), len(r) // 4, _dp(a), len(a) // 4)

    def _mol(self, molecules):
        offs = np.zeros(len(molecules) + 1, np.uint64)
        for i, mol in enumerate(molecules):
            offs[i + 1] = offs[i] + len(mol)
        idx = np.array([j for mol in molecules for j in mol], dtype=np.uint64)
        if idx.size == 0:
            idx = np.zeros(1, np.uint64)
        return offs, idx

    def recompute(self, x, y, z, q, molecules):
        offs, idx = self._mol(molecules)
        x, y, z, q = _f64(x), _f64(y), _f64(z), _f64(q)
        return self.orc.lib.orc_ews_recompute(ctypes.byref(self.s), len(x), _dp(x), _dp(y), _dp(z),
                                              _dp(q), len(molecules), _u64(offs), _u64(idx))

    def resync(self, x, y, z, q, molecules):
        offs, idx = self._mol(molecules)
        x, y, z, q = _f64(x), _f64(y), _f64(z), _f64(q)
        self.orc.lib.orc_ews_resync(ctypes.byref(self.s), len(x), _dp(x), _dp(y), _dp(z), _dp(q),
                                    len(molecules), _u64(offs), _u64(idx))

    def raw(self):
        n = self.nk
        sre = np.ctypeslib.as_array(self.s.sre, shape=(n,)).copy() if n else np.zeros(0)
        sim = np.ctypeslib.as_array(self.s.sim, shape=(n,)).copy() if n else np.zeros(0)
        return np.concatenate([sre, sim, [self.s.self_energy, self.s.exclusion_energy]])


class Reference:
    """The reference engine's own code (oracle/_ref). Raises if not built."""

    def __init__(self, path: Path | None = None):
        p = path or REF_SO
        if not Path(p).exists():
            raise FileNotFoundError(f"{p} not built (oracle/build_ref.sh needs the reference tree)")
        self.lib = ctypes.CDLL(str(p))
        L = self.lib
        L.ref_philox_u64.argtypes = [ctypes.c_uint64] * 4 + [_U64]
        L.ref_philox_uniform.argtypes = [ctypes.c_uint64] * 4 + [_D]
        L.ref_min_image.argtypes = [_D, _D, _D, ctypes.c_uint64, _D]
        L.ref_perpendicular_width.restype = ctypes.c_double
        L.ref_perpendicular_width.argtypes = [_D, ctypes.c_int]
        L.ref_grid_create.restype = ctypes.c_void_p
        L.ref_grid_create.argtypes = [_D, ctypes.c_uint64, _D, _D, _D, _U32, ctypes.c_uint32, _D, _D,
                                      ctypes.c_double, ctypes.c_int, ctypes.c_int, _U32,
                                      ctypes.c_uint32, ctypes.c_double]
        L.ref_grid_counts.argtypes = [ctypes.c_void_p, _I32]
        L.ref_grid_interpolate.argtypes = [ctypes.c_void_p, ctypes.c_uint32, _D, ctypes.c_uint64, _D]
        L.ref_grid_serialize.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _D, ctypes.c_uint64, _D,
                                         _D, _D, _U32, ctypes.c_uint32, _D, _D, ctypes.c_double,
                                         ctypes.c_int, ctypes.c_int, _U32, ctypes.c_uint32,
                                         ctypes.c_double]
        L.ref_grid_cache_name.argtypes = [ctypes.c_char_p, ctypes.c_uint64, _D, ctypes.c_uint64, _D,
                                          _D, _D, _U32, ctypes.c_uint32, _D, _D, ctypes.c_double,
                                          ctypes.c_int, ctypes.c_int, _U32, ctypes.c_uint32,
                                          ctypes.c_double]
        L.ref_grid_destroy.argtypes = [ctypes.c_void_p]
        L.ref_lj_particle_energy.argtypes = [_D, ctypes.c_uint64, _D, _D, _D, _U32, ctypes.c_uint32,
                                             _D, _D, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                             _U64, ctypes.c_uint64, _U64, ctypes.c_uint64, _D]
        L.ref_lj_energy_virial.argtypes = [_D, ctypes.c_uint64, _D, _D, _D, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_double, ctypes.c_int, _D]
        L.ref_lj_tail.restype = ctypes.c_double
        L.ref_lj_tail.argtypes = [_D, ctypes.c_uint64, _U32, ctypes.c_uint32, _D, _D,
                                  ctypes.c_double, ctypes.c_int]
        L.ref_ewald_terms.restype = ctypes.c_uint64
        L.ref_ewald_terms.argtypes = [_D, ctypes.c_double, ctypes.c_int, _D, _D, ctypes.c_uint64]
        L.ref_ewald_breakdown.argtypes = [_D, ctypes.c_uint64, _D, _D, _D, _D, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_int, _U64, ctypes.c_uint64,
                                          ctypes.c_double, _D]
        L.ref_ewald_real_space_particle_energy.argtypes = [
            _D, ctypes.c_uint64, _D, _D, _D, _D, ctypes.c_double, ctypes.c_double, _U64,
            ctypes.c_uint64, _U64, ctypes.c_uint64, _D]
        L.ref_ews_create.restype = ctypes.c_void_p
        L.ref_ews_create.argtypes = [_D, ctypes.c_uint64, _D, _D, _D, _D, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_int]
        L.ref_ews_energy.restype = ctypes.c_double
        L.ref_ews_energy.argtypes = [ctypes.c_void_p]
        L.ref_ews_propose.restype = ctypes.c_double
        L.ref_ews_propose.argtypes = [ctypes.c_void_p, _D, ctypes.c_uint64, _D, ctypes.c_uint64]
        L.ref_ews_commit.argtypes = [ctypes.c_void_p, _D, ctypes.c_uint64, _D, ctypes.c_uint64]
        L.ref_ews_recompute.restype = ctypes.c_double
        L.ref_ews_recompute.argtypes = [ctypes.c_void_p, ctypes.c_uint64, _D, _D, _D, _D,
                                        ctypes.c_uint64, _U64, _U64]
        L.ref_ews_resync.argtypes = [ctypes.c_void_p, ctypes.c_uint64, _D, _D, _D, _D,
                                     ctypes.c_uint64, _U64, _U64]
        L.ref_ews_raw.restype = ctypes.c_uint64
        L.ref_ews_raw.argtypes = [ctypes.c_void_p, _D, ctypes.c_uint64]
        L.ref_ews_destroy.argtypes = [ctypes.c_void_p]
        L.ref_widom.argtypes = [_D, ctypes.c_uint64, _D, _D, _D, _D, _U32, ctypes.c_uint32, _D, _D,
                                ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                ctypes.c_double, ctypes.c_int, ctypes.c_uint32, _D, _D, _D, _U32,
                                _D, ctypes.c_double, ctypes.c_uint64, ctypes.c_uint64,
                                ctypes.c_uint64, _D, _D, ctypes.c_int]
        L.ref_gcmc_create.restype = ctypes.c_void_p
        L.ref_gcmc_create.argtypes = [_D, ctypes.c_uint64, _D, _D, _D, _D, _U32, ctypes.c_uint32,
                                      _D, _D, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                      ctypes.c_uint32, _D, _D, _D, _U32, _D, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_uint64, ctypes.c_uint64]
        L.ref_gcmc_create_grid.restype = ctypes.c_void_p
        L.ref_gcmc_create_grid.argtypes = L.ref_gcmc_create.argtypes + [ctypes.c_double,
                                                                          ctypes.c_uint32, _U32]
        L.ref_gcmc_create_mixture.restype = ctypes.c_void_p
        L.ref_gcmc_create_mixture.argtypes = [_D, ctypes.c_uint64, _D, _D, _D, _D, _U32,
                                              ctypes.c_uint32, _D, _D, ctypes.c_double, ctypes.c_int,
                                              ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                              ctypes.c_int, ctypes.c_uint32, _U32, _D, _D, _D, _U32,
                                              _D, _D, ctypes.c_double, ctypes.c_double,
                                              ctypes.c_double, ctypes.c_uint64, ctypes.c_uint64,
                                              ctypes.c_double, ctypes.c_uint32, _U32]
        L.ref_gcmc_molecules_of.restype = ctypes.c_uint64
        L.ref_gcmc_molecules_of.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.ref_gcmc_run.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.ref_gcmc_molecules.restype = ctypes.c_uint64
        L.ref_gcmc_molecules.argtypes = [ctypes.c_void_p]
        L.ref_gcmc_particles.restype = ctypes.c_uint64
        L.ref_gcmc_particles.argtypes = [ctypes.c_void_p, _D, ctypes.c_uint64]
        L.ref_gcmc_ewald_energy.restype = ctypes.c_double
        L.ref_gcmc_ewald_energy.argtypes = [ctypes.c_void_p]
        L.ref_gcmc_ewald_drift.restype = ctypes.c_double
        L.ref_gcmc_ewald_drift.argtypes = [ctypes.c_void_p]
        L.ref_gcmc_destroy.argtypes = [ctypes.c_void_p]
        L.ref_pr_fugacity.restype = ctypes.c_double
        L.ref_pr_fugacity.argtypes = [ctypes.c_double] * 5
        L.ref_read_cif.restype = ctypes.c_void_p
        L.ref_read_cif.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]
        L.ref_structure_size.restype = ctypes.c_uint64
        L.ref_structure_size.argtypes = [ctypes.c_void_p]
        L.ref_structure_species.restype = ctypes.c_uint32
        L.ref_structure_species.argtypes = [ctypes.c_void_p]
        L.ref_structure_atoms.argtypes = [ctypes.c_void_p] + [_D] * 6 + [_U32, _D]
        L.ref_structure_symbol.restype = ctypes.c_char_p
        L.ref_structure_symbol.argtypes = [ctypes.c_void_p, ctypes.c_uint32]
        L.ref_structure_label.restype = ctypes.c_char_p
        L.ref_structure_label.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.ref_structure_free.argtypes = [ctypes.c_void_p]
        L.ref_pr_mixture.restype = ctypes.c_int
        L.ref_pr_mixture.argtypes = [ctypes.c_uint32, _D, _D, _D, _D, ctypes.c_double,
                                     ctypes.c_double, _D, _D, _D, ctypes.c_char_p, ctypes.c_size_t]

    def philox4x32_10(self, ctr, key):
        c = np.asarray(ctr, dtype=np.uint32)
        k = np.asarray(key, dtype=np.uint32)
        out = np.zeros(4, np.uint32)
        self.lib.ref_philox4x32_10(_u32(c), _u32(k), _u32(out))
        return out

    def philox_u64(self, seed, stream, first, n):
        out = np.zeros(n, np.uint64)
        self.lib.ref_philox_u64(seed, stream, first, n, _u64(out))
        return out

    def philox_uniform(self, seed, stream, first, n):
        out = np.zeros(n, np.float64)
        self.lib.ref_philox_uniform(seed, stream, first, n, _dp(out))
        return out

    def min_image(self, m, a, b):
        a = _f64(a).reshape(-1, 3)
        b = _f64(b).reshape(-1, 3)
        out = np.zeros_like(a)
        self.lib.ref_min_image(_dp(_mat(m)), _dp(a), _dp(b), a.shape[0], _dp(out))
        return out

    def perpendicular_width(self, m, axis):
        return self.lib.ref_perpendicular_width(_dp(_mat(m)), axis)

    def _grid_args(self, ff, m, x, y, z, species, guests, spacing):
        eps, sig = _f64(ff["eps"]), _f64(ff["sigma"])
        x, y, z = _f64(x), _f64(y), _f64(z)
        sp = np.ascontiguousarray(species, dtype=np.uint32)
        g = np.ascontiguousarray(guests, dtype=np.uint32)
        keep = (eps, sig, x, y, z, sp, g, _mat(m))
        args = (_dp(keep[7]), len(x), _dp(x), _dp(y), _dp(z), _u32(sp), len(eps), _dp(eps), _dp(sig),
                ff["cutoff"], ff.get("truncation", SHIFTED), ff.get("mixing", LORENTZ_BERTHELOT),
                _u32(g), len(g), spacing)
        return args, keep

    def grid(self, ff, m, x, y, z, species, guests, spacing):
        return ReferenceGrid(self, ff, m, x, y, z, species, guests, spacing)

    def lj_particle_energy(self, ff, m, x, y, z, species, queries, excluded=()):
        eps, sig = _f64(ff["eps"]), _f64(ff["sigma"])
        x, y, z = _f64(x), _f64(y), _f64(z)
        sp = np.ascontiguousarray(species, dtype=np.uint32)
        qq = np.asarray(queries, dtype=np.uint64)
        ex = np.asarray(excluded, dtype=np.uint64)
        out = np.zeros(len(qq))
        self.lib.ref_lj_particle_energy(_dp(_mat(m)), len(x), _dp(x), _dp(y), _dp(z), _u32(sp),
                                        len(eps), _dp(eps), _dp(sig), ff["cutoff"],
                                        ff.get("truncation", SHIFTED),
                                        ff.get("mixing", LORENTZ_BERTHELOT), _u64(qq), len(qq),
                                        _u64(ex), len(ex), _dp(out))
        return out

    def lj_energy_virial(self, m, x, y, z, eps, sigma, cutoff, truncation):
        out = np.zeros(3)
        x, y, z = _f64(x), _f64(y), _f64(z)
        self.lib.ref_lj_energy_virial(_dp(_mat(m)), len(x), _dp(x), _dp(y), _dp(z), eps, sigma,
                                      cutoff, truncation, _dp(out))
        return out

    def lj_tail(self, ff, m, species):
        eps, sig = _f64(ff["eps"]), _f64(ff["sigma"])
        sp = np.ascontiguousarray(species, dtype=np.uint32)
        return self.lib.ref_lj_tail(_dp(_mat(m)), len(sp), _u32(sp), len(eps), _dp(eps), _dp(sig),
                                    ff["cutoff"], ff.get("mixing", LORENTZ_BERTHELOT))

    def ewald_terms(self, m, alpha, kmax):
        mm = _mat(m)
        n = self.lib.ref_ewald_terms(_dp(mm), alpha, kmax, None, None, 0)
        k = np.zeros(3 * n)
        w = np.zeros(n)
        self.lib.ref_ewald_terms(_dp(mm), alpha, kmax, _dp(k), _dp(w), n)
        return k.reshape(n, 3), w

    def ewald_breakdown(self, m, x, y, z, q, alpha, rc, kmax, exclusions=(), skin=0.3):
        ex = np.asarray(exclusions, dtype=np.uint64).reshape(-1)
        out = np.zeros(5)
        x, y, z, q = _f64(x), _f64(y), _f64(z), _f64(q)
        self.lib.ref_ewald_breakdown(_dp(_mat(m)), len(x), _dp(x), _dp(y), _dp(z), _dp(q), alpha,
                                     rc, kmax, _u64(ex), len(ex) // 2, skin, _dp(out))
        return out

    def ewald_real_space_particle_energy(self, m, x, y, z, q, alpha, rc, queries, excluded=()):
        qq = np.asarray(queries, dtype=np.uint64)
        ex = np.asarray(excluded, dtype=np.uint64)
        out = np.zeros(len(qq))
        x, y, z, q = _f64(x), _f64(y), _f64(z), _f64(q)
        self.lib.ref_ewald_real_space_particle_energy(_dp(_mat(m)), len(x), _dp(x), _dp(y), _dp(z),
                                                      _dp(q), alpha, rc, _u64(qq), len(qq),
                                                      _u64(ex), len(ex), _dp(out))
        return out

    def ewald_state(self, m, x, y, z, q, alpha, kmax):
        return ReferenceEwaldState(self, m, x, y, z, q, alpha, kmax)

    def widom(self, ff, ewald, m, x, y, z, q, species, guest, temperature, seed, stream, n_trials,
              draw_order=DRAWS_RIGHT_TO_LEFT, per_trial=False):
        eps, sig = _f64(ff["eps"]), _f64(ff["sigma"])
        x, y, z = _f64(x), _f64(y), _f64(z)
        q = _f64(q if q is not None else np.zeros(len(x)))
        sp = np.ascontiguousarray(species, dtype=np.uint32)
        gx, gy, gz = _f64(guest["x"]), _f64(guest["y"]), _f64(guest["z"])
        gs = np.ascontiguousarray(guest["lj_species"], dtype=np.uint32)
        gq = _f64(guest["charge"])
        alpha = ewald["alpha"] if ewald else 0.0
        erc = ewald["rc"] if ewald else 0.0
        kmax = ewald["kmax"] if ewald else 0
        out = np.zeros(n_trials) if per_trial else None
        kh = np.zeros(2)
        self.lib.ref_widom(_dp(_mat(m)), len(x), _dp(x), _dp(y), _dp(z), _dp(q), _u32(sp), len(eps),
                           _dp(eps), _dp(sig), ff["cutoff"], ff.get("truncation", SHIFTED),
                           ff.get("mixing", LORENTZ_BERTHELOT), alpha, erc, kmax, len(gx), _dp(gx),
                           _dp(gy), _dp(gz), _u32(gs), _dp(gq), temperature, seed, stream,
                           n_trials, _dp(out), _dp(kh),
                           1 if draw_order == DRAWS_RIGHT_TO_LEFT else 0)
        return (kh, out) if per_trial else kh[0]

    def pr_fugacity(self, tc, pc, omega, t, p):
        return self.lib.ref_pr_fugacity(tc, pc, omega, t, p)

    def read_cif(self, path):
        """The reference's readCif: a dict of lattice, x, y, z, charge, mass,
        species, occupancy, symbols, labels; its exception message raised as
        RuntimeError."""
        L = self.lib
        msg = ctypes.create_string_buffer(1024)
        h = L.ref_read_cif(os.fsencode(str(path)), msg, 1024)
        if not h:
            raise RuntimeError(msg.value.decode())
        try:
            n = L.ref_structure_size(h)
            m = np.zeros(9)
            x, y, z, q, mass, occ = (np.zeros(n) for _ in range(6))
            sp = np.zeros(n, np.uint32)
            L.ref_structure_atoms(h, _dp(m), _dp(x), _dp(y), _dp(z), _dp(q), _dp(mass),
                                  sp.ctypes.data_as(_U32), _dp(occ))
            return dict(lattice=m.reshape(3, 3), x=x, y=y, z=z, charge=q, mass=mass, species=sp,
                        occupancy=occ,
                        symbols=[L.ref_structure_symbol(h, k).decode()
                                 for k in range(L.ref_structure_species(h))],
                        labels=[L.ref_structure_label(h, i).decode() for i in range(n)])
        finally:
            L.ref_structure_free(h)

    def pr_mixture(self, substances, t, p, x, kij=None):
        """(Z, [f_i]) from the reference's PengRobinsonMixture; its exception
        message raised as ValueError."""
        tc, pc, om = (np.ascontiguousarray([s[i] for s in substances], dtype=np.float64)
                      for i in range(3))
        xs = np.ascontiguousarray(x, dtype=np.float64)
        k = None if kij is None else np.ascontiguousarray(kij, dtype=np.float64)
        f = np.zeros(len(substances))
        z = ctypes.c_double()
        msg = ctypes.create_string_buffer(512)
        rc = self.lib.ref_pr_mixture(len(substances), _dp(tc), _dp(pc), _dp(om),
                                     None if k is None else _dp(k), t, p, _dp(xs),
                                     ctypes.byref(z), _dp(f), msg, 512)
        if rc != 0:
            raise ValueError(msg.value.decode())
        return z.value, f

    def gcmc(self, ff, ewald, m, x, y, z, q, species, guest, temperature, fugacity_pa, seed,
             stream, max_translation=1.5, max_rotation=0.5, grid=None):
        """grid: None, or {"spacing": s, "species": [...]}: the engine gets the
        reference's FrameworkEnergyGrid of those guest species."""
        return ReferenceGcmc(self, ff, ewald, m, x, y, z, q, species, guest, temperature,
                             fugacity_pa, seed, stream, max_translation, max_rotation, grid)

    def gcmc_mixture(self, ff, ewald, m, x, y, z, q, species, guests, temperature, fugacities_pa,
                     seed, stream, max_translation=1.5, max_rotation=0.5, grid=None):
        """The engine's mixture constructor (several rigid species); grid as in gcmc()."""
        return ReferenceGcmc(self, ff, ewald, m, x, y, z, q, species, list(guests), temperature,
                             list(fugacities_pa), seed, stream, max_translation, max_rotation,
                             grid)


class ReferenceGcmc:
    """MonteCarloEngine (the reference's own class) driven through the shim."""

    def __init__(self, ref, ff, ewald, m, x, y, z, q, species, guest, temperature, fugacity_pa,
                 seed, stream, max_translation, max_rotation, grid=None):
        self.ref = ref
        eps, sig = _f64(ff["eps"]), _f64(ff["sigma"])
        x, y, z = _f64(x), _f64(y), _f64(z)
        q = _f64(q if q is not None else np.zeros(len(x)))
        sp = np.ascontiguousarray(species, dtype=np.uint32)
        mixture = isinstance(guest, list)
        guests = guest if mixture else [guest]
        gx = _f64(np.concatenate([np.asarray(g["x"], float) for g in guests]))
        gy = _f64(np.concatenate([np.asarray(g["y"], float) for g in guests]))
        gz = _f64(np.concatenate([np.asarray(g["z"], float) for g in guests]))
        gs = np.ascontiguousarray(np.concatenate([np.asarray(g["lj_species"]) for g in guests]),
                                  dtype=np.uint32)
        gq = _f64(np.concatenate([np.asarray(g["charge"], float) for g in guests]))
        per = np.array([len(g["x"]) for g in guests], dtype=np.uint32)
        alpha = ewald["alpha"] if ewald else 0.0
        erc = ewald["rc"] if ewald else 0.0
        kmax = ewald["kmax"] if ewald else 0
        self._keep = (gx, gy, gz, gs, gq, per)
        args = [_dp(_mat(m)), len(x), _dp(x), _dp(y), _dp(z), _dp(q), _u32(sp), len(eps), _dp(eps),
                _dp(sig), ff["cutoff"], ff.get("truncation", SHIFTED),
                ff.get("mixing", LORENTZ_BERTHELOT), alpha, erc, kmax, len(gx), _dp(gx), _dp(gy),
                _dp(gz), _u32(gs), _dp(gq), temperature, fugacity_pa, max_translation,
                max_rotation, seed, stream]
        if mixture:
            fug = _f64(np.asarray(fugacity_pa, float))
            gids = np.ascontiguousarray(grid["species"] if grid is not None else [0], dtype=np.uint32)
            gids = gids if grid is not None else gids[:0]
            self._keep = self._keep + (fug, gids)
            self.h = ref.lib.ref_gcmc_create_mixture(
                _dp(_mat(m)), len(x), _dp(x), _dp(y), _dp(z), _dp(q), _u32(sp), len(eps), _dp(eps),
                _dp(sig), ff["cutoff"], ff.get("truncation", SHIFTED),
                ff.get("mixing", LORENTZ_BERTHELOT), alpha, erc, kmax, len(guests), _u32(per),
                _dp(gx), _dp(gy), _dp(gz), _u32(gs), _dp(gq), _dp(fug), temperature,
                max_translation, max_rotation, seed, stream,
                grid["spacing"] if grid is not None else 0.0, len(gids), _u32(gids))
        elif grid is None:
            self.h = ref.lib.ref_gcmc_create(*args)
        else:
            ids = np.ascontiguousarray(grid["species"], dtype=np.uint32)
            self.h = ref.lib.ref_gcmc_create_grid(*args, grid["spacing"], len(ids), _u32(ids))

    def __del__(self):
        try:
            self.ref.lib.ref_gcmc_destroy(self.h)
        except Exception:
            pass

    def run(self, steps):
        self.ref.lib.ref_gcmc_run(self.h, steps)

    def molecules(self):
        return int(self.ref.lib.ref_gcmc_molecules(self.h))

    def molecules_of(self, species):
        return int(self.ref.lib.ref_gcmc_molecules_of(self.h, species))

    def positions(self):
        n = self.ref.lib.ref_gcmc_particles(self.h, None, 0)
        out = np.zeros(3 * n)
        self.ref.lib.ref_gcmc_particles(self.h, _dp(out), n)
        return out.reshape(n, 3)

    def ewald_energy(self):
        return self.ref.lib.ref_gcmc_ewald_energy(self.h)


class ReferenceGrid:
    def __init__(self, ref: Reference, ff, m, x, y, z, species, guests, spacing):
        self.ref = ref
        self.args, self._keep = ref._grid_args(ff, m, x, y, z, species, guests, spacing)
        self.h = ref.lib.ref_grid_create(*self.args)
        c = np.zeros(3, np.int32)
        ref.lib.ref_grid_counts(self.h, c.ctypes.data_as(_I32))
        self.counts = tuple(int(v) for v in c)

    def __del__(self):
        try:
            self.ref.lib.ref_grid_destroy(self.h)
        except Exception:
            pass

    def interpolate(self, species, xyz):
        xyz = _f64(xyz).reshape(-1, 3)
        out = np.zeros(xyz.shape[0])
        self.ref.lib.ref_grid_interpolate(self.h, species, _dp(xyz), xyz.shape[0], _dp(out))
        return out

    def serialize(self, path):
        self.ref.lib.ref_grid_serialize(self.h, str(path).encode(), *self.args)

    def cache_name(self):
        buf = ctypes.create_string_buffer(512)
        self.ref.lib.ref_grid_cache_name(buf, 512, *self.args)
        return buf.value.decode()


class ReferenceEwaldState:
    def __init__(self, ref: Reference, m, x, y, z, q, alpha, kmax):
        self.ref = ref
        x, y, z, q = _f64(x), _f64(y), _f64(z), _f64(q)
        self.h = ref.lib.ref_ews_create(_dp(_mat(m)), len(x), _dp(x), _dp(y), _dp(z), _dp(q),
                                        alpha, 1.0, kmax)

    def __del__(self):
        try:
            self.ref.lib.ref_ews_destroy(self.h)
        except Exception:
            pass

    def energy(self):
        return self.ref.lib.ref_ews_energy(self.h)

    def propose(self, removed, added):
        r = _f64(removed).reshape(-1)
        a = _f64(added).reshape(-1)
        return self.ref.lib.ref_ews_propose(self.h, _dp(r), len(r) // 4, _dp(a), len(a) // 4)

    def commit(self, removed, added):
        r = _f64(removed).reshape(-1)
        a = _f64(added).reshape(-1)
        self.ref.lib.ref_ews_commit(self.h, _dp(r), len(r) // 4, _dp(a), len(a) // 4)

    def _mol(self, molecules):
        offs = np.zeros(len(molecules) + 1, np.uint64)
        for i, mol in enumerate(molecules):
            offs[i + 1] = offs[i] + len(mol)
        idx = np.array([j for mol in molecules for j in mol], dtype=np.uint64)
        if idx.size == 0:
            idx = np.zeros(1, np.uint64)
        return offs, idx

    def recompute(self, x, y, z, q, molecules):
        offs, idx = self._mol(molecules)
        x, y, z, q = _f64(x), _f64(y), _f64(z), _f64(q)
        return self.ref.lib.ref_ews_recompute(self.h, len(x), _dp(x), _dp(y), _dp(z), _dp(q),
                                              len(molecules), _u64(offs), _u64(idx))

    def resync(self, x, y, z, q, molecules):
        offs, idx = self._mol(molecules)
        x, y, z, q = _f64(x), _f64(y), _f64(z), _f64(q)
        self.ref.lib.ref_ews_resync(self.h, len(x), _dp(x), _dp(y), _dp(z), _dp(q), len(molecules),
                                    _u64(offs), _u64(idx))

    def raw(self):
        n = self.ref.lib.ref_ews_raw(self.h, None, 0)
        out = np.zeros(n)
        self.ref.lib.ref_ews_raw(self.h, _dp(out), n)
        return out
