"""ctypes binding of libaleator_gb300.so and the reference-shaped Python API."""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libaleator_gb300.so"

TRUNCATED, SHIFTED, LINEAR_FORCE_SHIFTED = 0, 1, 2
LORENTZ_BERTHELOT, GEOMETRIC = 0, 1
FP64, FP32 = 0, 1
ALEA_DRAWS_RIGHT_TO_LEFT, ALEA_DRAWS_LEFT_TO_RIGHT = 0, 1

_STATUS_EXC = {1: ValueError, 2: IndexError, 3: RuntimeError}


class AleatorError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


_D = ctypes.POINTER(ctypes.c_double)
_U32 = ctypes.POINTER(ctypes.c_uint32)
_U64 = ctypes.POINTER(ctypes.c_uint64)
_I32 = ctypes.POINTER(ctypes.c_int32)
_VP = ctypes.c_void_p


_F = ctypes.POINTER(ctypes.c_float)
SAMPLE_ROW = 5  # floats per training row {s0, s1, s2, -dU/T, lq} (ALEA_SAMPLE_ROW)


class _ProposalConfig(ctypes.Structure):
    _fields_ = [("n_freq", ctypes.c_uint32), ("width", ctypes.c_uint32), ("depth", ctypes.c_uint32),
                ("freq_max", ctypes.c_uint32), ("seed", ctypes.c_uint64)]


class _TrainConfig(ctypes.Structure):
    _fields_ = [("epochs", ctypes.c_uint32), ("batch", ctypes.c_uint32), ("lr", ctypes.c_double),
                ("tau", ctypes.c_double), ("beta1", ctypes.c_double), ("beta2", ctypes.c_double),
                ("eps", ctypes.c_double), ("seed", ctypes.c_uint64)]


class _Lattice(ctypes.Structure):
    _fields_ = [("m", ctypes.c_double * 9)]


class _LJ(ctypes.Structure):
    _fields_ = [("n_species", ctypes.c_uint32), ("epsilon", _D), ("sigma", _D),
                ("cutoff", ctypes.c_double), ("truncation", ctypes.c_int32),
                ("mixing", ctypes.c_int32)]


class _Ewald(ctypes.Structure):
    _fields_ = [("alpha", ctypes.c_double), ("real_space_cutoff", ctypes.c_double),
                ("kmax", ctypes.c_int32)]


class _Particles(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint64), ("x", _D), ("y", _D), ("z", _D), ("charge", _D),
                ("species", _U32)]


class _Species(ctypes.Structure):
    _fields_ = [("n_sites", ctypes.c_uint32), ("x", _D), ("y", _D), ("z", _D),
                ("lj_species", _U32), ("charge", _D)]


class _GridStats(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_uint64), ("algorithmic_pairs", ctypes.c_uint64),
                ("executed_pairs", ctypes.c_uint64), ("images", ctypes.c_uint64),
                ("bricks", ctypes.c_uint64), ("last_kernel_ms", ctypes.c_float),
                ("launches", ctypes.c_uint32)]


class _GridBatchStats(ctypes.Structure):
    _fields_ = [("grids", ctypes.c_uint32), ("nodes", ctypes.c_uint64),
                ("algorithmic_pairs", ctypes.c_uint64), ("executed_pairs", ctypes.c_uint64),
                ("bricks", ctypes.c_uint64), ("last_ms", ctypes.c_float), ("variant", ctypes.c_int32),
                ("tune_ms", ctypes.c_float * 2), ("graph_launches", ctypes.c_uint32)]


class _ChainInfo(ctypes.Structure):
    _fields_ = [("molecules", ctypes.c_uint64), ("guest_sites", ctypes.c_uint64),
                ("call_index", ctypes.c_uint64), ("steps", ctypes.c_uint64),
                ("resyncs", ctypes.c_uint64), ("attempted", ctypes.c_uint64 * 5),
                ("accepted", ctypes.c_uint64 * 5), ("species_molecules", ctypes.c_uint64 * 4),
                ("sum_molecules", ctypes.c_double),
                ("sum_molecules_sq", ctypes.c_double), ("last_du", ctypes.c_double),
                ("last_kernel_ms", ctypes.c_float)]


class _WidomResult(ctypes.Structure):
    _fields_ = [("henry", ctypes.c_double), ("log_mean_weight", ctypes.c_double),
                ("rel_std_error", ctypes.c_double), ("n_trials", ctypes.c_uint64),
                ("kernel_ms", ctypes.c_float)]


_SIGNATURES = {
    "alea_last_error": (ctypes.c_size_t, [ctypes.c_char_p, ctypes.c_size_t]),
    "alea_status_string": (ctypes.c_char_p, [ctypes.c_int32]),
    "alea_version": (ctypes.c_int32, [_I32, _I32, _I32]),
    "alea_device_info": (ctypes.c_int32, [ctypes.c_char_p, ctypes.c_size_t, _I32, _I32, _I32]),
    "alea_probe_fp32_fma_tflops": (ctypes.c_int32, [_D]),
    "alea_probe_fp32x2_fma_tflops": (ctypes.c_int32, [_D]),
    "alea_test_ff_near": (ctypes.c_int32, [ctypes.c_int32, _D, _D, ctypes.c_uint64, ctypes.c_double]),
    "alea_cached_bytes": (ctypes.c_int32, [_U64]),
    "alea_release_cached": (ctypes.c_int32, [_U64]),
    "alea_test_block_cache": (ctypes.c_int32, []),
    "alea_philox4x32_10": (ctypes.c_int32, [_U32, _U32, _U32, ctypes.c_uint64]),
    "alea_philox_fill_u64": (ctypes.c_int32, [ctypes.c_uint64] * 4 + [_U64]),
    "alea_philox_fill_uniform": (ctypes.c_int32, [ctypes.c_uint64] * 4 + [_D]),
    "alea_philox_fill_u64_device": (ctypes.c_int32, [ctypes.c_uint64] * 4 + [_VP, _VP]),
    "alea_philox_fill_uniform_device": (ctypes.c_int32, [ctypes.c_uint64] * 4 + [_VP, _VP]),
    "alea_grid_build": (ctypes.c_int32, [ctypes.POINTER(_LJ), ctypes.POINTER(_Particles),
                                         ctypes.POINTER(_Lattice), _U32, ctypes.c_uint32,
                                         ctypes.c_double, ctypes.c_int32, ctypes.POINTER(_VP)]),
    "alea_grid_point_counts": (ctypes.c_int32, [_VP, _I32]),
    "alea_grid_spacing": (ctypes.c_int32, [_VP, _D]),
    "alea_grid_species": (ctypes.c_int32, [_VP, _U32, ctypes.c_uint32, _U32]),
    "alea_grid_interpolate": (ctypes.c_int32, [_VP, ctypes.c_uint32, _D, ctypes.c_uint64, _D]),
    "alea_grid_interpolate_device": (ctypes.c_int32, [_VP, ctypes.c_uint32, _VP, ctypes.c_uint64,
                                                      _VP, _VP]),
    "alea_grid_download": (ctypes.c_int32, [_VP, ctypes.c_uint32, _D, ctypes.c_uint64]),
    "alea_grid_table_device": (ctypes.c_int32, [_VP, ctypes.c_uint32, ctypes.POINTER(_VP)]),
    "alea_grid_rebuild": (ctypes.c_int32, [_VP, _VP]),
    "alea_grid_stats_get": (ctypes.c_int32, [_VP, ctypes.POINTER(_GridStats)]),
    "alea_grid_serialize": (ctypes.c_int32, [_VP, ctypes.c_char_p, ctypes.POINTER(_LJ),
                                             ctypes.POINTER(_Particles), ctypes.POINTER(_Lattice),
                                             _U32, ctypes.c_uint32]),
    "alea_grid_cache_file_name": (ctypes.c_int32, [ctypes.POINTER(_LJ), ctypes.POINTER(_Particles),
                                                   ctypes.POINTER(_Lattice), _U32, ctypes.c_uint32,
                                                   ctypes.c_double, ctypes.c_char_p,
                                                   ctypes.c_size_t]),
    "alea_test_grid_tile_wait_limit": (ctypes.c_int32, [ctypes.c_int64]),
    "alea_grid_cache_hit": (ctypes.c_int32, [ctypes.c_char_p, ctypes.POINTER(_LJ),
                                             ctypes.POINTER(_Particles), ctypes.POINTER(_Lattice),
                                             _U32, ctypes.c_uint32, ctypes.c_double, _I32]),
    "alea_grid_load_cache": (ctypes.c_int32, [ctypes.c_char_p, ctypes.POINTER(_LJ),
                                              ctypes.POINTER(_Particles), ctypes.POINTER(_Lattice),
                                              _U32, ctypes.c_uint32, ctypes.c_double,
                                              ctypes.POINTER(_VP)]),
    "alea_grid_destroy": (ctypes.c_int32, [_VP]),
    "alea_lj_particle_energy": (ctypes.c_int32, [ctypes.POINTER(_LJ), ctypes.POINTER(_Particles),
                                                 ctypes.POINTER(_Lattice), _U64, ctypes.c_uint64,
                                                 _U64, ctypes.c_uint64, _D]),
    "alea_lj_tail_correction": (ctypes.c_int32, [ctypes.POINTER(_LJ), ctypes.POINTER(_Particles),
                                                 ctypes.POINTER(_Lattice), _D]),
    "alea_ewald_reciprocal_terms": (ctypes.c_int32, [ctypes.POINTER(_Lattice), ctypes.c_double,
                                                     ctypes.c_int32, _D, _D, ctypes.c_uint64,
                                                     _U64]),
    "alea_ewald_real_space_particle_energy": (ctypes.c_int32, [
        ctypes.POINTER(_Ewald), ctypes.POINTER(_Particles), ctypes.POINTER(_Lattice), _U64,
        ctypes.c_uint64, _U64, ctypes.c_uint64, _D]),
    "alea_ewald_energy_breakdown": (ctypes.c_int32, [ctypes.POINTER(_Ewald),
                                                     ctypes.POINTER(_Particles),
                                                     ctypes.POINTER(_Lattice), _U64,
                                                     ctypes.c_uint64, _D]),
    "alea_ewald_state_create": (ctypes.c_int32, [ctypes.POINTER(_Ewald), ctypes.POINTER(_Particles),
                                                 ctypes.POINTER(_Lattice), ctypes.POINTER(_VP)]),
    "alea_ewald_state_committed_energy": (ctypes.c_int32, [_VP, _D]),
    "alea_ewald_state_propose": (ctypes.c_int32, [_VP, _D, ctypes.c_uint64, _D, ctypes.c_uint64,
                                                  _D]),
    "alea_ewald_state_commit": (ctypes.c_int32, [_VP, _D, ctypes.c_uint64, _D, ctypes.c_uint64]),
    "alea_ewald_state_recompute": (ctypes.c_int32, [_VP, ctypes.POINTER(_Particles),
                                                    ctypes.c_uint64, _U64, _U64, _D]),
    "alea_ewald_state_resync": (ctypes.c_int32, [_VP, ctypes.POINTER(_Particles), ctypes.c_uint64,
                                                 _U64, _U64]),
    "alea_ewald_state_raw": (ctypes.c_int32, [_VP, _D, ctypes.c_uint64, _U64]),
    "alea_ewald_state_term_count": (ctypes.c_int32, [_VP, _U64]),
    "alea_ewald_state_destroy": (ctypes.c_int32, [_VP]),
    "alea_ewald_propose_no_alloc": (ctypes.c_int32, [_VP, _VP, _VP, _VP, ctypes.c_uint64,
                                                     ctypes.c_double, ctypes.POINTER(_Lattice), _D,
                                                     ctypes.c_uint64, _D, ctypes.c_uint64, _VP,
                                                     _VP]),
    "alea_widom_create": (ctypes.c_int32, [ctypes.POINTER(_LJ), ctypes.POINTER(_Ewald),
                                           ctypes.POINTER(_Particles), ctypes.POINTER(_Lattice),
                                           ctypes.POINTER(_Species), ctypes.c_double,
                                           ctypes.c_int32, ctypes.POINTER(_VP)]),
    "alea_widom_run": (ctypes.c_int32, [_VP, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                        ctypes.c_uint64, ctypes.c_int32,
                                        ctypes.POINTER(_WidomResult), _D]),
    "alea_widom_destroy": (ctypes.c_int32, [_VP]),
    "alea_widom_samples": (ctypes.c_int32, [_VP, _VP, ctypes.c_uint64, ctypes.c_uint64,
                                            ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int32, _VP]),
    "alea_widom_run_biased": (ctypes.c_int32, [_VP, _VP, ctypes.c_uint64, ctypes.c_uint64,
                                               ctypes.c_uint64, ctypes.c_uint64,
                                               ctypes.POINTER(_WidomResult), _D, _D]),
    "alea_proposal_create": (ctypes.c_int32, [ctypes.POINTER(_ProposalConfig),
                                              ctypes.POINTER(_VP)]),
    "alea_proposal_param_count": (ctypes.c_int32, [_VP, _U64]),
    "alea_proposal_wave_vectors": (ctypes.c_int32, [_VP, _I32, ctypes.c_uint64]),
    "alea_proposal_get_params": (ctypes.c_int32, [_VP, _F, ctypes.c_uint64]),
    "alea_proposal_set_params": (ctypes.c_int32, [_VP, _F, ctypes.c_uint64]),
    "alea_proposal_forward": (ctypes.c_int32, [_VP, _F, ctypes.c_uint64, _F]),
    "alea_proposal_loss_grad": (ctypes.c_int32, [_VP, _F, ctypes.c_uint64, ctypes.c_double, _D,
                                                 _F, ctypes.c_uint64]),
    "alea_proposal_train": (ctypes.c_int32, [_VP, _VP, ctypes.c_uint64,
                                             ctypes.POINTER(_TrainConfig), _D, _VP]),
    "alea_proposal_tabulate": (ctypes.c_int32, [_VP, ctypes.c_uint32, ctypes.c_double]),
    "alea_proposal_log_density": (ctypes.c_int32, [_VP, _D, ctypes.c_uint64, _D]),
    "alea_proposal_destroy": (ctypes.c_int32, [_VP]),
    "alea_gcmc_create": (ctypes.c_int32, [ctypes.POINTER(_LJ), ctypes.POINTER(_Ewald),
                                          ctypes.POINTER(_Particles), ctypes.POINTER(_Lattice),
                                          ctypes.POINTER(_Species), ctypes.c_double, _D, _U64, _U64,
                                          ctypes.c_uint32, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_int32, ctypes.c_uint32, ctypes.POINTER(_VP)]),
    "alea_gcmc_create_mixture": (ctypes.c_int32, [ctypes.POINTER(_LJ), ctypes.POINTER(_Ewald),
                                                  ctypes.POINTER(_Particles), ctypes.POINTER(_Lattice),
                                                  ctypes.c_uint32, ctypes.POINTER(_Species),
                                                  ctypes.c_double, _D, _U64, _U64, ctypes.c_uint32,
                                                  ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                                  ctypes.c_uint32, ctypes.POINTER(_VP)]),
    "alea_gcmc_run": (ctypes.c_int32, [_VP, ctypes.c_uint64, _VP]),
    "alea_gcmc_chain_info_get": (ctypes.c_int32, [_VP, ctypes.c_uint32, ctypes.POINTER(_ChainInfo)]),
    "alea_gcmc_particles": (ctypes.c_int32, [_VP, ctypes.c_uint32, _D, ctypes.c_uint64, _U64]),
    "alea_gcmc_ewald_energy": (ctypes.c_int32, [_VP, ctypes.c_uint32, _D]),
    "alea_gcmc_destroy": (ctypes.c_int32, [_VP]),
    "alea_gcmc_set_proposal": (ctypes.c_int32, [_VP, _VP]),
    "alea_gcmc_set_precision": (ctypes.c_int32, [_VP, ctypes.c_int32]),
    "alea_gcmc_set_grid": (ctypes.c_int32, [_VP, _VP]),
    "alea_gcmc_set_tail_correction": (ctypes.c_int32, [_VP, ctypes.c_int32]),
    "alea_gcmc_set_orientation_trials": (ctypes.c_int32, [_VP, ctypes.c_int32]),
    "alea_widom_set_tail_correction": (ctypes.c_int32, [_VP, ctypes.c_int32, _D]),
    "alea_gcmc_guest_sites": (ctypes.c_int32, [_VP, ctypes.c_uint32, _D, ctypes.POINTER(ctypes.c_uint32),
                                               ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]),
    "alea_grid_batch_create": (ctypes.c_int32, [ctypes.c_uint32, ctypes.POINTER(_LJ),
                                                ctypes.POINTER(_Particles), ctypes.POINTER(_Lattice),
                                                _U32, ctypes.c_uint32, ctypes.c_double,
                                                ctypes.POINTER(_VP)]),
    "alea_grid_batch_build": (ctypes.c_int32, [_VP, _VP]),
    "alea_grid_batch_stats_get": (ctypes.c_int32, [_VP, ctypes.POINTER(_GridBatchStats)]),
    "alea_grid_batch_point_counts": (ctypes.c_int32, [_VP, ctypes.c_uint32, _I32]),
    "alea_grid_batch_download": (ctypes.c_int32, [_VP, ctypes.c_uint32, ctypes.c_uint32, _D,
                                                  ctypes.c_uint64]),
    "alea_grid_batch_destroy": (ctypes.c_int32, [_VP]),
    "alea_widom_batch_create": (ctypes.c_int32, [ctypes.c_uint32, ctypes.POINTER(_LJ),
                                                 ctypes.POINTER(_Ewald), ctypes.POINTER(_Particles),
                                                 ctypes.POINTER(_Lattice), ctypes.POINTER(_Species),
                                                 ctypes.c_double, ctypes.c_int32,
                                                 ctypes.POINTER(_VP)]),
    "alea_widom_batch_run": (ctypes.c_int32, [_VP, _U64, _U64, ctypes.c_uint64, ctypes.c_uint64,
                                              ctypes.c_int32, ctypes.POINTER(_WidomResult), _VP]),
    "alea_widom_batch_destroy": (ctypes.c_int32, [_VP]),
    "alea_insertion_ratio": (ctypes.c_double, [ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                               ctypes.c_double, ctypes.c_double]),
    "alea_deletion_ratio": (ctypes.c_double, [ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                              ctypes.c_double, ctypes.c_double]),
    "alea_metropolis_ratio": (ctypes.c_double, [ctypes.c_double, ctypes.c_double]),
    "alea_swap_ratio": (ctypes.c_double, [ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                          ctypes.c_uint64, ctypes.c_double, ctypes.c_double]),
    "alea_peng_robinson_fugacity": (ctypes.c_int32, [ctypes.c_double] * 5 + [_D]),
    "alea_grid_build_to_host": (ctypes.c_int32, [ctypes.POINTER(_LJ), ctypes.POINTER(_Particles),
                                                 ctypes.POINTER(_Lattice), _U32, ctypes.c_uint32,
                                                 ctypes.c_double, ctypes.c_int32,
                                                 ctypes.POINTER(_D), ctypes.POINTER(_VP)]),
    "alea_read_cif": (ctypes.c_int32, [ctypes.c_char_p, ctypes.POINTER(_VP)]),
    "alea_structure_sizes": (ctypes.c_int32, [_VP, _U64, _U32]),
    "alea_structure_lattice": (ctypes.c_int32, [_VP, _D]),
    "alea_structure_atoms": (ctypes.c_int32, [_VP, _D, _D, _D, _D, _D, _U32, _D]),
    "alea_structure_species_symbol": (ctypes.c_int32, [_VP, ctypes.c_uint32, ctypes.c_char_p,
                                                       ctypes.c_size_t]),
    "alea_structure_source_label": (ctypes.c_int32, [_VP, ctypes.c_uint64, ctypes.c_char_p,
                                                     ctypes.c_size_t]),
    "alea_structure_destroy": (ctypes.c_int32, [_VP]),
    "alea_peng_robinson_mixture": (ctypes.c_int32, [ctypes.c_uint32, _D, _D, _D, _D,
                                                    ctypes.c_double, ctypes.c_double, _D, _D, _D]),
}

_LIB = None


def load_library(path: str | os.PathLike | None = None, build_if_missing: bool = False):
    """Loads libaleator_gb300.so (raising if absent) and declares every signature."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists() and build_if_missing:
        from .build import build
        build()
    if not p.exists():
        raise FileNotFoundError(
            f"{p} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def library():
    return load_library()


def _check(status: int):
    if status == 0:
        return
    lib = library()
    buf = ctypes.create_string_buffer(4096)
    lib.alea_last_error(buf, 4096)
    msg = buf.value.decode(errors="replace")
    exc = _STATUS_EXC.get(status)
    if exc is not None:
        raise exc(msg)
    raise AleatorError(status, msg)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _dp(a):
    return None if a is None else a.ctypes.data_as(_D)


def _u32p(a):
    return None if a is None else a.ctypes.data_as(_U32)


def _u64p(a):
    return None if a is None else a.ctypes.data_as(_U64)


def _lattice(m) -> _Lattice:
    arr = _f64(np.asarray(m, dtype=np.float64).reshape(9))
    out = _Lattice()
    for i in range(9):
        out.m[i] = arr[i]
    return out


class ParticleData:
    """core::ParticleData SoA (core/math/particle_data.hpp:20-25)."""

    def __init__(self, x, y, z, charge=None, species=None):
        self.x, self.y, self.z = _f64(x), _f64(y), _f64(z)
        n = self.x.shape[0]
        self.charge = _f64(charge) if charge is not None else np.zeros(n)
        self.species = (np.ascontiguousarray(species, dtype=np.uint32) if species is not None
                        else np.zeros(n, np.uint32))

    @classmethod
    def from_framework(cls, fw):
        return cls(fw.x, fw.y, fw.z, fw.charge, fw.species)

    def __len__(self):
        return int(self.x.shape[0])

    def c(self) -> _Particles:
        return _Particles(len(self), _dp(self.x), _dp(self.y), _dp(self.z), _dp(self.charge),
                          _u32p(self.species))


class LennardJones:
    """LennardJones(perSpecies, cutoff, truncation, mixing) (lennard_jones.hpp:64-66)."""

    def __init__(self, epsilon, sigma, cutoff, truncation=TRUNCATED, mixing=LORENTZ_BERTHELOT):
        self.epsilon = _f64(epsilon)
        self.sigma = _f64(sigma)
        self.cutoff = float(cutoff)
        self.truncation = int(truncation)
        self.mixing = int(mixing)

    def c(self) -> _LJ:
        return _LJ(len(self.epsilon), _dp(self.epsilon), _dp(self.sigma), self.cutoff,
                   self.truncation, self.mixing)


class Ewald:
    """Ewald(alpha, realSpaceCutoff, kMax) (ewald.hpp:76-77)."""

    def __init__(self, alpha, real_space_cutoff, kmax):
        self.alpha = float(alpha)
        self.real_space_cutoff = float(real_space_cutoff)
        self.kmax = int(kmax)

    def c(self) -> _Ewald:
        return _Ewald(self.alpha, self.real_space_cutoff, self.kmax)


# ---------------------------------------------------------------- Philox
def philox4x32_10(ctr, key):
    ctr = np.ascontiguousarray(np.asarray(ctr, dtype=np.uint32).reshape(-1, 4))
    key = np.ascontiguousarray(np.asarray(key, dtype=np.uint32).reshape(-1, 2))
    out = np.zeros_like(ctr)
    _check(library().alea_philox4x32_10(_u32p(ctr), _u32p(key), _u32p(out), ctr.shape[0]))
    return out


def philox_u64(seed, stream, first, n):
    out = np.zeros(n, np.uint64)
    _check(library().alea_philox_fill_u64(seed, stream, first, n, _u64p(out)))
    return out


def philox_uniform(seed, stream, first, n):
    out = np.zeros(n, np.float64)
    _check(library().alea_philox_fill_uniform(seed, stream, first, n, _dp(out)))
    return out


def device_info():
    name = ctypes.create_string_buffer(256)
    sms, ma, mi = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    _check(library().alea_device_info(name, 256, ctypes.byref(sms), ctypes.byref(ma),
                                      ctypes.byref(mi)))
    return {"name": name.value.decode(), "sm_count": sms.value, "cc": (ma.value, mi.value)}


def fp32_fma_tflops(packed: bool = False):
    """Sustained FP32 FMA throughput measured on the current device: scalar
    fmaf, or (packed=True) the two-lane fma.rn.f32x2 the grid sweep issues."""
    v = ctypes.c_double()
    fn = library().alea_probe_fp32x2_fma_tflops if packed else library().alea_probe_fp32_fma_tflops
    _check(fn(ctypes.byref(v)))
    return v.value


# ---------------------------------------------------------------- grid
class FrameworkEnergyGrid:
    """FrameworkEnergyGrid (engines/monte_carlo/framework_energy_grid.hpp:94-200) on the GPU."""

    def __init__(self, force_field: LennardJones, framework: ParticleData, lattice,
                 guest_species_ids, spacing_angstrom: float, precision: int = FP64, *,
                 _handle=None):
        self._lib = library()
        self._keep = (force_field, framework)
        self.lattice = np.asarray(lattice, dtype=np.float64).reshape(3, 3).copy()
        self._ff = force_field
        self._fw = framework
        self._guests = np.ascontiguousarray(guest_species_ids, dtype=np.uint32)
        self._h = _VP()
        if _handle is not None:
            self._h = _handle
        else:
            lj = force_field.c()
            p = framework.c()
            lat = _lattice(lattice)
            _check(self._lib.alea_grid_build(ctypes.byref(lj), ctypes.byref(p), ctypes.byref(lat),
                                             _u32p(self._guests), len(self._guests),
                                             float(spacing_angstrom), int(precision),
                                             ctypes.byref(self._h)))

    @classmethod
    def build_to_host(cls, force_field: LennardJones, framework: ParticleData, lattice,
                      guest_species_ids, spacing_angstrom: float, precision: int, host_ptrs,
                      keep: bool = True):
        """The constructor with every table copied to host memory as the build
        goes (alea_grid_build_to_host): host_ptrs[k] is the address of a host
        array of point-count-product doubles for guest_species_ids[k] (pinned
        memory lets the copies overlap the build). Returns the grid, or None
        when keep is False."""
        lib = library()
        lj = force_field.c()
        p = framework.c()
        lat = _lattice(lattice)
        guests = np.ascontiguousarray(guest_species_ids, dtype=np.uint32)
        ptrs = (_D * len(guests))(*[ctypes.cast(int(a), _D) for a in host_ptrs])
        h = _VP()
        _check(lib.alea_grid_build_to_host(ctypes.byref(lj), ctypes.byref(p), ctypes.byref(lat),
                                           _u32p(guests), len(guests), float(spacing_angstrom),
                                           int(precision), ptrs, ctypes.byref(h) if keep else None))
        if not keep:
            return None
        return cls(force_field, framework, lattice, guest_species_ids, spacing_angstrom, precision,
                   _handle=h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                self._lib.alea_grid_destroy(h)
            except Exception:
                pass
            self._h = None

    def point_counts(self):
        out = np.zeros(3, np.int32)
        _check(self._lib.alea_grid_point_counts(self._h, out.ctypes.data_as(_I32)))
        return tuple(int(v) for v in out)

    def spacing_angstrom(self):
        v = ctypes.c_double()
        _check(self._lib.alea_grid_spacing(self._h, ctypes.byref(v)))
        return v.value

    def species(self):
        n = ctypes.c_uint32()
        _check(self._lib.alea_grid_species(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, np.uint32)
        _check(self._lib.alea_grid_species(self._h, _u32p(out), n.value, ctypes.byref(n)))
        return [int(v) for v in out]

    def interpolate(self, species: int, positions):
        xyz = _f64(np.asarray(positions, dtype=np.float64).reshape(-1, 3))
        out = np.zeros(xyz.shape[0])
        _check(self._lib.alea_grid_interpolate(self._h, int(species), _dp(xyz), xyz.shape[0],
                                               _dp(out)))
        return out

    def interpolate_device(self, species: int, xyz_ptr: int, n: int, out_ptr: int, stream=0):
        _check(self._lib.alea_grid_interpolate_device(self._h, int(species), xyz_ptr, n, out_ptr,
                                                      stream))

    def table(self, species: int):
        nx, ny, nz = self.point_counts()
        out = np.zeros(nx * ny * nz)
        _check(self._lib.alea_grid_download(self._h, int(species), _dp(out), out.size))
        return out

    def download_into(self, species: int, out: np.ndarray):
        _check(self._lib.alea_grid_download(self._h, int(species), _dp(out), out.size))

    def rebuild(self, stream=0):
        _check(self._lib.alea_grid_rebuild(self._h, stream))

    def stats(self):
        s = _GridStats()
        _check(self._lib.alea_grid_stats_get(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def serialize(self, path):
        lj = self._ff.c()
        p = self._fw.c()
        lat = _lattice(self.lattice)
        _check(self._lib.alea_grid_serialize(self._h, str(path).encode(), ctypes.byref(lj),
                                             ctypes.byref(p), ctypes.byref(lat),
                                             _u32p(self._guests), len(self._guests)))

    @staticmethod
    def cache_file_name(force_field, framework, lattice, guest_species_ids, spacing):
        g = np.ascontiguousarray(guest_species_ids, dtype=np.uint32)
        lj = force_field.c()
        p = framework.c()
        lat = _lattice(lattice)
        buf = ctypes.create_string_buffer(512)
        _check(library().alea_grid_cache_file_name(ctypes.byref(lj), ctypes.byref(p),
                                                   ctypes.byref(lat), _u32p(g), len(g),
                                                   float(spacing), buf, 512))
        return buf.value.decode()

    @classmethod
    def load_from_cache(cls, cache_dir, force_field, framework, lattice, guest_species_ids,
                        spacing):
        g = np.ascontiguousarray(guest_species_ids, dtype=np.uint32)
        lj = force_field.c()
        p = framework.c()
        lat = _lattice(lattice)
        h = _VP()
        _check(library().alea_grid_load_cache(str(cache_dir).encode(), ctypes.byref(lj),
                                              ctypes.byref(p), ctypes.byref(lat), _u32p(g), len(g),
                                              float(spacing), ctypes.byref(h)))
        if not h:
            return None
        return cls(force_field, framework, lattice, g, spacing, _handle=h)

    @staticmethod
    def cache_hit(cache_dir, force_field, framework, lattice, guest_species_ids, spacing):
        """cacheHit (framework_energy_grid.cc:326-352): True when the key's file
        exists and matches, False when none is there; AleatorError (a
        RuntimeError) when a file at that path has another version or key."""
        g = np.ascontiguousarray(guest_species_ids, dtype=np.uint32)
        lj = force_field.c()
        p = framework.c()
        lat = _lattice(lattice)
        hit = ctypes.c_int32(0)
        _check(library().alea_grid_cache_hit(str(cache_dir).encode(), ctypes.byref(lj),
                                             ctypes.byref(p), ctypes.byref(lat), _u32p(g), len(g),
                                             float(spacing), ctypes.byref(hit)))
        return bool(hit.value)

    @classmethod
    def load_or_build(cls, cache_dir, force_field, framework, lattice, guest_species_ids,
                      spacing, precision=FP64):
        """loadOrBuildFrameworkEnergyGrid (framework_energy_grid.cc:411-435):
        the cached grid when the key's file is there, else a fresh build written
        to the cache. Returns (grid, was_hit)."""
        grid = cls.load_from_cache(cache_dir, force_field, framework, lattice, guest_species_ids,
                                   spacing)
        if grid is not None:
            return grid, True
        grid = cls(force_field, framework, lattice, guest_species_ids, spacing, precision)
        name = cls.cache_file_name(force_field, framework, lattice, guest_species_ids, spacing)
        grid.serialize(os.path.join(str(cache_dir), name))
        return grid, False


# ---------------------------------------------------------------- LJ / Ewald free functions
def lj_particle_energy(force_field: LennardJones, particles: ParticleData, lattice, queries,
                       excluded=()):
    q = np.ascontiguousarray(queries, dtype=np.uint64)
    ex = np.ascontiguousarray(excluded, dtype=np.uint64)
    out = np.zeros(len(q))
    lj = force_field.c()
    p = particles.c()
    lat = _lattice(lattice)
    _check(library().alea_lj_particle_energy(ctypes.byref(lj), ctypes.byref(p), ctypes.byref(lat),
                                             _u64p(q), len(q), _u64p(ex), len(ex), _dp(out)))
    return out


def lj_tail_correction(force_field: LennardJones, particles: ParticleData, lattice):
    v = ctypes.c_double()
    lj = force_field.c()
    p = particles.c()
    lat = _lattice(lattice)
    _check(library().alea_lj_tail_correction(ctypes.byref(lj), ctypes.byref(p), ctypes.byref(lat),
                                             ctypes.byref(v)))
    return v.value


def ewald_reciprocal_terms(lattice, alpha, kmax):
    lat = _lattice(lattice)
    n = ctypes.c_uint64()
    _check(library().alea_ewald_reciprocal_terms(ctypes.byref(lat), alpha, kmax, None, None, 0,
                                                 ctypes.byref(n)))
    k = np.zeros(3 * n.value)
    w = np.zeros(n.value)
    _check(library().alea_ewald_reciprocal_terms(ctypes.byref(lat), alpha, kmax, _dp(k), _dp(w),
                                                 n.value, ctypes.byref(n)))
    return k.reshape(-1, 3), w


def ewald_real_space_particle_energy(ewald: Ewald, particles: ParticleData, lattice, queries,
                                     excluded=()):
    q = np.ascontiguousarray(queries, dtype=np.uint64)
    ex = np.ascontiguousarray(excluded, dtype=np.uint64)
    out = np.zeros(len(q))
    e = ewald.c()
    p = particles.c()
    lat = _lattice(lattice)
    _check(library().alea_ewald_real_space_particle_energy(ctypes.byref(e), ctypes.byref(p),
                                                           ctypes.byref(lat), _u64p(q), len(q),
                                                           _u64p(ex), len(ex), _dp(out)))
    return out


def ewald_energy_breakdown(ewald: Ewald, particles: ParticleData, lattice, exclusions=()):
    ex = np.ascontiguousarray(np.asarray(exclusions, dtype=np.uint64).reshape(-1))
    out = np.zeros(5)
    e = ewald.c()
    p = particles.c()
    lat = _lattice(lattice)
    _check(library().alea_ewald_energy_breakdown(ctypes.byref(e), ctypes.byref(p),
                                                 ctypes.byref(lat), _u64p(ex), len(ex) // 2,
                                                 _dp(out)))
    return out


def _sites(s):
    s = _f64(np.asarray(s, dtype=np.float64).reshape(-1))
    if s.size % 4:
        raise ValueError("sites must be packed {x, y, z, q}")
    return s, s.size // 4


class EwaldIncrementalState:
    """EwaldIncrementalState (ewald_incremental_state.hpp:70-171) with S(k) in HBM."""

    def __init__(self, ewald: Ewald, particles: ParticleData, lattice):
        self._lib = library()
        self._h = _VP()
        e = ewald.c()
        p = particles.c()
        lat = _lattice(lattice)
        _check(self._lib.alea_ewald_state_create(ctypes.byref(e), ctypes.byref(p),
                                                 ctypes.byref(lat), ctypes.byref(self._h)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                self._lib.alea_ewald_state_destroy(h)
            except Exception:
                pass
            self._h = None

    def committed_energy(self):
        v = ctypes.c_double()
        _check(self._lib.alea_ewald_state_committed_energy(self._h, ctypes.byref(v)))
        return v.value

    def propose(self, removed, added):
        r, nr = _sites(removed)
        a, na = _sites(added)
        v = ctypes.c_double()
        _check(self._lib.alea_ewald_state_propose(self._h, _dp(r), nr, _dp(a), na,
                                                  ctypes.byref(v)))
        return v.value

    def commit(self, removed, added):
        r, nr = _sites(removed)
        a, na = _sites(added)
        _check(self._lib.alea_ewald_state_commit(self._h, _dp(r), nr, _dp(a), na))

    def propose_move(self, old, new):
        return self.propose(old, new)

    def propose_insertion(self, new):
        return self.propose(np.zeros((0, 4)), new)

    def propose_deletion(self, existing):
        return self.propose(existing, np.zeros((0, 4)))

    def commit_move(self, old, new):
        self.commit(old, new)

    def commit_insertion(self, new):
        self.commit(np.zeros((0, 4)), new)

    def commit_deletion(self, existing):
        self.commit(existing, np.zeros((0, 4)))

    @staticmethod
    def _csr(molecules):
        offs = np.zeros(len(molecules) + 1, np.uint64)
        for i, m in enumerate(molecules):
            offs[i + 1] = offs[i] + len(m)
        idx = np.array([j for m in molecules for j in m], dtype=np.uint64)
        return offs, (idx if idx.size else np.zeros(1, np.uint64))

    def recompute_from_scratch(self, particles: ParticleData, molecules):
        offs, idx = self._csr(molecules)
        p = particles.c()
        v = ctypes.c_double()
        _check(self._lib.alea_ewald_state_recompute(self._h, ctypes.byref(p), len(molecules),
                                                    _u64p(offs), _u64p(idx), ctypes.byref(v)))
        return v.value

    def resync(self, particles: ParticleData, molecules):
        offs, idx = self._csr(molecules)
        p = particles.c()
        _check(self._lib.alea_ewald_state_resync(self._h, ctypes.byref(p), len(molecules),
                                                 _u64p(offs), _u64p(idx)))

    def raw_state_for_testing(self):
        n = ctypes.c_uint64()
        _check(self._lib.alea_ewald_state_raw(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value)
        _check(self._lib.alea_ewald_state_raw(self._h, _dp(out), n.value, ctypes.byref(n)))
        return out

    def term_count(self):
        n = ctypes.c_uint64()
        _check(self._lib.alea_ewald_state_term_count(self._h, ctypes.byref(n)))
        return n.value


# ---------------------------------------------------------------- Widom
class Widom:
    """Device context for MonteCarloEngine::widomInsertionHenryCoefficient
    (monte_carlo_engine.cc:850-917)."""

    def __init__(self, force_field: LennardJones, framework: ParticleData, lattice, guest: dict,
                 temperature: float, ewald: Ewald | None = None, precision: int = FP64):
        self._lib = library()
        self._h = _VP()
        self._g = {k: (_f64(guest[k]) if k != "lj_species" else
                       np.ascontiguousarray(guest[k], dtype=np.uint32))
                   for k in ("x", "y", "z", "lj_species", "charge")}
        sp = _Species(len(self._g["x"]), _dp(self._g["x"]), _dp(self._g["y"]), _dp(self._g["z"]),
                      _u32p(self._g["lj_species"]), _dp(self._g["charge"]))
        lj = force_field.c()
        p = framework.c()
        lat = _lattice(lattice)
        e = ewald.c() if ewald is not None else None
        _check(self._lib.alea_widom_create(ctypes.byref(lj), ctypes.byref(e) if e else None,
                                           ctypes.byref(p), ctypes.byref(lat), ctypes.byref(sp),
                                           float(temperature), int(precision),
                                           ctypes.byref(self._h)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                self._lib.alea_widom_destroy(h)
            except Exception:
                pass
            self._h = None

    def run(self, seed, stream, n_trials, first_trial=0, draw_order=ALEA_DRAWS_RIGHT_TO_LEFT,
            per_trial=False):
        res = _WidomResult()
        out = np.zeros(n_trials) if per_trial else None
        _check(self._lib.alea_widom_run(self._h, seed, stream, first_trial, n_trials, draw_order,
                                        ctypes.byref(res), _dp(out)))
        r = {f: getattr(res, f) for f, _ in res._fields_}
        return (r, out) if per_trial else r

    def set_tail_correction(self, on=True):
        """Opt-in: every trial's deltaU gains U_tail(framework + molecule) -
        U_tail(framework); returns that constant (K)."""
        v = ctypes.c_double()
        _check(self._lib.alea_widom_set_tail_correction(self._h, 1 if on else 0, ctypes.byref(v)))
        return v.value

    def henry_coefficient(self, seed, stream, n_trials, draw_order=ALEA_DRAWS_RIGHT_TO_LEFT):
        return self.run(seed, stream, n_trials, draw_order=draw_order)["henry"]

    def samples(self, seed, stream, n_trials, out_device_ptr, first_trial=0,
                draw_order=ALEA_DRAWS_RIGHT_TO_LEFT, proposal=None):
        """Trials as training rows {s0, s1, s2, -dU/T, lq} (float32, SAMPLE_ROW per
        trial) written to a device buffer: uniform trials (lq = 0), or drawn from
        a tabulated proposal (lq = its log density at the position)."""
        _check(self._lib.alea_widom_samples(self._h, proposal._h if proposal else None, seed,
                                            stream, first_trial, n_trials, draw_order,
                                            out_device_ptr))

    def run_biased(self, proposal, seed, stream, n_trials, first_trial=0, per_trial=False):
        """Insertions drawn from the tabulated learned proposal; the weights are
        exp(-dU/T)/p(s), so `henry` estimates the same K_H as run()."""
        res = _WidomResult()
        du = np.zeros(n_trials) if per_trial else None
        fr = np.zeros((n_trials, 3)) if per_trial else None
        _check(self._lib.alea_widom_run_biased(self._h, proposal._h, seed, stream, first_trial,
                                               n_trials, ctypes.byref(res), _dp(du), _dp(fr)))
        r = {f: getattr(res, f) for f, _ in res._fields_}
        return (r, du, fr) if per_trial else r


class GridBatch:
    """Many independent FP32 energy grids (each framework with its own force
    field, atoms and cell) built together: one persistent launch per kernel,
    replayed from a CUDA graph captured after an autotuning first build."""

    def __init__(self, force_fields, frameworks, lattices, guests, spacing):
        self._lib = library()
        self._h = _VP()
        n = len(frameworks)
        assert len(force_fields) == n and len(lattices) == n and len(guests) == n
        self._keep = [ff for ff in force_fields] + list(frameworks)
        ljs = (_LJ * n)(*[ff.c() for ff in force_fields])
        ps = (_Particles * n)(*[p.c() for p in frameworks])
        lats = (_Lattice * n)(*[_lattice(m) for m in lattices])
        ng = len(guests[0])
        g = np.ascontiguousarray(np.asarray(guests, dtype=np.uint32).reshape(n, ng))
        self._lists = (ljs, ps, lats, g)
        _check(self._lib.alea_grid_batch_create(n, ljs, ps, lats, _u32p(g), ng, float(spacing),
                                                ctypes.byref(self._h)))
        self.n = n
        self.guests = g

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                self._lib.alea_grid_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    def build(self, stream=None):
        _check(self._lib.alea_grid_batch_build(self._h, stream))

    def stats(self):
        s = _GridBatchStats()
        _check(self._lib.alea_grid_batch_stats_get(self._h, ctypes.byref(s)))
        d = {f: getattr(s, f) for f, _ in s._fields_}
        d["tune_ms"] = list(s.tune_ms)
        return d

    def point_counts(self, i):
        out = np.zeros(3, np.int32)
        _check(self._lib.alea_grid_batch_point_counts(self._h, i, out.ctypes.data_as(_I32)))
        return tuple(int(v) for v in out)

    def table(self, i, species):
        nx, ny, nz = self.point_counts(i)
        out = np.zeros(nx * ny * nz)
        _check(self._lib.alea_grid_batch_download(self._h, i, species, _dp(out), out.size))
        return out


class WidomBatch:
    """Widom contexts for many frameworks run together (one persistent launch
    behind a captured CUDA graph); result i equals Widom.run on framework i."""

    def __init__(self, force_fields, frameworks, lattices, guests, temperature, ewalds=None,
                 precision=FP64):
        self._lib = library()
        self._h = _VP()
        n = len(frameworks)
        self.n = n
        gd = [{k: (_f64(g[k]) if k != "lj_species" else np.ascontiguousarray(g[k], dtype=np.uint32))
               for k in ("x", "y", "z", "lj_species", "charge")} for g in guests]
        sps = (_Species * n)(*[_Species(len(g["x"]), _dp(g["x"]), _dp(g["y"]), _dp(g["z"]),
                                        _u32p(g["lj_species"]), _dp(g["charge"])) for g in gd])
        ljs = (_LJ * n)(*[ff.c() for ff in force_fields])
        ps = (_Particles * n)(*[p.c() for p in frameworks])
        lats = (_Lattice * n)(*[_lattice(m) for m in lattices])
        ews = (_Ewald * n)(*[e.c() for e in ewalds]) if ewalds else None
        self._keep = (list(force_fields), list(frameworks), gd, sps, ljs, ps, lats, ews)
        _check(self._lib.alea_widom_batch_create(n, ljs, ews, ps, lats, sps, float(temperature),
                                                 int(precision), ctypes.byref(self._h)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                self._lib.alea_widom_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    def run(self, seeds, streams, n_trials, first_trial=0, draw_order=ALEA_DRAWS_RIGHT_TO_LEFT,
            stream=None):
        sd = np.ascontiguousarray(seeds, dtype=np.uint64)
        st = np.ascontiguousarray(streams, dtype=np.uint64)
        res = (_WidomResult * self.n)()
        _check(self._lib.alea_widom_batch_run(self._h, _u64p(sd), _u64p(st), first_trial, n_trials,
                                              draw_order, res, stream))
        return [{f: getattr(r, f) for f, _ in r._fields_} for r in res]


class Proposal:
    """Learned insertion proposal: a Fourier-feature MLP log-density f(s) over
    fractional positions, trained on the GPU, tabulated into the exact
    piecewise-constant density that Widom (run_biased) and GCMC sample from."""

    def __init__(self, n_freq=32, width=128, depth=3, freq_max=6, seed=7):
        self._lib = library()
        self._h = _VP()
        cfg = _ProposalConfig(n_freq, width, depth, freq_max, seed)
        _check(self._lib.alea_proposal_create(ctypes.byref(cfg), ctypes.byref(self._h)))
        self.n_freq, self.width, self.depth = n_freq, width, depth

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                self._lib.alea_proposal_destroy(h)
            except Exception:
                pass
            self._h = None

    def param_count(self):
        n = ctypes.c_uint64()
        _check(self._lib.alea_proposal_param_count(self._h, ctypes.byref(n)))
        return n.value

    def wave_vectors(self):
        k = np.zeros((self.n_freq, 3), np.int32)
        _check(self._lib.alea_proposal_wave_vectors(self._h, k.ctypes.data_as(_I32), k.size))
        return k

    def get_params(self):
        w = np.zeros(self.param_count(), np.float32)
        _check(self._lib.alea_proposal_get_params(self._h, w.ctypes.data_as(_F), w.size))
        return w

    def set_params(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        _check(self._lib.alea_proposal_set_params(self._h, w.ctypes.data_as(_F), w.size))

    def forward(self, s):
        s = np.ascontiguousarray(s, dtype=np.float32).reshape(-1, 3)
        out = np.zeros(len(s), np.float32)
        _check(self._lib.alea_proposal_forward(self._h, s.ctypes.data_as(_F), len(s),
                                               out.ctypes.data_as(_F)))
        return out

    def loss_grad(self, samples, tau=1.0):
        """Loss and gradient for host rows {s, l} or {s, l, lq} (lq = 0 if absent)."""
        samples = np.asarray(samples, dtype=np.float32)
        if samples.shape[1] == 4:
            samples = np.concatenate([samples, np.zeros((len(samples), 1), np.float32)], axis=1)
        samples = np.ascontiguousarray(samples, dtype=np.float32).reshape(-1, SAMPLE_ROW)
        g = np.zeros(self.param_count(), np.float32)
        loss = ctypes.c_double()
        _check(self._lib.alea_proposal_loss_grad(self._h, samples.ctypes.data_as(_F), len(samples),
                                                 float(tau), ctypes.byref(loss),
                                                 g.ctypes.data_as(_F), g.size))
        return loss.value, g

    def train(self, samples_device_ptr, n, epochs=20, batch=65536, lr=2e-3, tau=1.0,
              beta1=0.9, beta2=0.999, eps=1e-8, seed=11, stream=None):
        cfg = _TrainConfig(epochs, batch, lr, tau, beta1, beta2, eps, seed)
        loss = ctypes.c_double()
        _check(self._lib.alea_proposal_train(self._h, samples_device_ptr, n, ctypes.byref(cfg),
                                             ctypes.byref(loss), stream))
        return loss.value

    def fit(self, widom, n_samples=1 << 18, rounds=2, epochs=30, batch=16384, lr=2e-3, tau=1.0,
            cells=48, uniform_share=0.05, seed=1234, stream=7):
        """Trains on the Widom context's own trials and tabulates: round 0 on
        uniform trials, each further round on trials drawn from the previous
        round's table (importance-weighted by its density). Returns the final loss.
        Trial streams: (seed, stream + round)."""
        import torch

        rows = torch.empty((n_samples, SAMPLE_ROW), dtype=torch.float32, device="cuda")
        loss = float("nan")
        for r in range(rounds):
            widom.samples(seed, stream + r, n_samples, rows.data_ptr(),
                          proposal=self if r > 0 else None)
            loss = self.train(rows.data_ptr(), n_samples, epochs=epochs, batch=batch, lr=lr,
                              tau=tau, seed=seed + r)
            self.tabulate(cells, uniform_share)
        return loss

    def tabulate(self, cells=64, uniform_share=0.05):
        _check(self._lib.alea_proposal_tabulate(self._h, cells, float(uniform_share)))
        self.tabulated = True

    def fit_at_loading(self, chains, force_field, framework, lattice, guest, temperature,
                       ewald=None, chain_ids=(0,), n_samples=1 << 17, rounds=1, epochs=20,
                       batch=16384, lr=2e-3, tau=1.0, cells=48, uniform_share=0.2, seed=4321,
                       stream=100):
        """Refits on Widom trials in the loaded state: one Widom context per
        listed chain, whose framework is the framework plus that chain's guest
        sites now (so the trial energies include the guests already adsorbed).
        Rows are drawn from the current table when there is one (their log
        density enters the loss), else uniformly. Returns the final loss."""
        import torch

        ids = list(chain_ids)
        per = n_samples // len(ids)
        widoms = []
        for c in ids:
            sites, sp = chains.guest_sites(c)
            pd = ParticleData(np.concatenate([framework.x, sites[:, 0]]),
                              np.concatenate([framework.y, sites[:, 1]]),
                              np.concatenate([framework.z, sites[:, 2]]),
                              np.concatenate([framework.charge, sites[:, 3]]),
                              np.concatenate([framework.species, sp]))
            widoms.append(Widom(force_field, pd, lattice, guest, temperature, ewald=ewald))
        n = per * len(ids)
        rows = torch.empty((n, SAMPLE_ROW), dtype=torch.float32, device="cuda")
        row_bytes = SAMPLE_ROW * 4
        loss = float("nan")
        for r in range(rounds):
            for i, w in enumerate(widoms):
                w.samples(seed, stream + r * len(ids) + i, per, rows.data_ptr() + i * per * row_bytes,
                          proposal=self if getattr(self, "tabulated", False) else None)
            loss = self.train(rows.data_ptr(), n, epochs=epochs, batch=batch, lr=lr, tau=tau,
                              seed=seed + r)
            self.tabulate(cells, uniform_share)
        return loss

    def log_density(self, s):
        s = _f64(np.asarray(s, dtype=np.float64).reshape(-1, 3))
        out = np.zeros(len(s))
        _check(self._lib.alea_proposal_log_density(self._h, _dp(s), len(s), _dp(out)))
        return out


class GcmcChains:
    """MonteCarloEngine (monte_carlo_engine.hpp:76-83, 143-151) for many
    independent chains advanced together on the GPU. `guest` is one species
    (a dict: the single-species engine, one fugacity per chain) or a list of
    species (the mixture engine: per chain a list of fugacities)."""

    def __init__(self, force_field: LennardJones, framework: ParticleData, lattice, guest,
                 temperature: float, fugacities_pa, seeds, streams, ewald: Ewald | None = None,
                 max_translation=1.5, max_rotation=0.5, draw_order=ALEA_DRAWS_RIGHT_TO_LEFT,
                 max_molecules=256, precision=None):
        self._lib = library()
        self._h = _VP()
        mixture = isinstance(guest, (list, tuple))
        guests = list(guest) if mixture else [guest]
        self._g = [{k: (_f64(gd[k]) if k != "lj_species" else
                        np.ascontiguousarray(gd[k], dtype=np.uint32))
                    for k in ("x", "y", "z", "lj_species", "charge")} for gd in guests]
        sps = (_Species * len(guests))()
        for i, gd in enumerate(self._g):
            sps[i] = _Species(len(gd["x"]), _dp(gd["x"]), _dp(gd["y"]), _dp(gd["z"]),
                              _u32p(gd["lj_species"]), _dp(gd["charge"]))
        f = np.asarray(fugacities_pa, dtype=np.float64)
        if mixture:
            f = f.reshape(-1, len(guests))
        else:
            f = np.atleast_1d(f).reshape(-1, 1)
        f = _f64(f.reshape(-1))
        se = np.ascontiguousarray(np.atleast_1d(seeds), dtype=np.uint64)
        st = np.ascontiguousarray(np.atleast_1d(streams), dtype=np.uint64)
        self.n_chains = len(f) // len(guests)
        self.n_species = len(guests)
        if len(se) != self.n_chains or len(st) != self.n_chains:
            raise ValueError("one fugacity (per species), seed and stream per chain")
        lj = force_field.c()
        p = framework.c()
        lat = _lattice(lattice)
        e = ewald.c() if ewald is not None else None
        _check(self._lib.alea_gcmc_create_mixture(
            ctypes.byref(lj), ctypes.byref(e) if e else None, ctypes.byref(p), ctypes.byref(lat),
            len(guests), sps, float(temperature), _dp(f), _u64p(se), _u64p(st), self.n_chains,
            float(max_translation), float(max_rotation), int(draw_order), int(max_molecules),
            ctypes.byref(self._h)))
        if precision is not None:
            self.set_precision(precision)

    def set_grid(self, grid):
        """Dispersion from a FrameworkEnergyGrid of this cell (kept alive here)
        plus the guests' LJ, as the reference engine with its grid; None
        restores the direct scan."""
        _check(self._lib.alea_gcmc_set_grid(self._h, grid._h if grid is not None else None))
        self._grid = grid

    def set_orientation_trials(self, k):
        """Orientation-biased insertion and deletion with k trial orientations
        (k = 1: the reference's single random orientation)."""
        _check(self._lib.alea_gcmc_set_orientation_trials(self._h, int(k)))

    def set_tail_correction(self, on=True):
        """Opt-in: insertions, deletions and swaps add U_tail(after) - U_tail(before)
        (the reference engine's moves leave the tail correction out)."""
        _check(self._lib.alea_gcmc_set_tail_correction(self._h, 1 if on else 0))

    def set_precision(self, precision):
        """FP64 (the reference's arithmetic) or FP32 (FP32 pair terms and
        S(k) phases, FP64 sums) for the next runs."""
        _check(self._lib.alea_gcmc_set_precision(self._h, int(precision)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                self._lib.alea_gcmc_destroy(h)
            except Exception:
                pass
            self._h = None

    def run(self, steps, stream=0):
        _check(self._lib.alea_gcmc_run(self._h, int(steps), stream))

    def set_proposal(self, proposal):
        """Insert and delete with a tabulated learned Proposal from now on (its
        density enters the acceptance ratios); None restores uniform insertion."""
        _check(self._lib.alea_gcmc_set_proposal(self._h, proposal._h if proposal else None))

    def info(self, chain=0):
        s = _ChainInfo()
        _check(self._lib.alea_gcmc_chain_info_get(self._h, chain, ctypes.byref(s)))
        d = {f: getattr(s, f) for f, _ in s._fields_}
        d["attempted"] = list(s.attempted)
        d["accepted"] = list(s.accepted)
        d["species_molecules"] = list(s.species_molecules)
        return d

    def molecules(self, chain=0):
        return int(self.info(chain)["molecules"])

    def positions(self, chain=0):
        n = ctypes.c_uint64()
        _check(self._lib.alea_gcmc_particles(self._h, chain, None, 0, ctypes.byref(n)))
        out = np.zeros(3 * n.value)
        _check(self._lib.alea_gcmc_particles(self._h, chain, _dp(out), n.value, ctypes.byref(n)))
        return out.reshape(-1, 3)

    def guest_sites(self, chain=0):
        """This chain's guest sites: (n, 4) x, y, z, charge and (n,) LJ species."""
        n = ctypes.c_uint64()
        _check(self._lib.alea_gcmc_guest_sites(self._h, chain, None, None, 0, ctypes.byref(n)))
        xyzq = np.zeros(4 * max(n.value, 1))
        sp = np.zeros(max(n.value, 1), dtype=np.uint32)
        _check(self._lib.alea_gcmc_guest_sites(self._h, chain, _dp(xyzq), _u32p(sp), n.value,
                                               ctypes.byref(n)))
        return xyzq[:4 * n.value].reshape(-1, 4), sp[:n.value]

    def ewald_energy(self, chain=0):
        v = ctypes.c_double()
        _check(self._lib.alea_gcmc_ewald_energy(self._h, chain, ctypes.byref(v)))
        return v.value


def peng_robinson_fugacity(tc, pc, omega, t, p):
    v = ctypes.c_double()
    _check(library().alea_peng_robinson_fugacity(tc, pc, omega, t, p, ctypes.byref(v)))
    return v.value


class Structure:
    """readCif's StructureData (io/structure_io.hpp:18-40): `particles` (a
    ParticleData: x, y, z, charge, species), `lattice` (3x3 rows a_i), `mass`,
    `species_symbols` (element of each species id), `occupancy` and
    `source_label` (the atom_site label each atom was expanded from)."""

    def __init__(self, particles, lattice, mass, species_symbols, occupancy, source_label):
        self.particles = particles
        self.lattice = lattice
        self.mass = mass
        self.species_symbols = species_symbols
        self.occupancy = occupancy
        self.source_label = source_label


def read_cif(path) -> Structure:
    """readCif(file) (io/structure_io.hpp:51): a malformed file raises
    RuntimeError with the reference's CifParseError message."""
    lib = library()
    h = _VP()
    _check(lib.alea_read_cif(os.fsencode(str(path)), ctypes.byref(h)))
    try:
        n, ns = ctypes.c_uint64(), ctypes.c_uint32()
        _check(lib.alea_structure_sizes(h, ctypes.byref(n), ctypes.byref(ns)))
        m = np.zeros(9)
        _check(lib.alea_structure_lattice(h, _dp(m)))
        x, y, z, q, mass, occ = (np.zeros(n.value) for _ in range(6))
        sp = np.zeros(n.value, np.uint32)
        _check(lib.alea_structure_atoms(h, _dp(x), _dp(y), _dp(z), _dp(q), _dp(mass), _u32p(sp),
                                        _dp(occ)))
        buf = ctypes.create_string_buffer(4096)
        symbols = []
        for k in range(ns.value):
            _check(lib.alea_structure_species_symbol(h, k, buf, 4096))
            symbols.append(buf.value.decode())
        labels = []
        for i in range(n.value):
            _check(lib.alea_structure_source_label(h, i, buf, 4096))
            labels.append(buf.value.decode())
    finally:
        lib.alea_structure_destroy(h)
    return Structure(ParticleData(x, y, z, q, sp), m.reshape(3, 3), mass, symbols, occ, labels)


def peng_robinson_mixture(substances, t, p, mole_fractions, kij=None):
    """PengRobinsonMixture(substances, kij): (compressibilityFactor,
    fugacitiesPascal) at temperature t (K), total pressure p (Pa) and the mole
    fractions; substances = [(tc, pc, omega), ...], kij an n x n matrix or None."""
    n = len(substances)
    tc, pc, om = (np.ascontiguousarray([s[i] for s in substances], dtype=np.float64)
                  for i in range(3))
    k = None  # the constructor's check comes before fugacitiesPascal's
    if kij is not None:
        k = np.ascontiguousarray(kij, dtype=np.float64)
        if n >= 2 and k.shape != (n, n):
            raise ValueError("PengRobinsonMixture: binaryInteractionKij must be substances.size() x "
                             "substances.size()")
    x = np.ascontiguousarray(mole_fractions, dtype=np.float64)
    if n >= 2 and x.shape != (n,):
        raise ValueError("PengRobinsonMixture: moleFractions.size() must equal the number of substances")
    f = np.zeros(n)
    z = ctypes.c_double()
    _check(library().alea_peng_robinson_mixture(n, _dp(tc), _dp(pc), _dp(om),
                                                None if k is None else _dp(k), t, p, _dp(x),
                                                ctypes.byref(z), _dp(f)))
    return z.value, f
