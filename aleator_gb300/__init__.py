"""aleator_gb300 — GB300 (sm_103a) GCMC energy hot path behind a C ABI.

Python mirror of the reference engine's hot-path interfaces
(Defalt-Meh/aleator, src/): FrameworkEnergyGrid, EwaldIncrementalState,
Widom insertion (MonteCarloEngine::widomInsertionHenryCoefficient),
LennardJones / Ewald per-particle energies and the Philox4x32-10 streams. Every
call goes through ``libaleator_gb300.so`` (include/aleator_gb300.h); there is
no CPU fallback: a missing library or device raises.
"""
from ._lib import (  # noqa: F401
    ALEA_DRAWS_LEFT_TO_RIGHT,
    ALEA_DRAWS_RIGHT_TO_LEFT,
    FP32,
    FP64,
    GEOMETRIC,
    LINEAR_FORCE_SHIFTED,
    LORENTZ_BERTHELOT,
    SAMPLE_ROW,
    SHIFTED,
    TRUNCATED,
    AleatorError,
    Ewald,
    EwaldIncrementalState,
    FrameworkEnergyGrid,
    GcmcChains,
    GridBatch,
    LennardJones,
    ParticleData,
    Proposal,
    Widom,
    WidomBatch,
    device_info,
    ewald_energy_breakdown,
    ewald_real_space_particle_energy,
    ewald_reciprocal_terms,
    fp32_fma_tflops,
    library,
    lj_particle_energy,
    lj_tail_correction,
    load_library,
    peng_robinson_fugacity,
    peng_robinson_mixture,
    read_cif,
    Structure,
    philox4x32_10,
    philox_u64,
    philox_uniform,
)
