/*
 * aleator_gb300 — C ABI of the GB300 (sm_103a) GCMC energy hot path.
 *
 * Plain C: pointers, sizes and status codes only. Every entry point names
 * the reference interface it replaces (paths relative to the reference
 * project's src/). Host pointers are borrowed for the duration of a call;
 * opaque handles own their device memory. No exception crosses this
 * boundary: each call returns an alea_status and the calling thread's last
 * error message is available from alea_last_error(). The status codes map
 * one-to-one onto the exception types the reference throws:
 *   ALEA_ERR_INVALID_ARGUMENT -> std::invalid_argument
 *   ALEA_ERR_OUT_OF_RANGE     -> std::out_of_range
 *   ALEA_ERR_RUNTIME          -> std::runtime_error
 *
 * Units follow the reference: Å, K (energy / k_B), e, K/Å^3 for pressure.
 * Lattices are row-major double[9], row i = lattice vector a_i
 * (core/geometry/lattice.hpp:21-30).
 *
 * The engines (Widom, GCMC, the Ewald state) require cutoff <= L_perp/2 on
 * every axis, as the reference's do (Lattice::validateCutoff,
 * core/geometry/lattice.cc:286-300): under that condition at most one
 * periodic image of an atom lies within the cutoff, which is what makes the
 * device kernels' image handling equal to the reference's minimum-image
 * search. The energy grid accepts any cutoff, as the reference's constructor
 * does; above L_perp/2 it sums the reference's single minimum image per atom
 * (an FP64 kernel, whatever precision is asked for).
 */
#ifndef ALEATOR_GB300_H
#define ALEATOR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t alea_status;
enum {
    ALEA_OK = 0,
    ALEA_ERR_INVALID_ARGUMENT = 1,
    ALEA_ERR_OUT_OF_RANGE = 2,
    ALEA_ERR_RUNTIME = 3,
    ALEA_ERR_CUDA = 4,
    ALEA_ERR_NO_DEVICE = 5,
    ALEA_ERR_DEVICE_CHECK = 6 /* a kernel's own bounds / wait check fired */
};

/* LennardJonesTruncation (forcefield/pairwise/lennard_jones.hpp:21-38) */
enum { ALEA_TRUNCATED = 0, ALEA_SHIFTED = 1, ALEA_LINEAR_FORCE_SHIFTED = 2 };
/* MixingRule (forcefield/pairwise/lennard_jones.hpp:42-50) */
enum { ALEA_LORENTZ_BERTHELOT = 0, ALEA_GEOMETRIC = 1 };
/* Arithmetic of the pair sums. FP64 is the parity form; FP32 evaluates pair
 * terms in FP32 and accumulates them into FP64 per atom tile. */
enum { ALEA_FP64 = 0, ALEA_FP32 = 1 };
/* Order in which the reference's nested RNG draws reach their arguments
 * (monte_carlo_engine.cc:572-579, 882-888): C++ leaves it unspecified; GCC
 * evaluates right to left (a2 gets the first uniform), clang left to right. */
enum { ALEA_DRAWS_RIGHT_TO_LEFT = 0, ALEA_DRAWS_LEFT_TO_RIGHT = 1 };

typedef struct {
    double m[9];
} alea_lattice;

/* LennardJones(perSpecies, cutoff, truncation, mixingRule)
 * (forcefield/pairwise/lennard_jones.hpp:64-66) */
typedef struct {
    uint32_t n_species;
    const double* epsilon; /* K, per LJ species */
    const double* sigma;   /* Å, per LJ species */
    double cutoff;
    int32_t truncation;
    int32_t mixing;
} alea_lennard_jones;

/* Ewald(alpha, realSpaceCutoff, kMax) (forcefield/electrostatics/ewald.hpp:76-77) */
typedef struct {
    double alpha;
    double real_space_cutoff;
    int32_t kmax;
} alea_ewald;

/* core::ParticleData SoA (core/math/particle_data.hpp:20-25), host pointers.
 * charge may be NULL (all zero); species may be NULL (all zero). */
typedef struct {
    uint64_t n;
    const double* x;
    const double* y;
    const double* z;
    const double* charge;
    const uint32_t* species;
} alea_particles;

/* MoleculeSpecies / MoleculeSite (engines/monte_carlo/molecule_species.hpp:14-29) */
typedef struct {
    uint32_t n_sites;
    const double* x;
    const double* y;
    const double* z;
    const uint32_t* lj_species;
    const double* charge;
} alea_molecule_species;

/* ------------------------------------------------------------------ errors / device */
const char* alea_status_string(alea_status s);
/* Copies the calling thread's last error message; returns its full length. */
size_t alea_last_error(char* buf, size_t cap);
/* Library build identification: compute capability compiled for, e.g. 103. */
alea_status alea_version(int32_t* major, int32_t* minor, int32_t* arch);
/* Device name and SM count of the current device. */
alea_status alea_device_info(char* name, size_t cap, int32_t* sm_count, int32_t* cc_major,
                             int32_t* cc_minor);

/* Sustained FP32 FFMA throughput of the current device in TFLOP/s (a
 * measurement helper: the roofline denominator of the FP32 pair kernels). */
alea_status alea_probe_fp32_fma_tflops(double* out);
/* The same with the packed two-lane FMA (fma.rn.f32x2), the instruction the
 * FP32 grid sweep issues; an FMA lane counts 2 FLOP. */
alea_status alea_probe_fp32x2_fma_tflops(double* out);
/* Test support for the FP32 forms' double-float near-pair arithmetic (no
 * counterpart in the reference): n values from host arrays. mode 0: out[i] =
 * erfc(in[i]) for 0 <= in[i] <= 2; mode 1: in holds n records (dx, dy, dz, q)
 * and out[i] = q erfc(alpha r) / r, or NaN where alpha r is beyond the series
 * (the kernels then take the FP64 form). */
alea_status alea_test_ff_near(int32_t mode, const double* in, double* out, uint64_t n,
                              double alpha);

/* Device memory held idle by the library's block cache (no counterpart in the
 * reference, which allocates on the host). Device blocks of 64 MB and more are
 * kept on release, up to 16 GB idle over all devices, and handed out again for
 * a request of the same size on the same device, so that a grid rebuilt step
 * after step skips cudaMalloc/cudaFree. Keeping a block synchronizes its own
 * device first, the ordering cudaFree gives. Other jobs on a shared GPU do not
 * see the idle blocks as free: alea_release_cached gives them back (the freed
 * bytes in *freed, which may be NULL); an allocation that fails for memory
 * releases the device's idle blocks and tries once more. */
alea_status alea_cached_bytes(uint64_t* out);
alea_status alea_release_cached(uint64_t* freed);
/* Test support for the block cache: runs a scripted take / put / drain
 * sequence on its bookkeeping with fake pointers (no device call) and returns
 * ALEA_OK when each step returned what keying by (device, size) requires. */
alea_status alea_test_block_cache(void);

/* ------------------------------------------------------------------ Philox4x32-10 */
/* philox4x32_10 (core/math/counter_based_rng.hpp:43-44, .cc:42-54), evaluated
 * on the device for n (counter, key) pairs: ctr 4n, key 2n, out 4n words. */
alea_status alea_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out, uint64_t n);
/* Philox4x32Rng::seed(seed, stream) then n x nextU64() starting at call
 * index `first` (counter_based_rng.cc:56-71). Host output. */
alea_status alea_philox_fill_u64(uint64_t seed, uint64_t stream, uint64_t first, uint64_t n,
                                 uint64_t* out);
/* ... n x nextUniform() (counter_based_rng.cc:73-79). Host output. */
alea_status alea_philox_fill_uniform(uint64_t seed, uint64_t stream, uint64_t first, uint64_t n,
                                     double* out);
/* Device-resident variants (out is a device pointer; stream is a cudaStream_t). */
alea_status alea_philox_fill_u64_device(uint64_t seed, uint64_t stream_index, uint64_t first,
                                        uint64_t n, uint64_t* out, void* cuda_stream);
alea_status alea_philox_fill_uniform_device(uint64_t seed, uint64_t stream_index, uint64_t first,
                                            uint64_t n, double* out, void* cuda_stream);

/* ------------------------------------------------------------------ framework energy grid */
/* FrameworkEnergyGrid(forceField, frameworkParticles, lattice, guestSpeciesIds,
 * spacingAngstrom) (engines/monte_carlo/framework_energy_grid.hpp:118-120,
 * .cc:193-249): builds one table per distinct guest species on the device.
 * Fails with ALEA_ERR_INVALID_ARGUMENT when spacing <= 0 (as the reference)
 * or when cutoff > L_perp/2. */
typedef struct alea_grid alea_grid;
alea_status alea_grid_build(const alea_lennard_jones* lj, const alea_particles* framework,
                            const alea_lattice* lattice, const uint32_t* guest_species,
                            uint32_t n_guest, double spacing, int32_t precision, alea_grid** out);
/* pointCounts() / spacingAngstrom() (framework_energy_grid.hpp:131-132) */
alea_status alea_grid_point_counts(const alea_grid* g, int32_t out[3]);
alea_status alea_grid_spacing(const alea_grid* g, double* out);
/* Sorted distinct guest species with a table; n_out receives the count. */
alea_status alea_grid_species(const alea_grid* g, uint32_t* out, uint32_t cap, uint32_t* n_out);
/* interpolate(guestSpeciesId, position) (framework_energy_grid.hpp:128-129,
 * .cc:251-288) for n positions (xyz interleaved, host). Unknown species ->
 * ALEA_ERR_OUT_OF_RANGE, as the reference's tables_.at(). */
alea_status alea_grid_interpolate(const alea_grid* g, uint32_t species, const double* xyz,
                                  uint64_t n, double* out);
/* Same with device pointers on a caller stream (the HBM-resident form). */
alea_status alea_grid_interpolate_device(const alea_grid* g, uint32_t species, const double* xyz,
                                         uint64_t n, double* out, void* cuda_stream);
/* Copies one species' table (nx*ny*nz doubles, index (iz*ny+iy)*nx+ix,
 * framework_energy_grid.hpp:186-194) to host memory. */
alea_status alea_grid_download(const alea_grid* g, uint32_t species, double* out, uint64_t n);
/* Device pointer of one species' table (owned by the grid). */
alea_status alea_grid_table_device(const alea_grid* g, uint32_t species, const double** out);
/* Re-runs the build kernels into the grid's own tables with inputs already
 * resident in HBM; returns the kernel-only time. Used for measurement. */
alea_status alea_grid_rebuild(alea_grid* g, void* cuda_stream);
typedef struct {
    uint64_t nodes;             /* nx*ny*nz */
    uint64_t algorithmic_pairs; /* sum over species of nodes * framework atoms */
    uint64_t executed_pairs;    /* node-image pairs the kernel evaluated (all species) */
    uint64_t images;            /* periodic atom images staged */
    uint64_t bricks;            /* thread-block tiles of nodes */
    float last_kernel_ms;       /* duration of the last build's launches, CUDA events */
    uint32_t launches;          /* kernel launches of the last build */
} alea_grid_stats;
alea_status alea_grid_stats_get(const alea_grid* g, alea_grid_stats* out);
/* Writes the reference's on-disk cache file for this grid (format version 1,
 * framework_energy_grid.cc:290-316; key layout framework_energy_grid.cc:77-97).
 * The key fields are passed explicitly as in makeFrameworkEnergyGridCacheKey
 * (framework_energy_grid.cc:169-191). */
alea_status alea_grid_serialize(const alea_grid* g, const char* path,
                                const alea_lennard_jones* lj, const alea_particles* framework,
                                const alea_lattice* lattice, const uint32_t* guest_species,
                                uint32_t n_guest);
/* The constructor followed by reading every table, pipelined: the build runs
 * in z-slabs and each finished slab's node rows are copied to host_tables[k]
 * (one array of point_counts' product doubles per entry of guest_species, in
 * that order) while the next slab computes. Pinned host arrays
 * (cudaHostAlloc) let the copies overlap; pageable ones still work. *out may
 * be NULL when only the tables are wanted. */
alea_status alea_grid_build_to_host(const alea_lennard_jones* lj, const alea_particles* framework,
                                    const alea_lattice* lattice, const uint32_t* guest_species,
                                    uint32_t n_guest, double spacing_angstrom, int32_t precision,
                                    double* const* host_tables, alea_grid** out);
/* Test support for the device-side bounded waits (no counterpart in the
 * reference, which has no device code): the tile waits of the next FP64-form
 * grid build or rebuild in this process give up after `limit` polls (0: at the
 * first wait) instead of the usual ~2^20 (the FP32 form's tiles complete on
 * cp.async.wait_all, with no polled wait). The build then ends with
 * ALEA_ERR_DEVICE_CHECK ("wait") after each CTA has waited, with the usual
 * limit, for the copy it still had in flight; the device stays usable and the
 * build after it runs normally. limit < 0 cancels a pending setting. */
alea_status alea_test_grid_tile_wait_limit(int64_t limit);
/* cacheFilePath(cacheDirectory, key) (framework_energy_grid.cc:318-325). */
alea_status alea_grid_cache_file_name(const alea_lennard_jones* lj,
                                      const alea_particles* framework,
                                      const alea_lattice* lattice, const uint32_t* guest_species,
                                      uint32_t n_guest, double spacing, char* out, size_t cap);
/* cacheHit(cacheDirectory, key) (framework_energy_grid.cc:326-352): *hit = 1
 * when the file named by the key exists and its version and stored key match
 * exactly, 0 when no file is there; ALEA_ERR_RUNTIME when a file at that path
 * has another format version or another stored key (a collision or a foreign
 * file: never a miss, never a reuse). Host only: reads the file's header. */
alea_status alea_grid_cache_hit(const char* cache_dir, const alea_lennard_jones* lj,
                                const alea_particles* framework, const alea_lattice* lattice,
                                const uint32_t* guest_species, uint32_t n_guest, double spacing,
                                int32_t* hit);
/* loadFromCache (framework_energy_grid.cc:354-409): reads the file named by
 * the key in cache_dir; *out = NULL on a plain miss; ALEA_ERR_RUNTIME on a
 * version mismatch, key mismatch or truncated file. */
alea_status alea_grid_load_cache(const char* cache_dir, const alea_lennard_jones* lj,
                                 const alea_particles* framework, const alea_lattice* lattice,
                                 const uint32_t* guest_species, uint32_t n_guest, double spacing,
                                 alea_grid** out);
alea_status alea_grid_destroy(alea_grid* g);

/* ------------------------------------------------------------------ CIF structures */
/* readCif (io/structure_io.hpp:51, io/structure_io.cc:177-245): the cell
 * (a, b, c, alpha, beta, gamma; a along x, b in the xy plane), the symmetry
 * operations (_symmetry_equiv_pos_as_xyz or _space_group_symop_operation_xyz,
 * P1 when neither is present) and the _atom_site loop expanded through every
 * operation with images within 1e-3 A merged. Particles equal the reference's
 * bit for bit; a malformed file fails with ALEA_ERR_RUNTIME and the
 * reference's CifParseError message. Host only (no device needed). */
typedef struct alea_structure alea_structure;
alea_status alea_read_cif(const char* path, alea_structure** out);
/* particles.size(), speciesSymbols.size() */
alea_status alea_structure_sizes(const alea_structure* s, uint64_t* n_atoms, uint32_t* n_species);
/* lattice.matrix() rows a_i, row-major */
alea_status alea_structure_lattice(const alea_structure* s, double m[9]);
/* particles x, y, z, charge, mass, species and the per-atom occupancy, each
 * n_atoms long; any pointer may be NULL. x, y, z, charge, species are
 * alea_particles' arrays. */
alea_status alea_structure_atoms(const alea_structure* s, double* x, double* y, double* z,
                                 double* charge, double* mass, uint32_t* species,
                                 double* occupancy);
/* speciesSymbols[species], sourceLabel[atom]: NUL-terminated into out */
alea_status alea_structure_species_symbol(const alea_structure* s, uint32_t species, char* out,
                                          size_t cap);
alea_status alea_structure_source_label(const alea_structure* s, uint64_t atom, char* out,
                                        size_t cap);
alea_status alea_structure_destroy(alea_structure* s);

/* ------------------------------------------------------------------ batch of energy grids */
/* No counterpart in the reference (one FrameworkEnergyGrid per framework,
 * framework_energy_grid.cc:193-249). n independent frameworks, each with its
 * own force field, atoms and cell (so their node counts differ), built in the
 * FP32 form in one persistent launch: CTAs take (grid, brick) work items from
 * a global counter. The first build times the launch variants on the batch
 * (the autotuner) and captures the chosen launch into a CUDA graph; every
 * build replays it. Each grid equals a single
 * alea_grid_build of that framework (FP32), bit for bit. guest_species holds
 * n x n_guest ids; every grid must have the same number of distinct guests
 * (1..4) and the same truncation. */
typedef struct alea_grid_batch alea_grid_batch;
alea_status alea_grid_batch_create(uint32_t n, const alea_lennard_jones* lj,
                                   const alea_particles* frameworks, const alea_lattice* lattices,
                                   const uint32_t* guest_species, uint32_t n_guest, double spacing,
                                   alea_grid_batch** out);
alea_status alea_grid_batch_build(alea_grid_batch* b, void* cuda_stream);
typedef struct {
    uint32_t grids;
    uint64_t nodes;             /* over all grids */
    uint64_t algorithmic_pairs; /* sum of nodes x atoms x guests */
    uint64_t executed_pairs;    /* node-image pairs evaluated (all guests) */
    uint64_t bricks;            /* work items */
    float last_ms;              /* the last build (one graph launch), CUDA events */
    int32_t variant;            /* launch variant the autotuner chose (-1 before the first build) */
    float tune_ms[2];           /* the autotuner's timings of each variant */
    uint32_t graph_launches;
} alea_grid_batch_stats;
alea_status alea_grid_batch_stats_get(const alea_grid_batch* b, alea_grid_batch_stats* out);
alea_status alea_grid_batch_point_counts(const alea_grid_batch* b, uint32_t grid, int32_t out[3]);
alea_status alea_grid_batch_download(const alea_grid_batch* b, uint32_t grid, uint32_t species,
                                     double* out, uint64_t n);
alea_status alea_grid_batch_destroy(alea_grid_batch* b);

/* ------------------------------------------------------------------ Lennard-Jones */
/* LennardJones::computeParticleEnergy(index, particles, lattice, excluded)
 * (lennard_jones.cc:158-182) for n_query indices at once. */
alea_status alea_lj_particle_energy(const alea_lennard_jones* lj, const alea_particles* particles,
                                    const alea_lattice* lattice, const uint64_t* query,
                                    uint64_t n_query, const uint64_t* excluded,
                                    uint64_t n_excluded, double* out);
/* LennardJones::tailEnergyCorrection (lennard_jones.cc:246-257). */
alea_status alea_lj_tail_correction(const alea_lennard_jones* lj, const alea_particles* particles,
                                    const alea_lattice* lattice, double* out);

/* ------------------------------------------------------------------ Ewald */
/* Ewald::reciprocalTerms(lattice) (ewald.hpp:137-138, ewald.cc:137-161):
 * k (3 per term) and weight; n_out = total count even when cap is smaller. */
alea_status alea_ewald_reciprocal_terms(const alea_lattice* lattice, double alpha, int32_t kmax,
                                        double* k, double* weight, uint64_t cap, uint64_t* n_out);
/* Ewald::realSpaceParticleEnergy (ewald.hpp:159-161, ewald.cc:223-249) for
 * n_query indices. */
alea_status alea_ewald_real_space_particle_energy(const alea_ewald* ewald,
                                                  const alea_particles* particles,
                                                  const alea_lattice* lattice,
                                                  const uint64_t* query, uint64_t n_query,
                                                  const uint64_t* excluded, uint64_t n_excluded,
                                                  double* out);
/* Ewald::computeEnergyBreakdown (ewald.cc:251-313): out = {real, reciprocal,
 * self, exclusion, surface}; exclusions as index pairs (2 per pair).
 * ALEA_ERR_INVALID_ARGUMENT for a non-neutral system (ewald.cc:181-195). */
alea_status alea_ewald_energy_breakdown(const alea_ewald* ewald, const alea_particles* particles,
                                        const alea_lattice* lattice, const uint64_t* exclusions,
                                        uint64_t n_exclusions, double out[5]);

/* EwaldIncrementalState (forcefield/electrostatics/ewald_incremental_state.hpp:70-171):
 * the structure-factor cache lives in HBM. Sites are packed {x, y, z, q}. */
typedef struct alea_ewald_state alea_ewald_state;
/* EwaldIncrementalState(ewald, particles, lattice) (ewald_incremental_state.cc:55-83) */
alea_status alea_ewald_state_create(const alea_ewald* ewald, const alea_particles* particles,
                                    const alea_lattice* lattice, alea_ewald_state** out);
/* committedEnergy() (ewald_incremental_state.cc:85-93) */
alea_status alea_ewald_state_committed_energy(const alea_ewald_state* s, double* out);
/* proposeMove / proposeInsertion / proposeDeletion (ewald_incremental_state.cc:147-159):
 * removed -> added; never mutates the committed cache. */
alea_status alea_ewald_state_propose(const alea_ewald_state* s, const double* removed,
                                     uint64_t n_removed, const double* added, uint64_t n_added,
                                     double* delta);
/* commitMove / commitInsertion / commitDeletion (ewald_incremental_state.cc:161-172) */
alea_status alea_ewald_state_commit(alea_ewald_state* s, const double* removed,
                                    uint64_t n_removed, const double* added, uint64_t n_added);
/* recomputeFromScratch (ewald_incremental_state.cc:174-212); molecules as
 * CSR (offsets n_molecules+1, indices). */
alea_status alea_ewald_state_recompute(const alea_ewald_state* s, const alea_particles* particles,
                                       uint64_t n_molecules, const uint64_t* offsets,
                                       const uint64_t* indices, double* out);
/* resync (ewald_incremental_state.cc:214-247) */
alea_status alea_ewald_state_resync(alea_ewald_state* s, const alea_particles* particles,
                                    uint64_t n_molecules, const uint64_t* offsets,
                                    const uint64_t* indices);
/* rawStateForTesting (ewald_incremental_state.cc:249-257): sRe..., sIm...,
 * self, exclusion; n_out = full length. */
alea_status alea_ewald_state_raw(const alea_ewald_state* s, double* out, uint64_t cap,
                                 uint64_t* n_out);
alea_status alea_ewald_state_term_count(const alea_ewald_state* s, uint64_t* out);
alea_status alea_ewald_state_destroy(alea_ewald_state* s);

/* No counterpart in the reference. The energy change alea_ewald_state_propose
 * computes, for callers that cannot let a library allocate device memory: an
 * engine that hands out every device buffer from its own pre-reserved pool,
 * or one that cannot accept the device-wide synchronisation cudaMalloc and
 * cudaFree may imply while its other streams are busy. This call allocates
 * nothing. The caller passes device pointers to the terms' k vectors
 * (3 doubles each), weights and committed sRe / sIm (n_terms each), the
 * Ewald alpha and the lattice, the removed and added sites as host arrays
 * (packed {x, y, z, q}; at most 64 together), and a device pointer `out` to 4
 * doubles that receive {reciprocal, self, exclusion, total}. The call is
 * asynchronous on cuda_stream. Limit: n_terms <= 262144 (the size of the fixed
 * scratch array; larger requests fail with ALEA_ERR_INVALID_ARGUMENT). The
 * per-block partial sums live in one file-scope device array that every GPU
 * loading the library holds until exit; calls that overlap on the GPU race on
 * it, and the first call on each device looks up its address, so make that
 * first call before any stream capture. */
alea_status alea_ewald_propose_no_alloc(const double* k, const double* weight, const double* sre,
                                        const double* sim, uint64_t n_terms, double alpha,
                                        const alea_lattice* lattice, const double* removed,
                                        uint64_t n_removed, const double* added, uint64_t n_added,
                                        double* out, void* cuda_stream);

/* ------------------------------------------------------------------ Widom insertion */
/* MonteCarloEngine::widomInsertionHenryCoefficient(numTrials, speciesIndex)
 * (engines/monte_carlo/monte_carlo_engine.hpp:198-199, .cc:850-917) on the
 * device: trial t of stream (seed, stream) uses Philox call indices 3t..3t+2
 * (one site) or 6t..6t+5 (several sites), exactly the draws a freshly seeded
 * engine makes. A context holds the framework, force field, optional Ewald
 * S(k) of the framework and the guest template in HBM. */
typedef struct alea_widom alea_widom;
alea_status alea_widom_create(const alea_lennard_jones* lj, const alea_ewald* ewald /* nullable */,
                              const alea_particles* framework, const alea_lattice* lattice,
                              const alea_molecule_species* guest, double temperature,
                              int32_t precision, alea_widom** out);
typedef struct {
    double henry;             /* K_H = mean(exp(-dU/T)) / T, 1/K */
    double log_mean_weight;   /* log(mean(exp(-dU/T))), from the FP64 log-sum-exp */
    double rel_std_error;     /* standard error of K_H / K_H over the trials */
    uint64_t n_trials;
    float kernel_ms;          /* device time of the trial + reduction kernels */
} alea_widom_result;
/* Trials [first_trial, first_trial + n_trials); per_trial_du (nullable, host)
 * receives each trial's deltaU in K. */
alea_status alea_widom_run(alea_widom* w, uint64_t seed, uint64_t stream, uint64_t first_trial,
                           uint64_t n_trials, int32_t draw_order, alea_widom_result* out,
                           double* per_trial_du);
alea_status alea_widom_destroy(alea_widom* w);

/* ------------------------------------------------------------------ learned insertion proposal */
/* No counterpart in the reference, whose insertions are uniform
 * (monte_carlo_engine.cc:572-574, 882-884). A Fourier-feature MLP log-density
 * f(s) over fractional positions s in [0,1)^3 (2 n_freq periodic features
 * (sin, cos)(2 pi k.s) with integer k, `depth` SiLU layers of `width`, one
 * output; BF16 weights, FP32 accumulation), trained on the GPU on
 * Boltzmann-weighted uniform Widom samples, then tabulated on cells^3 cells
 * and mixed with a uniform share. Widom and GCMC sample from that table, so
 * the proposal density that enters their weights is exact. */
typedef struct alea_proposal alea_proposal;
typedef struct {
    uint32_t n_freq;   /* wave vectors: 2 n_freq features */
    uint32_t width;    /* hidden width */
    uint32_t depth;    /* hidden layers */
    uint32_t freq_max; /* wave-vector components uniform in [-freq_max, freq_max] */
    uint64_t seed;     /* wave vectors and initial weights (Philox streams 1, 2) */
} alea_proposal_config;
alea_status alea_proposal_create(const alea_proposal_config* config, alea_proposal** out);
alea_status alea_proposal_param_count(const alea_proposal* p, uint64_t* out);
/* n_freq x 3 integer wave vectors */
alea_status alea_proposal_wave_vectors(const alea_proposal* p, int32_t* out, uint64_t cap);
/* FP32 master weights: per layer W [out x in] row-major, then b [out] */
alea_status alea_proposal_get_params(const alea_proposal* p, float* out, uint64_t n);
alea_status alea_proposal_set_params(alea_proposal* p, const float* in, uint64_t n);
/* f(s) at n host positions (3 floats each) */
alea_status alea_proposal_forward(alea_proposal* p, const float* s, uint64_t n, float* out);
/* Training rows are ALEA_SAMPLE_ROW floats {s0, s1, s2, l, lq}: a fractional
 * position, its log-weight l = -dU/T and the log density lq (relative to
 * uniform) of the proposal it was drawn from (0 for uniform trials). */
#define ALEA_SAMPLE_ROW 5
/* Loss L = -sum_i softmax(tau l - lq)_i f_i + log mean_i exp(f_i - lq_i)
 * over one batch of host rows, and dL/dweights. */
alea_status alea_proposal_loss_grad(alea_proposal* p, const float* samples, uint64_t n,
                                    double tau, double* loss, float* grad, uint64_t n_grad);
typedef struct {
    uint32_t epochs;
    uint32_t batch;
    double lr, tau, beta1, beta2, eps;
    uint64_t seed;     /* per-epoch sample order (Philox stream 3) */
} alea_proposal_train_config;
/* Adam over n device rows (as alea_widom_samples writes them). */
alea_status alea_proposal_train(alea_proposal* p, const float* samples_device, uint64_t n,
                                const alea_proposal_train_config* config, double* final_loss,
                                void* cuda_stream);
/* P_c = (1 - uniform_share) softmax(f(centre_c)) + uniform_share / cells^3 */
alea_status alea_proposal_tabulate(alea_proposal* p, uint32_t cells, double uniform_share);
/* log of the tabulated density relative to uniform at n fractional positions (3 doubles each) */
alea_status alea_proposal_log_density(const alea_proposal* p, const double* s, uint64_t n,
                                      double* out);
alea_status alea_proposal_destroy(alea_proposal* p);

/* Widom trials as training rows (ALEA_SAMPLE_ROW floats each) written to
 * device memory: uniform trials as alea_widom_run draws them when proposal is
 * NULL (lq = 0), else trials drawn as alea_widom_run_biased draws them (lq =
 * log of the proposal's density at the position). */
alea_status alea_widom_samples(alea_widom* w, const alea_proposal* proposal, uint64_t seed,
                               uint64_t stream, uint64_t first_trial, uint64_t n_trials,
                               int32_t draw_order, float* samples_device);
/* Widom with insertion positions drawn from the tabulated proposal: trial t
 * uses Philox calls 8t (cell, from the CDF), 8t+1..8t+3 (point in the cell)
 * and 8t+4..8t+6 (orientation, several sites); its weight is
 * exp(-dU/T) / p(s) with p the density relative to uniform, so
 * henry = mean / T estimates the same K_H as the uniform method.
 * per_trial_du and per_trial_frac (3 doubles per trial) are optional. */
alea_status alea_widom_run_biased(alea_widom* w, const alea_proposal* p, uint64_t seed,
                                  uint64_t stream, uint64_t first_trial, uint64_t n_trials,
                                  alea_widom_result* out, double* per_trial_du,
                                  double* per_trial_frac);

/* A batch of Widom contexts (one per framework, each with its own force field,
 * atoms, cell and guest template) run together: one persistent launch over
 * (framework, block of 128 trials) work items and a per-framework combination,
 * replayed from a captured CUDA graph. Framework i's result equals
 * alea_widom_run on its own context with (seeds[i], streams[i]). ewald is
 * NULL (LJ only) or n entries. out holds n results. */
typedef struct alea_widom_batch alea_widom_batch;
alea_status alea_widom_batch_create(uint32_t n, const alea_lennard_jones* lj, const alea_ewald* ewald,
                                    const alea_particles* frameworks, const alea_lattice* lattices,
                                    const alea_molecule_species* guests, double temperature,
                                    int32_t precision, alea_widom_batch** out);
alea_status alea_widom_batch_run(alea_widom_batch* b, const uint64_t* seeds, const uint64_t* streams,
                                 uint64_t first_trial, uint64_t n_trials, int32_t draw_order,
                                 alea_widom_result* out, void* cuda_stream);
alea_status alea_widom_batch_destroy(alea_widom_batch* b);

/* ------------------------------------------------------------------ GCMC chains */
/* MonteCarloEngine (engines/monte_carlo/monte_carlo_engine.hpp:76-83, single
 * species, direct-scan dispersion) for n_chains independent chains at once:
 * chain c uses Philox stream (seeds[c], streams[c]) and fugacity_pa[c]
 * (PengRobinson::fugacityPascal output). ewald may be NULL (LJ only).
 * max_molecules bounds each chain's molecule count (device storage). */
typedef struct alea_gcmc alea_gcmc;
alea_status alea_gcmc_create(const alea_lennard_jones* lj, const alea_ewald* ewald,
                             const alea_particles* framework, const alea_lattice* lattice,
                             const alea_molecule_species* species, double temperature,
                             const double* fugacity_pa, const uint64_t* seeds,
                             const uint64_t* streams, uint32_t n_chains, double max_translation,
                             double max_rotation, int32_t draw_order, uint32_t max_molecules,
                             alea_gcmc** out);
/* The mixture constructor (monte_carlo_engine.hpp:143-151): n_species rigid
 * species (1..4), fugacity_pa holds n_chains x n_species values (chain-major).
 * With two or more species the move set is the reference's 5-way split with
 * identity swaps (monte_carlo_engine.cc:405-439, 673-792); with one it is
 * alea_gcmc_create. */
alea_status alea_gcmc_create_mixture(const alea_lennard_jones* lj, const alea_ewald* ewald,
                                     const alea_particles* framework, const alea_lattice* lattice,
                                     uint32_t n_species, const alea_molecule_species* species,
                                     double temperature, const double* fugacity_pa,
                                     const uint64_t* seeds, const uint64_t* streams,
                                     uint32_t n_chains, double max_translation,
                                     double max_rotation, int32_t draw_order,
                                     uint32_t max_molecules, alea_gcmc** out);
/* run(numSteps) (monte_carlo_engine.hpp:163, .cc:405-439) on every chain. */
alea_status alea_gcmc_run(alea_gcmc* g, uint64_t steps, void* cuda_stream);
typedef struct {
    uint64_t molecules;      /* moleculeCount() (monte_carlo_engine.hpp:168) */
    uint64_t guest_sites;
    uint64_t call_index;     /* Philox draws consumed so far */
    uint64_t steps;
    uint64_t resyncs;        /* S(k) rebuilds (maybeResyncEwald) */
    uint64_t attempted[5];   /* translate, rotate, insert, delete, swap */
    uint64_t accepted[5];
    uint64_t species_molecules[4]; /* moleculeCountOfSpecies(k) (monte_carlo_engine.hpp:179) */
    double sum_molecules;    /* sum over moves of the molecule count after the move */
    double sum_molecules_sq;
    double last_du;
    float last_kernel_ms;
} alea_gcmc_chain_info;
alea_status alea_gcmc_chain_info_get(const alea_gcmc* g, uint32_t chain, alea_gcmc_chain_info* out);
/* particles() positions (monte_carlo_engine.hpp:165): framework then guest
 * sites in the engine's particle order; n_out = count. */
alea_status alea_gcmc_particles(const alea_gcmc* g, uint32_t chain, double* xyz, uint64_t cap,
                                uint64_t* n_out);
/* One chain's guest sites in the engine's order: 4 doubles each (x, y, z,
 * charge) and the LJ species; when cap is below the count only n_out is set.
 * (No single reference call: the engine's particles() restricted to guests,
 * with their charges and species.) */
alea_status alea_gcmc_guest_sites(const alea_gcmc* g, uint32_t chain, double* xyzq,
                                  uint32_t* lj_species, uint64_t cap, uint64_t* n_out);
/* electrostaticEnergyForTesting() (monte_carlo_engine.hpp:214, .cc:928-930). */
alea_status alea_gcmc_ewald_energy(const alea_gcmc* g, uint32_t chain, double* out);
alea_status alea_gcmc_destroy(alea_gcmc* g);
/* Insertions and deletions of every chain from the next run on use the
 * tabulated learned proposal (its table is copied): the insertion's centroid
 * is drawn from it (Philox draws: move pick, cell, 3 in-cell, 3 orientation,
 * accept) with the template centred on its centroid, and the acceptance
 * ratios carry 1/p(centroid) (insertion) and p(centroid) (deletion), p the
 * density relative to uniform, so detailed balance holds. NULL restores the
 * reference's uniform insertion. Declared after alea_proposal below. */
struct alea_proposal;
alea_status alea_gcmc_set_proposal(alea_gcmc* g, const struct alea_proposal* p);
/* The chains' energy form from the next run on: ALEA_FP64 (default; the
 * reference's arithmetic, trajectories equal to the reference's) or ALEA_FP32
 * (LJ and real-space pair terms in FP32 after a double-float minimum image,
 * pairs closer than sigma and Coulomb pairs within 6 A in double-float,
 * per-term S(k) deltas from FP32 phases; the sums and S(k) in double-float or
 * FP64, the self and exclusion terms and the acceptance in FP64; up to 8
 * orientation trials of a biased move in one energy pass). ALEA_FP32 needs
 * framework atoms + max_molecules x sites below 2^24 (else
 * ALEA_ERR_INVALID_ARGUMENT). No counterpart in the reference. */
alea_status alea_gcmc_set_precision(alea_gcmc* g, int32_t precision);
/* MonteCarloEngine's frameworkEnergyGrid (monte_carlo_engine.hpp:76-83,
 * .cc:341-374): from the next run on, a site's dispersion energy is its LJ
 * species' table interpolated at the site plus the LJ with the guests (the
 * framework atoms are then visited only for real-space Ewald). The grid is
 * borrowed: it must stay alive while the chains run. Its cell must be the
 * chains', with a table for every site species (else ALEA_ERR_OUT_OF_RANGE).
 * NULL restores the direct scan. */
alea_status alea_gcmc_set_grid(alea_gcmc* g, const alea_grid* grid);
/* Opt-in LJ tail correction of particle-number moves. The reference engine
 * leaves it out of every move (its tailEnergyCorrection, lennard_jones.cc:
 * 246-257, is a whole-system energy); with on != 0 each insertion, deletion
 * and identity swap of the next runs adds U_tail(after) - U_tail(before) to
 * its deltaU, U_tail being tailEnergyCorrection over every particle of the
 * chain (framework and guests). Off by default. */
alea_status alea_gcmc_set_tail_correction(alea_gcmc* g, int32_t on);
/* Orientation-biased insertion and deletion of multi-site molecules (no
 * counterpart in the reference engine, which inserts with one random
 * orientation, monte_carlo_engine.cc:572-579): with k > 1 an insertion
 * evaluates k random orientations about the drawn centroid, keeps one with
 * probability exp(-dU_j/T) / W and is accepted with W / k in place of
 * exp(-dU/T) (gcmc_acceptance.hpp:28-44); a deletion evaluates the molecule's
 * own orientation and k - 1 random ones about its centroid and uses k / W in
 * place of exp(+U/T). Composes with the learned proposal (the centroid's
 * density) and the tail correction. k = 1 (the default) is the reference's
 * move; 1 <= k <= 16. */
alea_status alea_gcmc_set_orientation_trials(alea_gcmc* g, int32_t k);
/* The same for Widom insertions: every trial's deltaU gains the constant
 * U_tail(framework + molecule) - U_tail(framework), written to *du_tail (may
 * be NULL) whatever `on` is; K_H is multiplied by exp(-du_tail / T). Single
 * contexts only (alea_widom_run, alea_widom_run_biased); off by default. */
alea_status alea_widom_set_tail_correction(alea_widom* w, int32_t on, double* du_tail);

/* ------------------------------------------------------------------ acceptance / EOS (host) */
/* gcmc::insertionRatio ... clampToProbability (engines/monte_carlo/gcmc_acceptance.hpp:28-101) */
double alea_insertion_ratio(double f, double v, uint64_t n_before, double t, double du);
double alea_deletion_ratio(double f, double v, uint64_t n_before, double t, double du);
double alea_metropolis_ratio(double t, double du);
double alea_swap_ratio(double f_from, double f_to, uint64_t n_from, uint64_t n_to, double t,
                       double du);
/* PengRobinson::fugacityPascal (engines/monte_carlo/peng_robinson.cc:108-110) */
alea_status alea_peng_robinson_fugacity(double tc, double pc, double omega, double t, double p,
                                        double* out);
/* PengRobinsonMixture(substances, binaryInteractionKij).fugacitiesPascal and
 * .compressibilityFactor (engines/monte_carlo/peng_robinson.hpp:127-155,
 * peng_robinson.cc:112-309): n >= 2 substances (tc, pc, omega), kij an n x n
 * row-major matrix (symmetric, zero diagonal) or NULL for every k_ij = 0,
 * mole fractions x summing to 1. f_out[i] = x_i phi_i P (Pa); z_out (may be
 * NULL) the mixture's compressibility factor. */
alea_status alea_peng_robinson_mixture(uint32_t n, const double* tc, const double* pc,
                                       const double* omega, const double* kij, double t, double p,
                                       const double* x, double* z_out, double* f_out);

#ifdef __cplusplus
}
#endif
#endif /* ALEATOR_GB300_H */
