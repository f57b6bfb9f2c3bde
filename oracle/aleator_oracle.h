/*
 * ORACLE — test infrastructure, not product code.
 *
 * A plain-C, FP64, single-threaded restatement of the reference engine's
 * grand-canonical Monte Carlo energy hot path (Defalt-Meh/aleator), used only
 * as the checker: by tests/, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline leg. Each function cites the reference file:line it follows. The
 * restatement keeps the reference's operation order so that on one host it
 * reproduces the reference bit-for-bit; it is pinned against the reference
 * itself (oracle/_ref, built from the reference sources by oracle/build_ref.sh)
 * and against the golden vectors in tests/golden/.
 *
 * Lattice matrices are row-major double[9], row i = lattice vector a_i (Å).
 */
#ifndef ALEATOR_ORACLE_H
#define ALEATOR_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Argument evaluation order of the reference's nested RNG draws
 * (monte_carlo_engine.cc:572-574, 578-579, 882-888): C++ leaves it
 * unspecified. GCC evaluates right to left, clang left to right. */
enum { ORC_DRAWS_RIGHT_TO_LEFT = 0, ORC_DRAWS_LEFT_TO_RIGHT = 1 };

/* ---- Philox4x32-10 (counter_based_rng.cc:13-79) ---- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
uint64_t orc_philox_u64(uint64_t seed, uint64_t stream, uint64_t call_index);
double orc_philox_uniform(uint64_t seed, uint64_t stream, uint64_t call_index);
void orc_philox_fill_u64(uint64_t seed, uint64_t stream, uint64_t first, uint64_t n, uint64_t* out);
void orc_philox_fill_uniform(uint64_t seed, uint64_t stream, uint64_t first, uint64_t n, double* out);

/* ---- Lattice (lattice.hpp:35-41, lattice.cc:115-284) ---- */
double orc_volume(const double m[9]);
double orc_perpendicular_width(const double m[9], int axis);
int orc_is_orthorhombic(const double m[9]);
void orc_reduced_basis(const double m[9], double out[9]);
void orc_frac_to_cart(const double m[9], const double f[3], double out[3]);
void orc_cart_to_frac(const double m[9], const double c[3], double out[3]);
void orc_min_image(const double m[9], const double a[3], const double b[3], double out[3]);
void orc_supercell_replication(const double m[9], double cutoff, int out[3]);

/* ---- Lennard-Jones (lennard_jones.cc:15-86, 158-257) ---- */
enum { ORC_TRUNCATED = 0, ORC_SHIFTED = 1, ORC_LINEAR_FORCE_SHIFTED = 2 };
enum { ORC_LORENTZ_BERTHELOT = 0, ORC_GEOMETRIC = 1 };
typedef struct {
    uint32_t n_species;
    const double* eps;   /* per species, K */
    const double* sigma; /* per species, Å */
    double cutoff;
    int truncation;
    int mixing;
} orc_lj;
void orc_lj_mixed(const orc_lj* lj, uint32_t i, uint32_t j, double* eps, double* sigma);
double orc_lj_pair_energy(const orc_lj* lj, double r, double eps, double sigma);
/* sum over j != index, j not in excluded, ascending j */
double orc_lj_particle_energy(const orc_lj* lj, const double m[9], uint64_t n, const double* x,
                              const double* y, const double* z, const uint32_t* species,
                              uint64_t index, const uint64_t* excluded, uint64_t n_excluded);
double orc_lj_tail(const orc_lj* lj, const double m[9], uint64_t n, const uint32_t* species);

/* ---- Framework energy grid (framework_energy_grid.cc:193-288) ---- */
#define ORC_GRID_ENERGY_CAP 1.0e5
void orc_grid_point_counts(const double m[9], double spacing, int out[3]);
/* Node energies for one guest species over nodes [node_begin, node_end) of
 * the flat (iz*ny+iy)*nx+ix order, using n_threads host threads. */
void orc_grid_build_nodes(const orc_lj* lj, const double m[9], uint64_t n_atoms, const double* x,
                          const double* y, const double* z, const uint32_t* species,
                          uint32_t guest, double spacing, uint64_t node_begin, uint64_t node_end,
                          int n_threads, double* out);
double orc_grid_interpolate(const double m[9], const int counts[3], const double* table,
                            const double pos[3]);

/* ---- Ewald (ewald.cc:29-313) ---- */
#define ORC_COULOMB_K 167100.9468982874
uint64_t orc_ewald_terms(const double m[9], double alpha, int kmax, double* k, double* w,
                         uint64_t cap);
double orc_ewald_real_space_particle_energy(const double m[9], uint64_t n, const double* x,
                                            const double* y, const double* z, const double* q,
                                            double alpha, double rc, uint64_t index,
                                            const uint64_t* excluded, uint64_t n_excluded);
/* out = {real, reciprocal, self, exclusion, surface}; exclusions as index pairs */
void orc_ewald_breakdown(const double m[9], uint64_t n, const double* x, const double* y,
                         const double* z, const double* q, double alpha, double rc, int kmax,
                         const uint64_t* exclusions, uint64_t n_excl, double out[5]);

/* ---- EwaldIncrementalState (ewald_incremental_state.cc:24-257) ---- */
typedef struct {
    double m[9];
    double alpha;
    double volume;
    uint64_t nk;
    double* k;  /* 3*nk */
    double* w;  /* nk */
    double* sre;
    double* sim;
    double self_energy;
    double exclusion_energy;
} orc_ewald_state;
/* sites are packed {x, y, z, q} */
int orc_ews_init(orc_ewald_state* s, const double m[9], double alpha, int kmax, uint64_t n,
                 const double* x, const double* y, const double* z, const double* q);
void orc_ews_free(orc_ewald_state* s);
double orc_ews_energy(const orc_ewald_state* s);
/* delta for (removed -> added); if dre/dim non-NULL they receive the per-k delta */
double orc_ews_delta(const orc_ewald_state* s, const double* removed, uint64_t nr,
                     const double* added, uint64_t na, double* dre, double* dim, double* dself,
                     double* dexcl);
void orc_ews_commit(orc_ewald_state* s, const double* removed, uint64_t nr, const double* added,
                    uint64_t na);
double orc_ews_recompute(const orc_ewald_state* s, uint64_t n, const double* x, const double* y,
                         const double* z, const double* q, uint64_t n_mol,
                         const uint64_t* offsets, const uint64_t* indices);
void orc_ews_resync(orc_ewald_state* s, uint64_t n, const double* x, const double* y,
                    const double* z, const double* q, uint64_t n_mol, const uint64_t* offsets,
                    const uint64_t* indices);

/* ---- Rigid molecules and Widom (monte_carlo_engine.cc:40-72, 850-917) ---- */
typedef struct {
    uint32_t n_sites;
    const double* x; /* local frame, Å */
    const double* y;
    const double* z;
    const uint32_t* lj_species;
    const double* charge;
} orc_species;
void orc_random_unit_quaternion(double u0, double u1, double u2, double q[4]);
void orc_rotate_by_quaternion(const double v[3], const double q[4], double out[3]);
void orc_rotate_about_axis(const double v[3], const double axis[3], double theta, double out[3]);
typedef struct {
    double alpha;   /* <= 0: no electrostatics */
    double rc;      /* real-space cutoff */
    int kmax;
} orc_ewald_params;
/* Returns K_H; per_trial (optional) receives each trial's deltaU in K.
 * Trials [first_trial, first_trial + n_trials) of the stream (seed, stream). */
double orc_widom(const orc_lj* lj, const orc_ewald_params* ew, const double m[9], uint64_t n,
                 const double* x, const double* y, const double* z, const double* q,
                 const uint32_t* species, const orc_species* guest, double temperature,
                 uint64_t seed, uint64_t stream, uint64_t first_trial, uint64_t n_trials,
                 int draw_order, int n_threads, double* per_trial);

/* ---- Acceptance rules (gcmc_acceptance.hpp:28-101) ---- */
double orc_insertion_ratio(double f, double v, uint64_t n_before, double t, double du);
double orc_deletion_ratio(double f, double v, uint64_t n_before, double t, double du);
double orc_metropolis_ratio(double t, double du);
double orc_swap_ratio(double f_from, double f_to, uint64_t n_from, uint64_t n_to, double t,
                      double du);
double orc_clamp_probability(double r);
#define ORC_PASCAL_TO_INTERNAL (1.0 / (1.380649e-23 * 1.0e30))

/* ---- Peng-Robinson (peng_robinson.cc:10-110) ---- */
double orc_pr_fugacity(double tc, double pc, double omega, double t, double p);
/* PengRobinsonMixture::compressibilityFactor / fugacitiesPascal
 * (peng_robinson.cc:112-309); kij n x n row-major or NULL. Returns 0, or -1
 * for an argument the reference rejects. */
int orc_pr_mixture(uint32_t n, const double* tc, const double* pc, const double* omega,
                   const double* kij, double t, double p, const double* x, double* z_out,
                   double* f_out);

#ifdef __cplusplus
}
#endif
#endif
