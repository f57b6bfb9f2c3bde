/*
 * ORACLE — test infrastructure, not product code. GCMC chain (one or several
 * rigid species) restated from MonteCarloEngine
 * (engines/monte_carlo/monte_carlo_engine.cc).
 */
#ifndef ALEATOR_ORACLE_GCMC_H
#define ALEATOR_ORACLE_GCMC_H

#include "aleator_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_SPECIES 8
#define ORC_MOLW 16 /* molecule record stride: sites per molecule at most */

typedef struct {
    uint32_t ns;
    double x[ORC_MOLW], y[ORC_MOLW], z[ORC_MOLW], q[ORC_MOLW];
    double cx[ORC_MOLW], cy[ORC_MOLW], cz[ORC_MOLW]; /* the template about its centroid */
    uint32_t lj[ORC_MOLW];
    double fugacity; /* K / Å^3 */
} orc_gcmc_species;

typedef struct {
    orc_lj lj;
    uint32_t n_lj;
    double* eps;
    double* sigma;
    orc_ewald_params ew;
    double m[9];
    uint32_t n_species;
    orc_gcmc_species spc[ORC_MAX_SPECIES];
    double temperature, max_translation, max_rotation;
    uint64_t seed, stream, call;
    int draw_order;
    uint64_t n_fw, n, cap;
    double *x, *y, *z, *q;
    uint32_t* sp;
    uint64_t n_mol, mol_cap;
    uint64_t* mol;     /* n_mol x ORC_MOLW site indices */
    uint32_t* mol_sp;  /* species of each molecule */
    int charged;
    orc_ewald_state ews;
    uint64_t moves_since_resync, resyncs, steps;
    uint64_t attempted[5], accepted[5]; /* translate, rotate, insert, delete, swap */
    double last_du;
    /* opt-in (no counterpart in the reference engine): insertions, deletions
     * and swaps add U_tail(after) - U_tail(before), tailEnergyCorrection over
     * every particle (lennard_jones.cc:246-257) */
    int tail;
    /* opt-in (no counterpart in the reference engine): orientation-biased
     * insertion and deletion with `orient` trial orientations (1: the
     * reference's moves) */
    int orient;
    /* optional energy grid (tables borrowed, one per LJ species or NULL) */
    int grid;
    int gcounts[3];
    const double* gtab[64];
} orc_gcmc;

int orc_gcmc_create(orc_gcmc* g, const orc_lj* lj, const orc_ewald_params* ew, const double m[9],
                    uint64_t n, const double* x, const double* y, const double* z, const double* q,
                    const uint32_t* species, uint32_t n_species, const orc_species* guests,
                    double temperature, const double* fugacity_pa, double max_translation,
                    double max_rotation, uint64_t seed, uint64_t stream, int draw_order);
void orc_gcmc_run(orc_gcmc* g, uint64_t steps);
double orc_gcmc_ewald_energy(const orc_gcmc* g);
void orc_gcmc_free(orc_gcmc* g);
/* one species (MonteCarloEngine's single-species constructor) */
orc_gcmc* orc_gcmc_new(const orc_lj* lj, const orc_ewald_params* ew, const double m[9], uint64_t n,
                       const double* x, const double* y, const double* z, const double* q,
                       const uint32_t* species, const orc_species* guest, double temperature,
                       double fugacity_pa, double max_translation, double max_rotation,
                       uint64_t seed, uint64_t stream, int draw_order);
/* several species (the mixture constructor) */
orc_gcmc* orc_gcmc_new_mixture(const orc_lj* lj, const orc_ewald_params* ew, const double m[9],
                               uint64_t n, const double* x, const double* y, const double* z,
                               const double* q, const uint32_t* species, uint32_t n_species,
                               const orc_species* guests, double temperature,
                               const double* fugacity_pa, double max_translation,
                               double max_rotation, uint64_t seed, uint64_t stream,
                               int draw_order);
void orc_gcmc_delete(orc_gcmc* g);
uint64_t orc_gcmc_molecules(const orc_gcmc* g);
uint64_t orc_gcmc_molecules_of(const orc_gcmc* g, uint32_t species);
uint64_t orc_gcmc_particles(const orc_gcmc* g, double* xyz, uint64_t cap);
uint64_t orc_gcmc_calls(const orc_gcmc* g);
void orc_gcmc_counters(const orc_gcmc* g, uint64_t* out10);
/* MonteCarloEngine's frameworkEnergyGrid: per-species tables of a grid with
 * `counts` nodes on the chain's cell (borrowed; NULL entries for species
 * without a table); n_tables == 0 removes it. */
/* the opt-in tail-correction change of insertions, deletions and swaps */
void orc_gcmc_set_tail(orc_gcmc* g, int on);
/* orientation-biased insertion and deletion with k trials (1 <= k <= 16) */
void orc_gcmc_set_orientation_trials(orc_gcmc* g, int k);
void orc_gcmc_set_grid(orc_gcmc* g, const int counts[3], uint32_t n_tables, const uint32_t* species,
                       const double* const* tables);

#ifdef __cplusplus
}
#endif
#endif
