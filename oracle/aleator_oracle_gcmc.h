/*
 * ORACLE — test infrastructure, not product code. Single-species GCMC chain
 * restated from MonteCarloEngine (engines/monte_carlo/monte_carlo_engine.cc).
 */
#ifndef ALEATOR_ORACLE_GCMC_H
#define ALEATOR_ORACLE_GCMC_H

#include "aleator_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    orc_lj lj;
    uint32_t n_lj;
    double* eps;
    double* sigma;
    orc_ewald_params ew;
    double m[9];
    uint32_t ns;
    double gx[16], gy[16], gz[16], gq[16];
    uint32_t glj[16];
    double temperature, fugacity, max_translation, max_rotation;
    uint64_t seed, stream, call;
    int draw_order;
    uint64_t n_fw, n, cap;
    double *x, *y, *z, *q;
    uint32_t* sp;
    uint64_t n_mol, mol_cap;
    uint64_t* mol; /* n_mol x ns site indices */
    int charged;
    orc_ewald_state ews;
    uint64_t moves_since_resync, resyncs, steps;
    uint64_t attempted[4], accepted[4];
    double last_du;
    /* optional energy grid (tables borrowed, one per LJ species or NULL) */
    int grid;
    int gcounts[3];
    const double* gtab[64];
} orc_gcmc;

int orc_gcmc_create(orc_gcmc* g, const orc_lj* lj, const orc_ewald_params* ew, const double m[9],
                    uint64_t n, const double* x, const double* y, const double* z, const double* q,
                    const uint32_t* species, const orc_species* guest, double temperature,
                    double fugacity_pa, double max_translation, double max_rotation,
                    uint64_t seed, uint64_t stream, int draw_order);
void orc_gcmc_run(orc_gcmc* g, uint64_t steps);
double orc_gcmc_ewald_energy(const orc_gcmc* g);
void orc_gcmc_free(orc_gcmc* g);
orc_gcmc* orc_gcmc_new(const orc_lj* lj, const orc_ewald_params* ew, const double m[9], uint64_t n,
                       const double* x, const double* y, const double* z, const double* q,
                       const uint32_t* species, const orc_species* guest, double temperature,
                       double fugacity_pa, double max_translation, double max_rotation,
                       uint64_t seed, uint64_t stream, int draw_order);
void orc_gcmc_delete(orc_gcmc* g);
uint64_t orc_gcmc_molecules(const orc_gcmc* g);
uint64_t orc_gcmc_particles(const orc_gcmc* g, double* xyz, uint64_t cap);
uint64_t orc_gcmc_calls(const orc_gcmc* g);
void orc_gcmc_counters(const orc_gcmc* g, uint64_t* out8);
/* MonteCarloEngine's frameworkEnergyGrid: per-species tables of a grid with
 * `counts` nodes on the chain's cell (borrowed; NULL entries for species
 * without a table); n_tables == 0 removes it. */
void orc_gcmc_set_grid(orc_gcmc* g, const int counts[3], uint32_t n_tables, const uint32_t* species,
                       const double* const* tables);

#ifdef __cplusplus
}
#endif
#endif
