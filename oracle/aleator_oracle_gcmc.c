/*
 * ORACLE — test infrastructure, not product code.
 *
 * Plain-C restatement of MonteCarloEngine's single-species GCMC chain
 * (engines/monte_carlo/monte_carlo_engine.cc:159-439 run, :441-671 moves,
 * :814-848 removal), FP64, in the reference's operation order. The
 * reference's guest-guest cell-list candidates are a superset of the guests
 * within the cutoff visited in ascending index order (monte_carlo_engine.cc:
 * 316-374), and pairEnergy beyond the cutoff is exactly 0.0, so an ascending
 * scan gives the same sums bit for bit; this port scans. Without an energy
 * grid the scan covers every particle (framework first); with one, a site's
 * dispersion is the grid's interpolation plus the scan over guests only
 * (monte_carlo_engine.cc:353-372).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "aleator_oracle.h"
#include "aleator_oracle_gcmc.h"

#define ORC_PI 3.14159265358979323846

static double u01(orc_gcmc* g) { return orc_philox_uniform(g->seed, g->stream, g->call++); }

static void ensure_capacity(orc_gcmc* g, uint64_t need) {
    if (need <= g->cap) return;
    uint64_t cap = g->cap ? g->cap : 64;
    while (cap < need) cap *= 2;
    g->x = (double*)realloc(g->x, sizeof(double) * cap);
    g->y = (double*)realloc(g->y, sizeof(double) * cap);
    g->z = (double*)realloc(g->z, sizeof(double) * cap);
    g->q = (double*)realloc(g->q, sizeof(double) * cap);
    g->sp = (uint32_t*)realloc(g->sp, sizeof(uint32_t) * cap);
    g->cap = cap;
}

static void ensure_mol_capacity(orc_gcmc* g, uint64_t need) {
    if (need <= g->mol_cap) return;
    uint64_t cap = g->mol_cap ? g->mol_cap : 16;
    while (cap < need) cap *= 2;
    g->mol = (uint64_t*)realloc(g->mol, sizeof(uint64_t) * cap * g->ns);
    g->mol_cap = cap;
}

int orc_gcmc_create(orc_gcmc* g, const orc_lj* lj, const orc_ewald_params* ew, const double m[9],
                    uint64_t n, const double* x, const double* y, const double* z, const double* q,
                    const uint32_t* species, const orc_species* guest, double temperature,
                    double fugacity_pa, double max_translation, double max_rotation,
                    uint64_t seed, uint64_t stream, int draw_order) {
    memset(g, 0, sizeof(*g));
    g->n_lj = lj->n_species;
    g->eps = (double*)malloc(sizeof(double) * lj->n_species);
    g->sigma = (double*)malloc(sizeof(double) * lj->n_species);
    memcpy(g->eps, lj->eps, sizeof(double) * lj->n_species);
    memcpy(g->sigma, lj->sigma, sizeof(double) * lj->n_species);
    g->lj = *lj;
    g->lj.eps = g->eps;
    g->lj.sigma = g->sigma;
    if (ew) g->ew = *ew;
    memcpy(g->m, m, sizeof(double) * 9);
    g->ns = guest->n_sites;
    for (uint32_t s = 0; s < g->ns && s < 16; ++s) {
        g->gx[s] = guest->x[s];
        g->gy[s] = guest->y[s];
        g->gz[s] = guest->z[s];
        g->glj[s] = guest->lj_species[s];
        g->gq[s] = guest->charge[s];
    }
    g->temperature = temperature;
    g->fugacity = fugacity_pa * ORC_PASCAL_TO_INTERNAL;  /* monte_carlo_engine.cc:212-219 */
    g->max_translation = max_translation;
    g->max_rotation = max_rotation;
    g->seed = seed;
    g->stream = stream;
    g->draw_order = draw_order;
    g->n_fw = n;
    ensure_capacity(g, n + 64);
    memcpy(g->x, x, sizeof(double) * n);
    memcpy(g->y, y, sizeof(double) * n);
    memcpy(g->z, z, sizeof(double) * n);
    for (uint64_t i = 0; i < n; ++i) {
        g->q[i] = q ? q[i] : 0.0;
        g->sp[i] = species ? species[i] : 0u;
    }
    g->n = n;
    g->charged = ew && ew->alpha > 0.0;
    if (g->charged) orc_ews_init(&g->ews, m, ew->alpha, ew->kmax, n, g->x, g->y, g->z, g->q);
    return 0;
}

void orc_gcmc_free(orc_gcmc* g) {
    free(g->x);
    free(g->y);
    free(g->z);
    free(g->q);
    free(g->sp);
    free(g->mol);
    free(g->eps);
    free(g->sigma);
    if (g->charged) orc_ews_free(&g->ews);
    memset(g, 0, sizeof(*g));
}

/* computeParticleEnergyOverCandidates over the guests (indices from n_fw),
 * ascending (lennard_jones.cc:179-209) */
static double lj_over_guests(orc_gcmc* g, uint64_t index, const uint64_t* excluded, uint32_t n_ex) {
    double energy = 0.0;
    const double pi[3] = {g->x[index], g->y[index], g->z[index]};
    for (uint64_t j = g->n_fw; j < g->n; ++j) {
        if (j == index) continue;
        int ex = 0;
        for (uint32_t k = 0; k < n_ex; ++k) ex |= excluded[k] == j;
        if (ex) continue;
        double eps, sigma;
        orc_lj_mixed(&g->lj, g->sp[index], g->sp[j], &eps, &sigma);
        const double pj[3] = {g->x[j], g->y[j], g->z[j]};
        double d[3];
        orc_min_image(g->m, pi, pj, d);
        energy += orc_lj_pair_energy(&g->lj, sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]), eps, sigma);
    }
    return energy;
}

/* moleculeDispersionEnergy + moleculeElectrostaticRealSpaceEnergy
 * (monte_carlo_engine.cc:299-314, 341-374) */
static double dispersion(orc_gcmc* g, const uint64_t* idx) {
    double e = 0.0;
    for (uint32_t s = 0; s < g->ns; ++s) {
        if (g->grid) {
            const double p[3] = {g->x[idx[s]], g->y[idx[s]], g->z[idx[s]]};
            e += orc_grid_interpolate(g->m, g->gcounts, g->gtab[g->sp[idx[s]]], p);
            e += lj_over_guests(g, idx[s], idx, g->ns);
        } else {
            e += orc_lj_particle_energy(&g->lj, g->m, g->n, g->x, g->y, g->z, g->sp, idx[s], idx, g->ns);
        }
    }
    return e;
}

void orc_gcmc_set_grid(orc_gcmc* g, const int counts[3], uint32_t n_tables, const uint32_t* species,
                       const double* const* tables) {
    g->grid = n_tables > 0;
    for (int i = 0; i < 64; ++i) g->gtab[i] = NULL;
    for (int a = 0; a < 3; ++a) g->gcounts[a] = counts ? counts[a] : 0;
    for (uint32_t i = 0; i < n_tables; ++i)
        if (species[i] < 64) g->gtab[species[i]] = tables[i];
}

static double electro_real(orc_gcmc* g, const uint64_t* idx) {
    if (!g->charged) return 0.0;
    double e = 0.0;
    for (uint32_t s = 0; s < g->ns; ++s)
        e += orc_ewald_real_space_particle_energy(g->m, g->n, g->x, g->y, g->z, g->q, g->ew.alpha,
                                                  g->ew.rc, idx[s], idx, g->ns);
    return e;
}

static void pack_sites(orc_gcmc* g, const uint64_t* idx, double* out) {
    for (uint32_t s = 0; s < g->ns; ++s) {
        out[4 * s] = g->x[idx[s]];
        out[4 * s + 1] = g->y[idx[s]];
        out[4 * s + 2] = g->z[idx[s]];
        out[4 * s + 3] = g->q[idx[s]];
    }
}

/* maybeResyncEwald (monte_carlo_engine.cc:380-403) */
static void maybe_resync(orc_gcmc* g) {
    if (!g->charged) return;
    g->moves_since_resync++;
    if (g->moves_since_resync >= 100) {
        uint64_t* offs = (uint64_t*)malloc(sizeof(uint64_t) * (g->n_mol + 1));
        for (uint64_t k = 0; k <= g->n_mol; ++k) offs[k] = k * g->ns;
        orc_ews_resync(&g->ews, g->n, g->x, g->y, g->z, g->q, g->n_mol, offs,
                       g->n_mol ? g->mol : offs);
        free(offs);
        g->moves_since_resync = 0;
        g->resyncs++;
    }
}

static int accept(orc_gcmc* g, double ratio) { return u01(g) < orc_clamp_probability(ratio); }

/* attemptTranslation (monte_carlo_engine.cc:441-484) */
static void attempt_translation(orc_gcmc* g) {
    if (g->n_mol == 0) return;
    const uint64_t mi = (uint64_t)(u01(g) * (double)g->n_mol);
    const uint64_t* idx = g->mol + mi * g->ns;
    g->attempted[0]++;
    const double u_before = dispersion(g, idx);
    const double e_before = electro_real(g, idx);
    double old_s[64], new_s[64], orig[48];
    if (g->charged) pack_sites(g, idx, old_s);
    const double d0 = (2.0 * u01(g) - 1.0) * g->max_translation;
    const double d1 = (2.0 * u01(g) - 1.0) * g->max_translation;
    const double d2 = (2.0 * u01(g) - 1.0) * g->max_translation;
    for (uint32_t s = 0; s < g->ns; ++s) {
        const uint64_t i = idx[s];
        orig[3 * s] = g->x[i];
        orig[3 * s + 1] = g->y[i];
        orig[3 * s + 2] = g->z[i];
        g->x[i] = orig[3 * s] + d0;
        g->y[i] = orig[3 * s + 1] + d1;
        g->z[i] = orig[3 * s + 2] + d2;
    }
    const double u_after = dispersion(g, idx);
    const double e_after = electro_real(g, idx);
    double rec = 0.0;
    if (g->charged) {
        pack_sites(g, idx, new_s);
        rec = orc_ews_delta(&g->ews, old_s, g->ns, new_s, g->ns, NULL, NULL, NULL, NULL);
    }
    const double du = (u_after - u_before) + (e_after - e_before) + rec;
    g->last_du = du;
    if (accept(g, orc_metropolis_ratio(g->temperature, du))) {
        if (g->charged) {
            orc_ews_commit(&g->ews, old_s, g->ns, new_s, g->ns);
            maybe_resync(g);
        }
        g->accepted[0]++;
        return;
    }
    for (uint32_t s = 0; s < g->ns; ++s) {
        const uint64_t i = idx[s];
        g->x[i] = orig[3 * s];
        g->y[i] = orig[3 * s + 1];
        g->z[i] = orig[3 * s + 2];
    }
}

/* attemptRotation (monte_carlo_engine.cc:486-554) */
static void attempt_rotation(orc_gcmc* g) {
    if (g->n_mol == 0) return;
    if (g->ns < 2) return; /* single species, single site: no draw */
    const uint64_t mi = (uint64_t)(u01(g) * (double)g->n_mol);
    const uint64_t* idx = g->mol + mi * g->ns;
    g->attempted[1]++;
    const double u_before = dispersion(g, idx);
    const double e_before = electro_real(g, idx);
    double old_s[64], new_s[64], orig[48];
    if (g->charged) pack_sites(g, idx, old_s);
    double c[3] = {0.0, 0.0, 0.0};
    for (uint32_t s = 0; s < g->ns; ++s) {
        c[0] = c[0] + g->x[idx[s]];
        c[1] = c[1] + g->y[idx[s]];
        c[2] = c[2] + g->z[idx[s]];
    }
    const double inv = 1.0 / (double)g->ns;
    c[0] = c[0] * inv;
    c[1] = c[1] * inv;
    c[2] = c[2] * inv;
    const double cos_t = 2.0 * u01(g) - 1.0;
    const double sin_t = sqrt(fmax(0.0, 1.0 - cos_t * cos_t));
    const double phi = 2.0 * ORC_PI * u01(g);
    const double axis[3] = {sin_t * cos(phi), sin_t * sin(phi), cos_t};
    const double angle = (2.0 * u01(g) - 1.0) * g->max_rotation;
    for (uint32_t s = 0; s < g->ns; ++s) {
        const uint64_t i = idx[s];
        orig[3 * s] = g->x[i];
        orig[3 * s + 1] = g->y[i];
        orig[3 * s + 2] = g->z[i];
        const double v[3] = {g->x[i] - c[0], g->y[i] - c[1], g->z[i] - c[2]};
        double r[3];
        orc_rotate_about_axis(v, axis, angle, r);
        g->x[i] = c[0] + r[0];
        g->y[i] = c[1] + r[1];
        g->z[i] = c[2] + r[2];
    }
    const double u_after = dispersion(g, idx);
    const double e_after = electro_real(g, idx);
    double rec = 0.0;
    if (g->charged) {
        pack_sites(g, idx, new_s);
        rec = orc_ews_delta(&g->ews, old_s, g->ns, new_s, g->ns, NULL, NULL, NULL, NULL);
    }
    const double du = (u_after - u_before) + (e_after - e_before) + rec;
    g->last_du = du;
    if (accept(g, orc_metropolis_ratio(g->temperature, du))) {
        if (g->charged) {
            orc_ews_commit(&g->ews, old_s, g->ns, new_s, g->ns);
            maybe_resync(g);
        }
        g->accepted[1]++;
        return;
    }
    for (uint32_t s = 0; s < g->ns; ++s) {
        const uint64_t i = idx[s];
        g->x[i] = orig[3 * s];
        g->y[i] = orig[3 * s + 1];
        g->z[i] = orig[3 * s + 2];
    }
}

/* attemptInsertion (monte_carlo_engine.cc:556-619), single species */
static void attempt_insertion(orc_gcmc* g) {
    g->attempted[2]++;
    const double* m = g->m;
    double u[3];
    u[0] = u01(g);
    u[1] = u01(g);
    u[2] = u01(g);
    if (g->draw_order == ORC_DRAWS_RIGHT_TO_LEFT) {
        const double t = u[0];
        u[0] = u[2];
        u[2] = t;
    }
    double ref[3];
    for (int c = 0; c < 3; ++c) ref[c] = (m[c] * u[0] + m[3 + c] * u[1]) + m[6 + c] * u[2];
    double quat[4] = {1.0, 0.0, 0.0, 0.0};
    if (g->ns > 1) {
        double v[3];
        v[0] = u01(g);
        v[1] = u01(g);
        v[2] = u01(g);
        if (g->draw_order == ORC_DRAWS_RIGHT_TO_LEFT) {
            const double t = v[0];
            v[0] = v[2];
            v[2] = t;
        }
        orc_random_unit_quaternion(v[0], v[1], v[2], quat);
    }
    ensure_capacity(g, g->n + g->ns);
    uint64_t idx[16];
    for (uint32_t s = 0; s < g->ns; ++s) {
        const double local[3] = {g->gx[s], g->gy[s], g->gz[s]};
        double rot[3] = {local[0], local[1], local[2]};
        if (g->ns > 1) orc_rotate_by_quaternion(local, quat, rot);
        const uint64_t k = g->n++;
        g->x[k] = ref[0] + rot[0];
        g->y[k] = ref[1] + rot[1];
        g->z[k] = ref[2] + rot[2];
        g->q[k] = g->gq[s];
        g->sp[k] = g->glj[s];
        idx[s] = k;
    }
    const double disp = dispersion(g, idx);
    const double elec = electro_real(g, idx);
    double new_s[64];
    double rec = 0.0;
    if (g->charged) {
        pack_sites(g, idx, new_s);
        rec = orc_ews_delta(&g->ews, NULL, 0, new_s, g->ns, NULL, NULL, NULL, NULL);
    }
    const double du = disp + elec + rec;
    g->last_du = du;
    const double volume = fabs(orc_volume(m));
    const double ratio = orc_insertion_ratio(g->fugacity, volume, g->n_mol, g->temperature, du);
    if (accept(g, ratio)) {
        if (g->charged) orc_ews_commit(&g->ews, NULL, 0, new_s, g->ns);
        ensure_mol_capacity(g, g->n_mol + 1);
        memcpy(g->mol + g->n_mol * g->ns, idx, sizeof(uint64_t) * g->ns);
        g->n_mol++;
        maybe_resync(g);
        g->accepted[2]++;
        return;
    }
    g->n -= g->ns;
}

/* removeParticleIndices (monte_carlo_engine.cc:825-848) */
static void remove_particle_indices(orc_gcmc* g, uint64_t* indices, uint32_t count) {
    for (uint32_t k = 0; k < count; ++k) {
        const uint64_t site = indices[k];
        const uint64_t last = g->n - 1;
        if (site != last) {
            g->x[site] = g->x[last];
            g->y[site] = g->y[last];
            g->z[site] = g->z[last];
            g->q[site] = g->q[last];
            g->sp[site] = g->sp[last];
            for (uint64_t j = 0; j < g->n_mol * g->ns; ++j)
                if (g->mol[j] == last) g->mol[j] = site;
            for (uint32_t k2 = k + 1; k2 < count; ++k2)
                if (indices[k2] == last) indices[k2] = site;
        }
        g->n--;
    }
}

/* attemptDeletion (monte_carlo_engine.cc:621-671) + removeMolecule (:814-823) */
static void attempt_deletion(orc_gcmc* g) {
    if (g->n_mol == 0) return;
    g->attempted[3]++;
    const uint64_t mi = (uint64_t)(u01(g) * (double)g->n_mol);
    const uint64_t count_before = g->n_mol;
    uint64_t idx[16];
    memcpy(idx, g->mol + mi * g->ns, sizeof(uint64_t) * g->ns);
    const double ui = dispersion(g, idx);
    const double ei = electro_real(g, idx);
    double old_s[64];
    double rec = 0.0;
    if (g->charged) {
        pack_sites(g, idx, old_s);
        rec = orc_ews_delta(&g->ews, old_s, g->ns, NULL, 0, NULL, NULL, NULL, NULL);
    }
    const double du = -(ui + ei) + rec;
    g->last_du = du;
    const double volume = fabs(orc_volume(g->m));
    const double ratio = orc_deletion_ratio(g->fugacity, volume, count_before, g->temperature, du);
    if (accept(g, ratio)) {
        if (g->charged) orc_ews_commit(&g->ews, old_s, g->ns, NULL, 0);
        /* molecules_.erase(begin + mi): later molecules shift down */
        memmove(g->mol + mi * g->ns, g->mol + (mi + 1) * g->ns,
                sizeof(uint64_t) * (g->n_mol - mi - 1) * g->ns);
        g->n_mol--;
        remove_particle_indices(g, idx, g->ns);
        maybe_resync(g);
        g->accepted[3]++;
    }
}

/* run (monte_carlo_engine.cc:405-439), single species: 25% each */
void orc_gcmc_run(orc_gcmc* g, uint64_t steps) {
    for (uint64_t step = 0; step < steps; ++step) {
        const double pick = u01(g);
        if (pick < 0.25)
            attempt_translation(g);
        else if (pick < 0.5)
            attempt_rotation(g);
        else if (pick < 0.75)
            attempt_insertion(g);
        else
            attempt_deletion(g);
        g->steps++;
    }
}

double orc_gcmc_ewald_energy(const orc_gcmc* g) { return g->charged ? orc_ews_energy(&g->ews) : 0.0; }

/* Heap handles for the Python binding. */
orc_gcmc* orc_gcmc_new(const orc_lj* lj, const orc_ewald_params* ew, const double m[9], uint64_t n,
                       const double* x, const double* y, const double* z, const double* q,
                       const uint32_t* species, const orc_species* guest, double temperature,
                       double fugacity_pa, double max_translation, double max_rotation,
                       uint64_t seed, uint64_t stream, int draw_order) {
    orc_gcmc* g = (orc_gcmc*)malloc(sizeof(orc_gcmc));
    orc_gcmc_create(g, lj, ew, m, n, x, y, z, q, species, guest, temperature, fugacity_pa,
                    max_translation, max_rotation, seed, stream, draw_order);
    return g;
}
void orc_gcmc_delete(orc_gcmc* g) {
    orc_gcmc_free(g);
    free(g);
}
uint64_t orc_gcmc_molecules(const orc_gcmc* g) { return g->n_mol; }
uint64_t orc_gcmc_particles(const orc_gcmc* g, double* xyz, uint64_t cap) {
    for (uint64_t i = 0; i < g->n && i < cap; ++i) {
        xyz[3 * i] = g->x[i];
        xyz[3 * i + 1] = g->y[i];
        xyz[3 * i + 2] = g->z[i];
    }
    return g->n;
}
uint64_t orc_gcmc_calls(const orc_gcmc* g) { return g->call; }
void orc_gcmc_counters(const orc_gcmc* g, uint64_t* out8) {
    for (int i = 0; i < 4; ++i) {
        out8[i] = g->attempted[i];
        out8[4 + i] = g->accepted[i];
    }
}
