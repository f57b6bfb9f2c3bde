/*
 * ORACLE — test infrastructure, not product code.
 *
 * Plain-C restatement of MonteCarloEngine's GCMC chain, one or several rigid
 * species (engines/monte_carlo/monte_carlo_engine.cc:159-439 run, :441-792
 * moves, :814-848 removal), FP64, in the reference's operation order. One
 * species keeps the single-species draw sequence (4-way move split, no
 * species draws); several use the 5-way split with identity swaps and the
 * per-species draws of insertion, deletion and rotation. The reference's
 * guest-guest cell-list candidates are a superset of the guests within the
 * cutoff visited in ascending index order (monte_carlo_engine.cc:316-374), and
 * pairEnergy beyond the cutoff is exactly 0.0, so an ascending scan gives the
 * same sums bit for bit; this port scans. Without an energy grid the scan
 * covers every particle (framework first); with one, a site's dispersion is
 * the grid's interpolation plus the scan over guests only
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
    g->mol = (uint64_t*)realloc(g->mol, sizeof(uint64_t) * cap * ORC_MOLW);
    g->mol_sp = (uint32_t*)realloc(g->mol_sp, sizeof(uint32_t) * cap);
    g->mol_cap = cap;
}

int orc_gcmc_create(orc_gcmc* g, const orc_lj* lj, const orc_ewald_params* ew, const double m[9],
                    uint64_t n, const double* x, const double* y, const double* z, const double* q,
                    const uint32_t* species, uint32_t n_species, const orc_species* guests,
                    double temperature, const double* fugacity_pa, double max_translation,
                    double max_rotation, uint64_t seed, uint64_t stream, int draw_order) {
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
    g->n_species = n_species < ORC_MAX_SPECIES ? n_species : ORC_MAX_SPECIES;
    for (uint32_t k = 0; k < g->n_species; ++k) {
        orc_gcmc_species* sp = &g->spc[k];
        sp->ns = guests[k].n_sites < ORC_MOLW ? guests[k].n_sites : ORC_MOLW;
        for (uint32_t s = 0; s < sp->ns; ++s) {
            sp->x[s] = guests[k].x[s];
            sp->y[s] = guests[k].y[s];
            sp->z[s] = guests[k].z[s];
            sp->lj[s] = guests[k].lj_species[s];
            sp->q[s] = guests[k].charge[s];
        }
        sp->fugacity = fugacity_pa[k] * ORC_PASCAL_TO_INTERNAL; /* monte_carlo_engine.cc:212-219 */
        /* the template about its centroid: per axis the sum over the sites in
         * order, then each site less the sum / ns */
        double c[3] = {0.0, 0.0, 0.0};
        for (uint32_t s = 0; s < sp->ns; ++s) {
            c[0] += sp->x[s];
            c[1] += sp->y[s];
            c[2] += sp->z[s];
        }
        for (uint32_t s = 0; s < sp->ns; ++s) {
            sp->cx[s] = sp->x[s] - c[0] / (double)sp->ns;
            sp->cy[s] = sp->y[s] - c[1] / (double)sp->ns;
            sp->cz[s] = sp->z[s] - c[2] / (double)sp->ns;
        }
    }
    g->orient = 1;
    g->temperature = temperature;
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
    free(g->mol_sp);
    free(g->eps);
    free(g->sigma);
    if (g->charged) orc_ews_free(&g->ews);
    memset(g, 0, sizeof(*g));
}

static int excluded_in(const uint64_t* ex, uint32_t n_ex, uint64_t j) {
    for (uint32_t k = 0; k < n_ex; ++k)
        if (ex[k] == j) return 1;
    return 0;
}

/* computeParticleEnergyOverCandidates over the guests (indices from n_fw),
 * ascending (lennard_jones.cc:179-209) */
static double lj_over_guests(orc_gcmc* g, uint64_t index, const uint64_t* excluded, uint32_t n_ex) {
    double energy = 0.0;
    const double pi[3] = {g->x[index], g->y[index], g->z[index]};
    for (uint64_t j = g->n_fw; j < g->n; ++j) {
        if (j == index || excluded_in(excluded, n_ex, j)) continue;
        double eps, sigma;
        orc_lj_mixed(&g->lj, g->sp[index], g->sp[j], &eps, &sigma);
        const double pj[3] = {g->x[j], g->y[j], g->z[j]};
        double d[3];
        orc_min_image(g->m, pi, pj, d);
        energy += orc_lj_pair_energy(&g->lj, sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]), eps, sigma);
    }
    return energy;
}

/* moleculeDispersionEnergy(sites, alsoExclude) (monte_carlo_engine.cc:341-374):
 * excluded = the molecule's own sites, then alsoExclude */
static double dispersion(orc_gcmc* g, const uint64_t* idx, uint32_t n, const uint64_t* also,
                         uint32_t n_also) {
    uint64_t ex[2 * ORC_MOLW];
    memcpy(ex, idx, sizeof(uint64_t) * n);
    if (n_also) memcpy(ex + n, also, sizeof(uint64_t) * n_also);
    const uint32_t n_ex = n + n_also;
    double e = 0.0;
    for (uint32_t s = 0; s < n; ++s) {
        if (g->grid) {
            const double p[3] = {g->x[idx[s]], g->y[idx[s]], g->z[idx[s]]};
            e += orc_grid_interpolate(g->m, g->gcounts, g->gtab[g->sp[idx[s]]], p);
            e += lj_over_guests(g, idx[s], ex, n_ex);
        } else {
            e += orc_lj_particle_energy(&g->lj, g->m, g->n, g->x, g->y, g->z, g->sp, idx[s], ex, n_ex);
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

/* moleculeElectrostaticRealSpaceEnergy(sites, alsoExclude)
 * (monte_carlo_engine.cc:299-314): per site, excluded = sites + alsoExclude */
static double electro_real(orc_gcmc* g, const uint64_t* idx, uint32_t n, const uint64_t* also,
                           uint32_t n_also) {
    if (!g->charged) return 0.0;
    uint64_t ex[2 * ORC_MOLW];
    memcpy(ex, idx, sizeof(uint64_t) * n);
    if (n_also) memcpy(ex + n, also, sizeof(uint64_t) * n_also);
    double e = 0.0;
    for (uint32_t s = 0; s < n; ++s)
        e += orc_ewald_real_space_particle_energy(g->m, g->n, g->x, g->y, g->z, g->q, g->ew.alpha,
                                                  g->ew.rc, idx[s], ex, n + n_also);
    return e;
}

static void pack_sites(orc_gcmc* g, const uint64_t* idx, uint32_t n, double* out) {
    for (uint32_t s = 0; s < n; ++s) {
        out[4 * s] = g->x[idx[s]];
        out[4 * s + 1] = g->y[idx[s]];
        out[4 * s + 2] = g->z[idx[s]];
        out[4 * s + 3] = g->q[idx[s]];
    }
}

static uint32_t mol_ns(const orc_gcmc* g, uint64_t mi) { return g->spc[g->mol_sp[mi]].ns; }

/* maybeResyncEwald (monte_carlo_engine.cc:380-403) */
static void maybe_resync(orc_gcmc* g) {
    if (!g->charged) return;
    g->moves_since_resync++;
    if (g->moves_since_resync >= 100) {
        uint64_t* offs = (uint64_t*)malloc(sizeof(uint64_t) * (g->n_mol + 1));
        uint64_t* flat = (uint64_t*)malloc(sizeof(uint64_t) * (g->n_mol * ORC_MOLW + 1));
        offs[0] = 0;
        for (uint64_t k = 0; k < g->n_mol; ++k) {
            const uint32_t ns = mol_ns(g, k);
            memcpy(flat + offs[k], g->mol + k * ORC_MOLW, sizeof(uint64_t) * ns);
            offs[k + 1] = offs[k] + ns;
        }
        orc_ews_resync(&g->ews, g->n, g->x, g->y, g->z, g->q, g->n_mol, offs, flat);
        free(offs);
        free(flat);
        g->moves_since_resync = 0;
        g->resyncs++;
    }
}

static int accept(orc_gcmc* g, double ratio) { return u01(g) < orc_clamp_probability(ratio); }

/* randomUnitQuaternion over three draws taken in the engine's argument order */
static void draw_orientation(orc_gcmc* g, double quat[4]) {
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

/* Appends the species' sites at reference point ref (rotated by quat when it
 * has several sites); their indices into idx. */
static void place_sites(orc_gcmc* g, uint32_t k, const double ref[3], const double quat[4],
                        uint64_t* idx) {
    const orc_gcmc_species* sp = &g->spc[k];
    ensure_capacity(g, g->n + sp->ns);
    for (uint32_t s = 0; s < sp->ns; ++s) {
        const double local[3] = {sp->x[s], sp->y[s], sp->z[s]};
        double rot[3] = {local[0], local[1], local[2]};
        if (sp->ns > 1) orc_rotate_by_quaternion(local, quat, rot);
        const uint64_t i = g->n++;
        g->x[i] = ref[0] + rot[0];
        g->y[i] = ref[1] + rot[1];
        g->z[i] = ref[2] + rot[2];
        g->q[i] = sp->q[s];
        g->sp[i] = sp->lj[s];
        idx[s] = i;
    }
}

/* attemptTranslation (monte_carlo_engine.cc:441-484) */
static void attempt_translation(orc_gcmc* g) {
    if (g->n_mol == 0) return;
    const uint64_t mi = (uint64_t)(u01(g) * (double)g->n_mol);
    const uint64_t* idx = g->mol + mi * ORC_MOLW;
    const uint32_t ns = mol_ns(g, mi);
    g->attempted[0]++;
    const double u_before = dispersion(g, idx, ns, NULL, 0);
    const double e_before = electro_real(g, idx, ns, NULL, 0);
    double old_s[4 * ORC_MOLW], new_s[4 * ORC_MOLW], orig[3 * ORC_MOLW];
    if (g->charged) pack_sites(g, idx, ns, old_s);
    const double d0 = (2.0 * u01(g) - 1.0) * g->max_translation;
    const double d1 = (2.0 * u01(g) - 1.0) * g->max_translation;
    const double d2 = (2.0 * u01(g) - 1.0) * g->max_translation;
    for (uint32_t s = 0; s < ns; ++s) {
        const uint64_t i = idx[s];
        orig[3 * s] = g->x[i];
        orig[3 * s + 1] = g->y[i];
        orig[3 * s + 2] = g->z[i];
        g->x[i] = orig[3 * s] + d0;
        g->y[i] = orig[3 * s + 1] + d1;
        g->z[i] = orig[3 * s + 2] + d2;
    }
    const double u_after = dispersion(g, idx, ns, NULL, 0);
    const double e_after = electro_real(g, idx, ns, NULL, 0);
    double rec = 0.0;
    if (g->charged) {
        pack_sites(g, idx, ns, new_s);
        rec = orc_ews_delta(&g->ews, old_s, ns, new_s, ns, NULL, NULL, NULL, NULL);
    }
    const double du = (u_after - u_before) + (e_after - e_before) + rec;
    g->last_du = du;
    if (accept(g, orc_metropolis_ratio(g->temperature, du))) {
        if (g->charged) {
            orc_ews_commit(&g->ews, old_s, ns, new_s, ns);
            maybe_resync(g);
        }
        g->accepted[0]++;
        return;
    }
    for (uint32_t s = 0; s < ns; ++s) {
        const uint64_t i = idx[s];
        g->x[i] = orig[3 * s];
        g->y[i] = orig[3 * s + 1];
        g->z[i] = orig[3 * s + 2];
    }
}

/* attemptRotation (monte_carlo_engine.cc:486-554) */
static void attempt_rotation(orc_gcmc* g) {
    if (g->n_mol == 0) return;
    if (g->n_species == 1 && g->spc[0].ns < 2) return; /* single species, single site: no draw */
    const uint64_t mi = (uint64_t)(u01(g) * (double)g->n_mol);
    const uint32_t ns = mol_ns(g, mi);
    if (ns < 2) return; /* this molecule's species is single-site */
    const uint64_t* idx = g->mol + mi * ORC_MOLW;
    g->attempted[1]++;
    const double u_before = dispersion(g, idx, ns, NULL, 0);
    const double e_before = electro_real(g, idx, ns, NULL, 0);
    double old_s[4 * ORC_MOLW], new_s[4 * ORC_MOLW], orig[3 * ORC_MOLW];
    if (g->charged) pack_sites(g, idx, ns, old_s);
    double c[3] = {0.0, 0.0, 0.0};
    for (uint32_t s = 0; s < ns; ++s) {
        c[0] = c[0] + g->x[idx[s]];
        c[1] = c[1] + g->y[idx[s]];
        c[2] = c[2] + g->z[idx[s]];
    }
    const double inv = 1.0 / (double)ns;
    c[0] = c[0] * inv;
    c[1] = c[1] * inv;
    c[2] = c[2] * inv;
    const double cos_t = 2.0 * u01(g) - 1.0;
    const double sin_t = sqrt(fmax(0.0, 1.0 - cos_t * cos_t));
    const double phi = 2.0 * ORC_PI * u01(g);
    const double axis[3] = {sin_t * cos(phi), sin_t * sin(phi), cos_t};
    const double angle = (2.0 * u01(g) - 1.0) * g->max_rotation;
    for (uint32_t s = 0; s < ns; ++s) {
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
    const double u_after = dispersion(g, idx, ns, NULL, 0);
    const double e_after = electro_real(g, idx, ns, NULL, 0);
    double rec = 0.0;
    if (g->charged) {
        pack_sites(g, idx, ns, new_s);
        rec = orc_ews_delta(&g->ews, old_s, ns, new_s, ns, NULL, NULL, NULL, NULL);
    }
    const double du = (u_after - u_before) + (e_after - e_before) + rec;
    g->last_du = du;
    if (accept(g, orc_metropolis_ratio(g->temperature, du))) {
        if (g->charged) {
            orc_ews_commit(&g->ews, old_s, ns, new_s, ns);
            maybe_resync(g);
        }
        g->accepted[1]++;
        return;
    }
    for (uint32_t s = 0; s < ns; ++s) {
        const uint64_t i = idx[s];
        g->x[i] = orig[3 * s];
        g->y[i] = orig[3 * s + 1];
        g->z[i] = orig[3 * s + 2];
    }
}

/* U_tail(after) - U_tail(before) as two tailEnergyCorrection evaluations
 * (lennard_jones.cc:246-257): before = particles [0, n_before); after = the
 * same without the n_rem sites rem[] plus the n_add sites at [n_before,
 * n_before + n_add) (a trial's sites are appended to the arrays). */
static double tail_change(const orc_gcmc* g, uint64_t n_before, const uint64_t* rem, uint32_t n_rem,
                          uint32_t n_add) {
    if (!g->tail) return 0.0;
    const double before = orc_lj_tail(&g->lj, g->m, n_before, g->sp);
    uint32_t* after = (uint32_t*)malloc(sizeof(uint32_t) * (n_before + n_add + 1));
    uint64_t n = 0;
    for (uint64_t i = 0; i < n_before + n_add; ++i) {
        int gone = 0;
        for (uint32_t r = 0; r < n_rem; ++r) gone |= rem[r] == i;
        if (!gone) after[n++] = g->sp[i];
    }
    const double a = orc_lj_tail(&g->lj, g->m, n, after);
    free(after);
    return a - before;
}

void orc_gcmc_set_tail(orc_gcmc* g, int on) { g->tail = on; }
void orc_gcmc_set_orientation_trials(orc_gcmc* g, int k) { g->orient = k < 1 ? 1 : k > 16 ? 16 : k; }

/* ---- orientation-biased insertion and deletion (no reference counterpart):
 * the standard orientational configurational-bias scheme, in the draw order
 * and arithmetic of the GPU chains' FP64 form. An insertion draws its point
 * as the molecule's centroid and a first orientation (the move's own draws),
 * then k - 1 orientations (three calls each, the engine's argument order),
 * evaluates the energy U_j of each trial, picks one with probability w_j / W
 * (one call; w = exp(-U / T)) and accepts with W / k in place of exp(-dU/T).
 * A deletion evaluates the molecule's energy U_0 (minus its removal's dU),
 * then k - 1 random orientations of it about its centroid, each drawn just
 * before its evaluation (U_j = U_0 + dU of that rotation), and accepts with
 * k / W in place of exp(+U_0 / T). */
#define ORC_MAXCB 16

static uint64_t count_of_species(const orc_gcmc* g, uint32_t k);

static void draw_trial_orientation(orc_gcmc* g, double quat[4]) {
    double v[3];
    v[0] = u01(g);
    v[1] = u01(g);
    v[2] = u01(g);
    orc_random_unit_quaternion(v[0], v[1], v[2], quat);
}

/* the centred template of species k rotated by quat, about ref, into pos */
static void trial_sites(const orc_gcmc* g, uint32_t k, const double ref[3], const double quat[4],
                        double* pos) {
    const orc_gcmc_species* sp = &g->spc[k];
    for (uint32_t s = 0; s < sp->ns; ++s) {
        const double local[3] = {sp->cx[s], sp->cy[s], sp->cz[s]};
        double rot[3];
        orc_rotate_by_quaternion(local, quat, rot);
        pos[3 * s] = ref[0] + rot[0];
        pos[3 * s + 1] = ref[1] + rot[1];
        pos[3 * s + 2] = ref[2] + rot[2];
    }
}

/* log(sum_j exp(lw_j) / k) and, when pick is non-NULL, one draw picking j
 * with probability exp(lw_j) / sum */
static double rosenbluth(orc_gcmc* g, const double* lw, int k, int* pick) {
    double m = lw[0];
    for (int j = 1; j < k; ++j) m = fmax(m, lw[j]);
    double tot = 0.0;
    for (int j = 0; j < k; ++j) tot += exp(lw[j] - m);
    const double logw = m + log(tot / (double)k);
    if (pick) {
        const double u = u01(g) * tot;
        *pick = k - 1;
        double cum = 0.0;
        for (int j = 0; j < k; ++j) {
            cum += exp(lw[j] - m);
            if (u < cum) {
                *pick = j;
                break;
            }
        }
    }
    return logw;
}

static void insertion_trials(orc_gcmc* g, uint32_t k, const double ref[3], const double q0[4]) {
    const orc_gcmc_species* sp = &g->spc[k];
    const int kt = g->orient < ORC_MAXCB ? g->orient : ORC_MAXCB;
    const double T = g->temperature;
    double quat[ORC_MAXCB][4];
    memcpy(quat[0], q0, sizeof(double) * 4);
    for (int j = 1; j < kt; ++j) draw_trial_orientation(g, quat[j]);
    double lw[ORC_MAXCB] = {0.0}, pos[ORC_MAXCB][3 * ORC_MOLW];
    uint64_t idx[ORC_MOLW];
    for (int j = 0; j < kt; ++j) {
        trial_sites(g, k, ref, quat[j], pos[j]);
        place_sites(g, k, ref, quat[j], idx); /* the sites appended, then set to the trial's */
        for (uint32_t s = 0; s < sp->ns; ++s) {
            g->x[idx[s]] = pos[j][3 * s];
            g->y[idx[s]] = pos[j][3 * s + 1];
            g->z[idx[s]] = pos[j][3 * s + 2];
        }
        const double disp = dispersion(g, idx, sp->ns, NULL, 0);
        const double elec = electro_real(g, idx, sp->ns, NULL, 0);
        double rec = 0.0;
        if (g->charged) {
            double new_s[4 * ORC_MOLW];
            pack_sites(g, idx, sp->ns, new_s);
            rec = orc_ews_delta(&g->ews, NULL, 0, new_s, sp->ns, NULL, NULL, NULL, NULL);
        }
        lw[j] = -((disp + elec) + rec) / T;
        g->n -= sp->ns;
    }
    int pick = kt - 1;
    const double logw = rosenbluth(g, lw, kt, &pick);
    const double cb_du = -lw[pick] * T;
    place_sites(g, k, ref, quat[pick], idx);
    for (uint32_t s = 0; s < sp->ns; ++s) {
        g->x[idx[s]] = pos[pick][3 * s];
        g->y[idx[s]] = pos[pick][3 * s + 1];
        g->z[idx[s]] = pos[pick][3 * s + 2];
    }
    const double dut = tail_change(g, g->n - sp->ns, NULL, 0, sp->ns);
    g->last_du = cb_du + dut;
    const double volume = fabs(orc_volume(g->m));
    const uint64_t before = g->n_species == 1 ? g->n_mol : count_of_species(g, k);
    const double ratio = (sp->fugacity * volume / T) / (double)(before + 1) * exp(logw - dut / T);
    if (accept(g, ratio)) {
        if (g->charged) {
            double new_s[4 * ORC_MOLW];
            pack_sites(g, idx, sp->ns, new_s);
            orc_ews_commit(&g->ews, NULL, 0, new_s, sp->ns);
        }
        ensure_mol_capacity(g, g->n_mol + 1);
        memcpy(g->mol + g->n_mol * ORC_MOLW, idx, sizeof(uint64_t) * sp->ns);
        g->mol_sp[g->n_mol] = k;
        g->n_mol++;
        maybe_resync(g);
        g->accepted[2]++;
        return;
    }
    g->n -= sp->ns;
}

/* the deletion of molecule mi (species k, count_before of it) with trials;
 * returns 1 when accepted (the caller removes the molecule) */
static int deletion_trials(orc_gcmc* g, uint64_t mi, uint32_t k, uint64_t count_before) {
    const uint32_t ns = g->spc[k].ns;
    const int kt = g->orient < ORC_MAXCB ? g->orient : ORC_MAXCB;
    const double T = g->temperature;
    uint64_t idx[ORC_MOLW];
    memcpy(idx, g->mol + mi * ORC_MOLW, sizeof(uint64_t) * ns);
    const double u_old = dispersion(g, idx, ns, NULL, 0);
    const double e_old = electro_real(g, idx, ns, NULL, 0);
    double old_s[4 * ORC_MOLW], orig[3 * ORC_MOLW];
    double rec0 = 0.0;
    if (g->charged) {
        pack_sites(g, idx, ns, old_s);
        rec0 = orc_ews_delta(&g->ews, old_s, ns, NULL, 0, NULL, NULL, NULL, NULL);
    }
    const double u0 = (u_old + e_old) - rec0;
    double lw[ORC_MAXCB];
    lw[0] = -u0 / T;
    double ref[3] = {0.0, 0.0, 0.0};
    for (uint32_t s = 0; s < ns; ++s) {
        ref[0] += g->x[idx[s]];
        ref[1] += g->y[idx[s]];
        ref[2] += g->z[idx[s]];
    }
    for (int a = 0; a < 3; ++a) ref[a] /= (double)ns;
    for (uint32_t s = 0; s < ns; ++s) {
        orig[3 * s] = g->x[idx[s]];
        orig[3 * s + 1] = g->y[idx[s]];
        orig[3 * s + 2] = g->z[idx[s]];
    }
    for (int j = 1; j < kt; ++j) {
        double quat[4], pos[3 * ORC_MOLW];
        draw_trial_orientation(g, quat);
        trial_sites(g, k, ref, quat, pos);
        for (uint32_t s = 0; s < ns; ++s) {
            g->x[idx[s]] = pos[3 * s];
            g->y[idx[s]] = pos[3 * s + 1];
            g->z[idx[s]] = pos[3 * s + 2];
        }
        const double u_new = dispersion(g, idx, ns, NULL, 0);
        const double e_new = electro_real(g, idx, ns, NULL, 0);
        double rec = 0.0;
        if (g->charged) {
            double new_s[4 * ORC_MOLW];
            pack_sites(g, idx, ns, new_s);
            rec = orc_ews_delta(&g->ews, old_s, ns, new_s, ns, NULL, NULL, NULL, NULL);
        }
        lw[j] = -(u0 + ((u_new - u_old) + (e_new - e_old) + rec)) / T;
        for (uint32_t s = 0; s < ns; ++s) {
            g->x[idx[s]] = orig[3 * s];
            g->y[idx[s]] = orig[3 * s + 1];
            g->z[idx[s]] = orig[3 * s + 2];
        }
    }
    const double logw = rosenbluth(g, lw, kt, NULL);
    const double dut = tail_change(g, g->n, idx, ns, 0);
    g->last_du = -u0 + dut;
    const double volume = fabs(orc_volume(g->m));
    const double ratio =
        (double)count_before / (g->spc[k].fugacity * volume / T) * exp(-logw - dut / T);
    return accept(g, ratio);
}

static uint64_t count_of_species(const orc_gcmc* g, uint32_t k) {
    uint64_t c = 0;
    for (uint64_t mi = 0; mi < g->n_mol; ++mi) c += g->mol_sp[mi] == k;
    return c;
}

/* attemptInsertion (monte_carlo_engine.cc:556-619) */
static void attempt_insertion(orc_gcmc* g) {
    const uint32_t k = g->n_species == 1 ? 0u : (uint32_t)(u01(g) * (double)g->n_species);
    const orc_gcmc_species* sp = &g->spc[k];
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
    if (sp->ns > 1) draw_orientation(g, quat);
    if (g->orient > 1 && sp->ns > 1) {  /* orientation trials about the drawn centroid */
        insertion_trials(g, k, ref, quat);
        return;
    }
    uint64_t idx[ORC_MOLW];
    place_sites(g, k, ref, quat, idx);
    const double disp = dispersion(g, idx, sp->ns, NULL, 0);
    const double elec = electro_real(g, idx, sp->ns, NULL, 0);
    double new_s[4 * ORC_MOLW];
    double rec = 0.0;
    if (g->charged) {
        pack_sites(g, idx, sp->ns, new_s);
        rec = orc_ews_delta(&g->ews, NULL, 0, new_s, sp->ns, NULL, NULL, NULL, NULL);
    }
    const double du = disp + elec + rec + tail_change(g, g->n - sp->ns, NULL, 0, sp->ns);
    g->last_du = du;
    const double volume = fabs(orc_volume(m));
    const uint64_t before = g->n_species == 1 ? g->n_mol : count_of_species(g, k);
    const double ratio = orc_insertion_ratio(sp->fugacity, volume, before, g->temperature, du);
    if (accept(g, ratio)) {
        if (g->charged) orc_ews_commit(&g->ews, NULL, 0, new_s, sp->ns);
        ensure_mol_capacity(g, g->n_mol + 1);
        memcpy(g->mol + g->n_mol * ORC_MOLW, idx, sizeof(uint64_t) * sp->ns);
        g->mol_sp[g->n_mol] = k;
        g->n_mol++;
        maybe_resync(g);
        g->accepted[2]++;
        return;
    }
    g->n -= sp->ns;
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
            for (uint64_t mi = 0; mi < g->n_mol; ++mi) {
                uint64_t* ms = g->mol + mi * ORC_MOLW;
                const uint32_t ns = mol_ns(g, mi);
                for (uint32_t s = 0; s < ns; ++s)
                    if (ms[s] == last) ms[s] = site;
            }
            for (uint32_t k2 = k + 1; k2 < count; ++k2)
                if (indices[k2] == last) indices[k2] = site;
        }
        g->n--;
    }
}

/* attemptDeletion (monte_carlo_engine.cc:621-671) + removeMolecule (:814-823) */
static void attempt_deletion(orc_gcmc* g) {
    if (g->n_mol == 0) return;
    uint64_t mi, count_before;
    uint32_t k;
    if (g->n_species == 1) {
        mi = (uint64_t)(u01(g) * (double)g->n_mol);
        k = 0;
        count_before = g->n_mol;
    } else {
        k = (uint32_t)(u01(g) * (double)g->n_species);
        count_before = count_of_species(g, k);
        if (count_before == 0) return;
        /* the species' molecules in index order; the draw picks one */
        const uint64_t pick = (uint64_t)(u01(g) * (double)count_before);
        uint64_t seen = 0;
        mi = 0;
        for (uint64_t j = 0; j < g->n_mol; ++j)
            if (g->mol_sp[j] == k && seen++ == pick) {
                mi = j;
                break;
            }
    }
    g->attempted[3]++;
    const uint32_t ns = g->spc[k].ns;
    uint64_t idx[ORC_MOLW];
    memcpy(idx, g->mol + mi * ORC_MOLW, sizeof(uint64_t) * ns);
    if (g->orient > 1 && ns > 1) {
        if (deletion_trials(g, mi, k, count_before)) {
            if (g->charged) {
                double old_s[4 * ORC_MOLW];
                pack_sites(g, idx, ns, old_s);
                orc_ews_commit(&g->ews, old_s, ns, NULL, 0);
            }
            memmove(g->mol + mi * ORC_MOLW, g->mol + (mi + 1) * ORC_MOLW,
                    sizeof(uint64_t) * (g->n_mol - mi - 1) * ORC_MOLW);
            memmove(g->mol_sp + mi, g->mol_sp + mi + 1, sizeof(uint32_t) * (g->n_mol - mi - 1));
            g->n_mol--;
            remove_particle_indices(g, idx, ns);
            maybe_resync(g);
            g->accepted[3]++;
        }
        return;
    }
    const double ui = dispersion(g, idx, ns, NULL, 0);
    const double ei = electro_real(g, idx, ns, NULL, 0);
    double old_s[4 * ORC_MOLW];
    double rec = 0.0;
    if (g->charged) {
        pack_sites(g, idx, ns, old_s);
        rec = orc_ews_delta(&g->ews, old_s, ns, NULL, 0, NULL, NULL, NULL, NULL);
    }
    const double du = -(ui + ei) + rec + tail_change(g, g->n, idx, ns, 0);
    g->last_du = du;
    const double volume = fabs(orc_volume(g->m));
    const double ratio =
        orc_deletion_ratio(g->spc[k].fugacity, volume, count_before, g->temperature, du);
    if (accept(g, ratio)) {
        if (g->charged) orc_ews_commit(&g->ews, old_s, ns, NULL, 0);
        /* molecules_.erase(begin + mi): later molecules shift down */
        memmove(g->mol + mi * ORC_MOLW, g->mol + (mi + 1) * ORC_MOLW,
                sizeof(uint64_t) * (g->n_mol - mi - 1) * ORC_MOLW);
        memmove(g->mol_sp + mi, g->mol_sp + mi + 1, sizeof(uint32_t) * (g->n_mol - mi - 1));
        g->n_mol--;
        remove_particle_indices(g, idx, ns);
        maybe_resync(g);
        g->accepted[3]++;
    }
}

/* attemptSwap (monte_carlo_engine.cc:673-792): a molecule of one species
 * becomes one of another at its centroid, fresh orientation */
static void attempt_swap(orc_gcmc* g) {
    if (g->n_mol == 0 || g->n_species < 2) return;
    const uint32_t from = (uint32_t)(u01(g) * (double)g->n_species);
    const uint64_t count_from = count_of_species(g, from);
    if (count_from == 0) return;
    const uint64_t pick = (uint64_t)(u01(g) * (double)count_from);
    uint64_t mi = 0, seen = 0;
    for (uint64_t j = 0; j < g->n_mol; ++j)
        if (g->mol_sp[j] == from && seen++ == pick) {
            mi = j;
            break;
        }
    uint32_t to = (uint32_t)(u01(g) * (double)(g->n_species - 1));
    if (to >= from) ++to;
    g->attempted[4]++;
    const uint32_t ns_old = g->spc[from].ns;
    uint64_t old_idx[ORC_MOLW];
    memcpy(old_idx, g->mol + mi * ORC_MOLW, sizeof(uint64_t) * ns_old);
    const double u_before = dispersion(g, old_idx, ns_old, NULL, 0);
    const double e_before = electro_real(g, old_idx, ns_old, NULL, 0);
    double old_s[4 * ORC_MOLW], new_s[4 * ORC_MOLW];
    if (g->charged) pack_sites(g, old_idx, ns_old, old_s);
    /* moleculeCentroid (:74-80) */
    double ref[3] = {0.0, 0.0, 0.0};
    for (uint32_t s = 0; s < ns_old; ++s) {
        ref[0] = ref[0] + g->x[old_idx[s]];
        ref[1] = ref[1] + g->y[old_idx[s]];
        ref[2] = ref[2] + g->z[old_idx[s]];
    }
    const double inv = 1.0 / (double)ns_old;
    ref[0] = ref[0] * inv;
    ref[1] = ref[1] * inv;
    ref[2] = ref[2] * inv;
    const orc_gcmc_species* ts = &g->spc[to];
    double quat[4] = {1.0, 0.0, 0.0, 0.0};
    if (ts->ns > 1) draw_orientation(g, quat);
    uint64_t new_idx[ORC_MOLW];
    place_sites(g, to, ref, quat, new_idx);
    const double u_after = dispersion(g, new_idx, ts->ns, old_idx, ns_old);
    const double e_after = electro_real(g, new_idx, ts->ns, old_idx, ns_old);
    double rec = 0.0;
    if (g->charged) {
        pack_sites(g, new_idx, ts->ns, new_s);
        rec = orc_ews_delta(&g->ews, old_s, ns_old, new_s, ts->ns, NULL, NULL, NULL, NULL);
    }
    const double du = (u_after - u_before) + (e_after - e_before) + rec +
                      tail_change(g, g->n - ts->ns, old_idx, ns_old, ts->ns);
    g->last_du = du;
    const uint64_t count_to = count_of_species(g, to);
    const double ratio = orc_swap_ratio(g->spc[from].fugacity, ts->fugacity, count_from, count_to,
                                        g->temperature, du);
    if (accept(g, ratio)) {
        if (g->charged) orc_ews_commit(&g->ews, old_s, ns_old, new_s, ts->ns);
        /* the molecule becomes the new species first, then the old sites go */
        memcpy(g->mol + mi * ORC_MOLW, new_idx, sizeof(uint64_t) * ts->ns);
        g->mol_sp[mi] = to;
        remove_particle_indices(g, old_idx, ns_old);
        maybe_resync(g);
        g->accepted[4]++;
        return;
    }
    g->n -= ts->ns;
}

/* run (monte_carlo_engine.cc:405-439): 25 % each of translate, rotate,
 * insert, delete for one species; 20 % each plus swap for several */
void orc_gcmc_run(orc_gcmc* g, uint64_t steps) {
    const int mixture = g->n_species >= 2;
    for (uint64_t step = 0; step < steps; ++step) {
        const double pick = u01(g);
        if (!mixture) {
            if (pick < 0.25)
                attempt_translation(g);
            else if (pick < 0.5)
                attempt_rotation(g);
            else if (pick < 0.75)
                attempt_insertion(g);
            else
                attempt_deletion(g);
        } else {
            if (pick < 0.2)
                attempt_translation(g);
            else if (pick < 0.4)
                attempt_rotation(g);
            else if (pick < 0.6)
                attempt_insertion(g);
            else if (pick < 0.8)
                attempt_deletion(g);
            else
                attempt_swap(g);
        }
        g->steps++;
    }
}

double orc_gcmc_ewald_energy(const orc_gcmc* g) { return g->charged ? orc_ews_energy(&g->ews) : 0.0; }

/* Heap handles for the Python binding. */
orc_gcmc* orc_gcmc_new_mixture(const orc_lj* lj, const orc_ewald_params* ew, const double m[9],
                               uint64_t n, const double* x, const double* y, const double* z,
                               const double* q, const uint32_t* species, uint32_t n_species,
                               const orc_species* guests, double temperature,
                               const double* fugacity_pa, double max_translation,
                               double max_rotation, uint64_t seed, uint64_t stream,
                               int draw_order) {
    orc_gcmc* g = (orc_gcmc*)malloc(sizeof(orc_gcmc));
    orc_gcmc_create(g, lj, ew, m, n, x, y, z, q, species, n_species, guests, temperature,
                    fugacity_pa, max_translation, max_rotation, seed, stream, draw_order);
    return g;
}
orc_gcmc* orc_gcmc_new(const orc_lj* lj, const orc_ewald_params* ew, const double m[9], uint64_t n,
                       const double* x, const double* y, const double* z, const double* q,
                       const uint32_t* species, const orc_species* guest, double temperature,
                       double fugacity_pa, double max_translation, double max_rotation,
                       uint64_t seed, uint64_t stream, int draw_order) {
    return orc_gcmc_new_mixture(lj, ew, m, n, x, y, z, q, species, 1, guest, temperature,
                                &fugacity_pa, max_translation, max_rotation, seed, stream,
                                draw_order);
}
void orc_gcmc_delete(orc_gcmc* g) {
    orc_gcmc_free(g);
    free(g);
}
uint64_t orc_gcmc_molecules(const orc_gcmc* g) { return g->n_mol; }
uint64_t orc_gcmc_molecules_of(const orc_gcmc* g, uint32_t species) {
    return count_of_species(g, species);
}
uint64_t orc_gcmc_particles(const orc_gcmc* g, double* xyz, uint64_t cap) {
    for (uint64_t i = 0; i < g->n && i < cap; ++i) {
        xyz[3 * i] = g->x[i];
        xyz[3 * i + 1] = g->y[i];
        xyz[3 * i + 2] = g->z[i];
    }
    return g->n;
}
uint64_t orc_gcmc_calls(const orc_gcmc* g) { return g->call; }
void orc_gcmc_counters(const orc_gcmc* g, uint64_t* out10) {
    for (int i = 0; i < 5; ++i) {
        out10[i] = g->attempted[i];
        out10[5 + i] = g->accepted[i];
    }
}
