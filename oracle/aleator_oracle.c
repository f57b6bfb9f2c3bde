/*
 * ORACLE — test infrastructure, not product code. See aleator_oracle.h.
 *
 * Plain-C FP64 restatement of the reference's hot path. Each function keeps
 * the reference's operation order (compile with -ffp-contract=off) and cites
 * the reference file:line it restates; paths are relative to the reference
 * project's src/ directory.
 */
#include "aleator_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.14159265358979323846

/* ------------------------------------------------------------------ vectors
 * lattice.cc:145-183 / ewald.cc:17-23: dot is (a0*b0 + a1*b1) + a2*b2. */
static double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static void cross3(const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
static double norm2_3(const double* a) { return dot3(a, a); }

/* ------------------------------------------------------------------ Philox
 * counter_based_rng.cc:13-17 constants, :29-38 round, :42-54 bijection. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int round = 0; round < 10; ++round) {
        if (round > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n1 = lo1;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        const uint32_t n3 = lo0;
        c0 = n0;
        c1 = n1;
        c2 = n2;
        c3 = n3;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* counter_based_rng.cc:56-71: key = (seed lo, seed hi); counter = (call lo,
 * call hi, stream lo, stream hi); u64 = out0 << 32 | out1. */
uint64_t orc_philox_u64(uint64_t seed, uint64_t stream, uint64_t call_index) {
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    const uint32_t ctr[4] = {(uint32_t)call_index, (uint32_t)(call_index >> 32), (uint32_t)stream,
                             (uint32_t)(stream >> 32)};
    uint32_t out[4];
    orc_philox4x32_10(ctr, key, out);
    return ((uint64_t)out[0] << 32) | (uint64_t)out[1];
}

/* counter_based_rng.cc:73-79: (u64 >> 11) * 2^-53. */
double orc_philox_uniform(uint64_t seed, uint64_t stream, uint64_t call_index) {
    return (double)(orc_philox_u64(seed, stream, call_index) >> 11) * (1.0 / 9007199254740992.0);
}

void orc_philox_fill_u64(uint64_t seed, uint64_t stream, uint64_t first, uint64_t n, uint64_t* out) {
    for (uint64_t i = 0; i < n; ++i) out[i] = orc_philox_u64(seed, stream, first + i);
}

void orc_philox_fill_uniform(uint64_t seed, uint64_t stream, uint64_t first, uint64_t n, double* out) {
    for (uint64_t i = 0; i < n; ++i) out[i] = orc_philox_uniform(seed, stream, first + i);
}

/* ------------------------------------------------------------------ Lattice */

/* lattice.hpp:35-41 */
double orc_volume(const double m[9]) {
    const double cx = m[4] * m[8] - m[5] * m[7];
    const double cy = m[5] * m[6] - m[3] * m[8];
    const double cz = m[3] * m[7] - m[4] * m[6];
    return m[0] * cx + m[1] * cy + m[2] * cz;
}

/* lattice.cc:257-284 */
double orc_perpendicular_width(const double m[9], int axis) {
    const double* a0 = m;
    const double* a1 = m + 3;
    const double* a2 = m + 6;
    const double *o0, *o1;
    if (axis == 0) {
        o0 = a1;
        o1 = a2;
    } else if (axis == 1) {
        o0 = a2;
        o1 = a0;
    } else {
        o0 = a0;
        o1 = a1;
    }
    double c[3];
    cross3(o0, o1, c);
    const double face = sqrt(norm2_3(c));
    return fabs(orc_volume(m)) / face;
}

/* lattice.cc:115-132 */
int orc_is_orthorhombic(const double m[9]) {
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) {
            if (i == j) continue;
            double scale = fabs(m[4 * i]);
            if (fabs(m[4 * j]) > scale) scale = fabs(m[4 * j]);
            if (1.0 > scale) scale = 1.0;
            if (fabs(m[3 * i + j]) > 1e-9 * scale) return 0;
        }
    }
    return 1;
}

/* lattice.cc:70-101 (greedyReduce); the 3-element std::sort there is a
 * stable insertion sort on squared length, restated as such. */
void orc_reduced_basis(const double m[9], double out[9]) {
    double v[3][3];
    for (int i = 0; i < 3; ++i)
        for (int c = 0; c < 3; ++c) v[i][c] = m[3 * i + c];
    for (int iter = 0; iter < 50; ++iter) {
        int changed = 0;
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j) {
                if (i == j) continue;
                const double nj2 = norm2_3(v[j]);
                if (nj2 < 1e-10) continue;
                const double t = round(dot3(v[i], v[j]) / nj2);
                if (t != 0.0) {
                    for (int c = 0; c < 3; ++c) v[i][c] = v[i][c] - v[j][c] * t;
                    changed = 1;
                }
            }
        }
        for (int i = 1; i < 3; ++i) {
            double tmp[3] = {v[i][0], v[i][1], v[i][2]};
            const double key = norm2_3(tmp);
            int j = i - 1;
            while (j >= 0 && key < norm2_3(v[j])) {
                for (int c = 0; c < 3; ++c) v[j + 1][c] = v[j][c];
                --j;
            }
            for (int c = 0; c < 3; ++c) v[j + 1][c] = tmp[c];
        }
        if (!changed) break;
    }
    for (int i = 0; i < 3; ++i)
        for (int c = 0; c < 3; ++c) out[3 * i + c] = v[i][c];
}

/* lattice.cc:157-163 */
void orc_frac_to_cart(const double m[9], const double f[3], double out[3]) {
    for (int c = 0; c < 3; ++c) out[c] = f[0] * m[c] + f[1] * m[3 + c] + f[2] * m[6 + c];
}

/* lattice.cc:54-60 (fractionalOf) with the signed volume, lattice.cc:166-175 */
static void fractional_of(const double* c, const double* b0, const double* b1, const double* b2,
                          double vol, double* out) {
    double t[3];
    cross3(b1, b2, t);
    out[0] = dot3(c, t) / vol;
    cross3(b2, b0, t);
    out[1] = dot3(c, t) / vol;
    cross3(b0, b1, t);
    out[2] = dot3(c, t) / vol;
}

void orc_cart_to_frac(const double m[9], const double c[3], double out[3]) {
    fractional_of(c, m, m + 3, m + 6, orc_volume(m), out);
}

/* lattice.cc:185-255 */
void orc_min_image(const double m[9], const double a[3], const double b[3], double out[3]) {
    const double d[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    if (orc_is_orthorhombic(m)) {
        for (int axis = 0; axis < 3; ++axis) {
            const double length = m[4 * axis];
            out[axis] = d[axis] - length * round(d[axis] / length);
        }
        return;
    }
    double r[9];
    orc_reduced_basis(m, r);
    double cr[3];
    cross3(r + 3, r + 6, cr);
    const double rvol = dot3(r, cr);
    double nearest[3];
    fractional_of(d, r, r + 3, r + 6, rvol, nearest);
    const long n0 = lround(nearest[0]), n1 = lround(nearest[1]), n2 = lround(nearest[2]);
    double best[3] = {d[0], d[1], d[2]};
    double best2 = norm2_3(d);
    for (long dn0 = -2; dn0 <= 2; ++dn0) {
        for (long dn1 = -2; dn1 <= 2; ++dn1) {
            for (long dn2 = -2; dn2 <= 2; ++dn2) {
                const double c0 = (double)(n0 + dn0);
                const double c1 = (double)(n1 + dn1);
                const double c2 = (double)(n2 + dn2);
                double cand[3];
                for (int c = 0; c < 3; ++c) {
                    const double tr = (r[c] * c0 + r[3 + c] * c1) + r[6 + c] * c2;
                    cand[c] = d[c] - tr;
                }
                const double cn2 = norm2_3(cand);
                if (cn2 < best2) {
                    best2 = cn2;
                    best[0] = cand[0];
                    best[1] = cand[1];
                    best[2] = cand[2];
                }
            }
        }
    }
    out[0] = best[0];
    out[1] = best[1];
    out[2] = best[2];
}

/* supercell.cc:7-20 */
void orc_supercell_replication(const double m[9], double cutoff, int out[3]) {
    for (int axis = 0; axis < 3; ++axis) {
        const double w = orc_perpendicular_width(m, axis);
        int n = 1;
        while ((double)n * w <= 2.0 * cutoff) ++n;
        out[axis] = n;
    }
}

/* ------------------------------------------------------------------ Lennard-Jones */

/* lennard_jones.cc:49-68 */
void orc_lj_mixed(const orc_lj* lj, uint32_t i, uint32_t j, double* eps, double* sigma) {
    if (i == j) {
        *eps = lj->eps[i];
        *sigma = lj->sigma[i];
        return;
    }
    *eps = sqrt(lj->eps[i] * lj->eps[j]);
    if (lj->mixing == ORC_LORENTZ_BERTHELOT)
        *sigma = 0.5 * (lj->sigma[i] + lj->sigma[j]);
    else
        *sigma = sqrt(lj->sigma[i] * lj->sigma[j]);
}

/* lennard_jones.cc:15-20 */
static double lj_raw(double r, double eps, double sigma) {
    const double sr = sigma / r;
    const double sr6 = sr * sr * sr * sr * sr * sr;
    const double sr12 = sr6 * sr6;
    return 4.0 * eps * (sr12 - sr6);
}

/* lennard_jones.cc:23-28 */
static double lj_raw_derivative(double r, double eps, double sigma) {
    const double sr = sigma / r;
    const double sr6 = sr * sr * sr * sr * sr * sr;
    const double sr12 = sr6 * sr6;
    return (24.0 * eps / r) * (sr6 - 2.0 * sr12);
}

/* lennard_jones.cc:70-86 */
double orc_lj_pair_energy(const orc_lj* lj, double r, double eps, double sigma) {
    const double rc = lj->cutoff;
    if (r > rc) return 0.0;
    switch (lj->truncation) {
        case ORC_TRUNCATED:
            return lj_raw(r, eps, sigma);
        case ORC_SHIFTED:
            return lj_raw(r, eps, sigma) - lj_raw(rc, eps, sigma);
        default: {
            const double v = lj_raw(rc, eps, sigma);
            const double dv = lj_raw_derivative(rc, eps, sigma);
            return lj_raw(r, eps, sigma) - v - (r - rc) * dv;
        }
    }
}

static int contains_u64(const uint64_t* v, uint64_t n, uint64_t x) {
    for (uint64_t i = 0; i < n; ++i)
        if (v[i] == x) return 1;
    return 0;
}

/* lennard_jones.cc:158-182 */
double orc_lj_particle_energy(const orc_lj* lj, const double m[9], uint64_t n, const double* x,
                              const double* y, const double* z, const uint32_t* species,
                              uint64_t index, const uint64_t* excluded, uint64_t n_excluded) {
    double energy = 0.0;
    const double pi[3] = {x[index], y[index], z[index]};
    for (uint64_t j = 0; j < n; ++j) {
        if (j == index) continue;
        if (contains_u64(excluded, n_excluded, j)) continue;
        double eps, sigma;
        orc_lj_mixed(lj, species[index], species[j], &eps, &sigma);
        const double pj[3] = {x[j], y[j], z[j]};
        double d[3];
        orc_min_image(m, pi, pj, d);
        energy += orc_lj_pair_energy(lj, sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]), eps, sigma);
    }
    return energy;
}

/* lennard_jones.cc:217-257 */
double orc_lj_tail(const orc_lj* lj, const double m[9], uint64_t n, const uint32_t* species) {
    const double volume = fabs(orc_volume(m));
    const double rc = lj->cutoff;
    uint64_t* counts = (uint64_t*)calloc(lj->n_species, sizeof(uint64_t));
    for (uint64_t i = 0; i < n; ++i) counts[species[i]] += 1;
    double total = 0.0;
    for (uint32_t a = 0; a < lj->n_species; ++a) {
        if (counts[a] == 0) continue;
        for (uint32_t b = 0; b < lj->n_species; ++b) {
            if (counts[b] == 0) continue;
            double eps, sigma;
            orc_lj_mixed(lj, a, b, &eps, &sigma);
            const double sr3 = sigma * sigma * sigma;
            const double sr9 = sr3 * sr3 * sr3 / (rc * rc * rc * rc * rc * rc * rc * rc * rc);
            const double sr3rc3 = sr3 / (rc * rc * rc);
            const double integral = eps * sr3 * ((4.0 / 9.0) * sr9 - (4.0 / 3.0) * sr3rc3);
            total += (double)counts[a] * (double)counts[b] * integral;
        }
    }
    free(counts);
    return (2.0 * ORC_PI / volume) * total;
}

/* ------------------------------------------------------------------ Energy grid */

/* framework_energy_grid.cc:207-211 */
void orc_grid_point_counts(const double m[9], double spacing, int out[3]) {
    for (int axis = 0; axis < 3; ++axis) {
        const double w = orc_perpendicular_width(m, axis);
        const int n = (int)lround(w / spacing);
        out[axis] = n < 1 ? 1 : n;
    }
}

typedef struct {
    const orc_lj* lj;
    const double* m;
    uint64_t n_atoms;
    const double *x, *y, *z;
    const uint32_t* species;
    uint32_t guest;
    int counts[3];
    uint64_t begin, end;
    double* out;
} grid_job;

/* framework_energy_grid.cc:224-243: one node = fractional (ix/nx, iy/ny,
 * iz/nz) -> Cartesian -> ascending sum of pairEnergy(min-image r) -> min(E, cap). */
static void* grid_worker(void* arg) {
    const grid_job* j = (const grid_job*)arg;
    const int nx = j->counts[0], ny = j->counts[1], nz = j->counts[2];
    (void)nz;
    for (uint64_t node = j->begin; node < j->end; ++node) {
        const int ix = (int)(node % (uint64_t)nx);
        const int iy = (int)((node / (uint64_t)nx) % (uint64_t)ny);
        const int iz = (int)(node / ((uint64_t)nx * (uint64_t)ny));
        const double f[3] = {(double)ix / (double)nx, (double)iy / (double)ny,
                             (double)iz / (double)j->counts[2]};
        double cart[3];
        orc_frac_to_cart(j->m, f, cart);
        double energy = 0.0;
        for (uint64_t a = 0; a < j->n_atoms; ++a) {
            double eps, sigma;
            orc_lj_mixed(j->lj, j->guest, j->species[a], &eps, &sigma);
            const double pa[3] = {j->x[a], j->y[a], j->z[a]};
            double d[3];
            orc_min_image(j->m, cart, pa, d);
            const double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            energy += orc_lj_pair_energy(j->lj, r, eps, sigma);
        }
        j->out[node - j->begin] = (ORC_GRID_ENERGY_CAP < energy) ? ORC_GRID_ENERGY_CAP : energy;
    }
    return NULL;
}

void orc_grid_build_nodes(const orc_lj* lj, const double m[9], uint64_t n_atoms, const double* x,
                          const double* y, const double* z, const uint32_t* species,
                          uint32_t guest, double spacing, uint64_t node_begin, uint64_t node_end,
                          int n_threads, double* out) {
    int counts[3];
    orc_grid_point_counts(m, spacing, counts);
    if (n_threads < 1) n_threads = 1;
    const uint64_t total = node_end - node_begin;
    if ((uint64_t)n_threads > total) n_threads = total > 0 ? (int)total : 1;
    grid_job* jobs = (grid_job*)calloc((size_t)n_threads, sizeof(grid_job));
    pthread_t* th = (pthread_t*)calloc((size_t)n_threads, sizeof(pthread_t));
    for (int t = 0; t < n_threads; ++t) {
        grid_job* jb = &jobs[t];
        jb->lj = lj;
        jb->m = m;
        jb->n_atoms = n_atoms;
        jb->x = x;
        jb->y = y;
        jb->z = z;
        jb->species = species;
        jb->guest = guest;
        memcpy(jb->counts, counts, sizeof(counts));
        jb->begin = node_begin + total * (uint64_t)t / (uint64_t)n_threads;
        jb->end = node_begin + total * (uint64_t)(t + 1) / (uint64_t)n_threads;
        jb->out = out + (jb->begin - node_begin);
    }
    if (n_threads == 1) {
        grid_worker(&jobs[0]);
    } else {
        for (int t = 0; t < n_threads; ++t) pthread_create(&th[t], NULL, grid_worker, &jobs[t]);
        for (int t = 0; t < n_threads; ++t) pthread_join(th[t], NULL);
    }
    free(jobs);
    free(th);
}

/* framework_energy_grid.cc:251-288 */
double orc_grid_interpolate(const double m[9], const int counts[3], const double* table,
                            const double pos[3]) {
    double f[3];
    orc_cart_to_frac(m, pos, f);
    for (int a = 0; a < 3; ++a) f[a] -= floor(f[a]);
    int i0[3], i1[3];
    double t[3];
    for (int a = 0; a < 3; ++a) {
        const int n = counts[a];
        const double g = f[a] * (double)n;
        const int base = (int)floor(g);
        t[a] = g - (double)base;
        const int wrapped = ((base % n) + n) % n;
        i0[a] = wrapped;
        i1[a] = (wrapped + 1) % n;
    }
    const uint64_t nx = (uint64_t)counts[0], ny = (uint64_t)counts[1];
#define V(ix, iy, iz) table[((uint64_t)(iz) * ny + (uint64_t)(iy)) * nx + (uint64_t)(ix)]
    const double c00 = V(i0[0], i0[1], i0[2]) * (1.0 - t[0]) + V(i1[0], i0[1], i0[2]) * t[0];
    const double c10 = V(i0[0], i1[1], i0[2]) * (1.0 - t[0]) + V(i1[0], i1[1], i0[2]) * t[0];
    const double c01 = V(i0[0], i0[1], i1[2]) * (1.0 - t[0]) + V(i1[0], i0[1], i1[2]) * t[0];
    const double c11 = V(i0[0], i1[1], i1[2]) * (1.0 - t[0]) + V(i1[0], i1[1], i1[2]) * t[0];
#undef V
    const double c0 = c00 * (1.0 - t[1]) + c10 * t[1];
    const double c1 = c01 * (1.0 - t[1]) + c11 * t[1];
    return c0 * (1.0 - t[2]) + c1 * t[2];
}

/* ------------------------------------------------------------------ Ewald */

/* ewald.cc:33-45 (reciprocal vectors) and ewald.cc:137-161 (spherical index
 * set n != 0, |n|^2 < kMax^2 + 2; weight exp(-k^2/4a^2)/k^2). */
uint64_t orc_ewald_terms(const double m[9], double alpha, int kmax, double* k, double* w,
                         uint64_t cap) {
    const double vol = orc_volume(m);
    const double two_pi_over_v = 2.0 * ORC_PI / vol;
    double b[3][3];
    cross3(m + 3, m + 6, b[0]);
    cross3(m + 6, m, b[1]);
    cross3(m, m + 3, b[2]);
    for (int i = 0; i < 3; ++i)
        for (int c = 0; c < 3; ++c) b[i][c] = b[i][c] * two_pi_over_v;
    const double four_a2 = 4.0 * alpha * alpha;
    const int bound = kmax * kmax + 2;
    uint64_t count = 0;
    for (int n0 = -kmax; n0 <= kmax; ++n0) {
        for (int n1 = -kmax; n1 <= kmax; ++n1) {
            for (int n2 = -kmax; n2 <= kmax; ++n2) {
                if (n0 == 0 && n1 == 0 && n2 == 0) continue;
                if (n0 * n0 + n1 * n1 + n2 * n2 >= bound) continue;
                double kv[3];
                for (int c = 0; c < 3; ++c)
                    kv[c] = (b[0][c] * (double)n0 + b[1][c] * (double)n1) + b[2][c] * (double)n2;
                const double k2 = dot3(kv, kv);
                if (count < cap) {
                    if (k) {
                        k[3 * count] = kv[0];
                        k[3 * count + 1] = kv[1];
                        k[3 * count + 2] = kv[2];
                    }
                    if (w) w[count] = exp(-k2 / four_a2) / k2;
                }
                ++count;
            }
        }
    }
    return count;
}

/* ewald.cc:223-249 */
double orc_ewald_real_space_particle_energy(const double m[9], uint64_t n, const double* x,
                                            const double* y, const double* z, const double* q,
                                            double alpha, double rc, uint64_t index,
                                            const uint64_t* excluded, uint64_t n_excluded) {
    double energy = 0.0;
    const double pi[3] = {x[index], y[index], z[index]};
    for (uint64_t j = 0; j < n; ++j) {
        if (j == index) continue;
        if (contains_u64(excluded, n_excluded, j)) continue;
        const double pj[3] = {x[j], y[j], z[j]};
        double d[3];
        orc_min_image(m, pi, pj, d);
        const double r = sqrt(dot3(d, d));
        if (r > rc) continue;
        energy += q[index] * q[j] * (erfc(alpha * r) / r);
    }
    return energy * ORC_COULOMB_K;
}

/* ewald.cc:73-79, ewald_incremental_state.cc:24-30 */
static double erf_over_r(double r, double alpha) {
    if (r < 1e-8) return 2.0 * alpha / sqrt(ORC_PI);
    return erf(alpha * r) / r;
}

/* ewald.cc:251-313, with the neighbour-pair real-space sum taken over every
 * pair i < j within rc (the set VerletList::pairs() filters to). */
void orc_ewald_breakdown(const double m[9], uint64_t n, const double* x, const double* y,
                         const double* z, const double* q, double alpha, double rc, int kmax,
                         const uint64_t* exclusions, uint64_t n_excl, double out[5]) {
    double u_real = 0.0;
    for (uint64_t i = 0; i < n; ++i) {
        for (uint64_t j = i + 1; j < n; ++j) {
            int ex = 0;
            for (uint64_t e = 0; e < n_excl; ++e) {
                const uint64_t a = exclusions[2 * e], b = exclusions[2 * e + 1];
                if ((a == i && b == j) || (a == j && b == i)) {
                    ex = 1;
                    break;
                }
            }
            if (ex) continue;
            const double pi[3] = {x[i], y[i], z[i]}, pj[3] = {x[j], y[j], z[j]};
            double d[3];
            orc_min_image(m, pi, pj, d);
            const double r = sqrt(dot3(d, d));
            if (r > rc) continue;
            u_real += q[i] * q[j] * (erfc(alpha * r) / r);
        }
    }
    out[0] = u_real * ORC_COULOMB_K;
    const double volume = fabs(orc_volume(m));
    const uint64_t nk = orc_ewald_terms(m, alpha, kmax, NULL, NULL, 0);
    double* k = (double*)malloc(sizeof(double) * 3 * nk);
    double* w = (double*)malloc(sizeof(double) * nk);
    orc_ewald_terms(m, alpha, kmax, k, w, nk);
    double u_rec = 0.0;
    for (uint64_t t = 0; t < nk; ++t) {
        double re = 0.0, im = 0.0;
        for (uint64_t i = 0; i < n; ++i) {
            const double p[3] = {x[i], y[i], z[i]};
            const double kr = dot3(k + 3 * t, p);
            re += q[i] * cos(kr);
            im += q[i] * sin(kr);
        }
        u_rec += w[t] * (re * re + im * im);
    }
    free(k);
    free(w);
    out[1] = u_rec * ORC_COULOMB_K * (2.0 * ORC_PI / volume);
    double q2 = 0.0;
    for (uint64_t i = 0; i < n; ++i) q2 += q[i] * q[i];
    out[2] = -ORC_COULOMB_K * (alpha / sqrt(ORC_PI)) * q2;
    double u_ex = 0.0;
    for (uint64_t e = 0; e < n_excl; ++e) {
        const uint64_t i = exclusions[2 * e], j = exclusions[2 * e + 1];
        const double pi[3] = {x[i], y[i], z[i]}, pj[3] = {x[j], y[j], z[j]};
        double d[3];
        orc_min_image(m, pi, pj, d);
        u_ex += q[i] * q[j] * erf_over_r(sqrt(dot3(d, d)), alpha);
    }
    out[3] = -u_ex * ORC_COULOMB_K;
    out[4] = 0.0;
}

/* ------------------------------------------------------------------ EwaldIncrementalState */

/* ewald_incremental_state.cc:32-43 */
static double pair_exclusion_sum(const double m[9], const double* s, uint64_t n, double alpha) {
    double sum = 0.0;
    for (uint64_t i = 0; i < n; ++i) {
        for (uint64_t j = i + 1; j < n; ++j) {
            double d[3];
            orc_min_image(m, s + 4 * i, s + 4 * j, d);
            const double r = sqrt(dot3(d, d));
            sum += s[4 * i + 3] * s[4 * j + 3] * erf_over_r(r, alpha);
        }
    }
    return sum;
}

/* ewald_incremental_state.cc:45-51 */
static double sum_q2(const double* s, uint64_t n) {
    double sum = 0.0;
    for (uint64_t i = 0; i < n; ++i) sum += s[4 * i + 3] * s[4 * i + 3];
    return sum;
}

static void structure_factor(const orc_ewald_state* s, uint64_t n, const double* x,
                             const double* y, const double* z, const double* q, double* sre,
                             double* sim) {
    for (uint64_t t = 0; t < s->nk; ++t) {
        const double* k = s->k + 3 * t;
        double re = 0.0, im = 0.0;
        for (uint64_t i = 0; i < n; ++i) {
            const double kr = k[0] * x[i] + k[1] * y[i] + k[2] * z[i];
            re += q[i] * cos(kr);
            im += q[i] * sin(kr);
        }
        sre[t] = re;
        sim[t] = im;
    }
}

/* ewald_incremental_state.cc:55-83 */
int orc_ews_init(orc_ewald_state* s, const double m[9], double alpha, int kmax, uint64_t n,
                 const double* x, const double* y, const double* z, const double* q) {
    memcpy(s->m, m, sizeof(double) * 9);
    s->alpha = alpha;
    s->volume = fabs(orc_volume(m));
    s->nk = orc_ewald_terms(m, alpha, kmax, NULL, NULL, 0);
    s->k = (double*)malloc(sizeof(double) * 3 * (s->nk ? s->nk : 1));
    s->w = (double*)malloc(sizeof(double) * (s->nk ? s->nk : 1));
    s->sre = (double*)malloc(sizeof(double) * (s->nk ? s->nk : 1));
    s->sim = (double*)malloc(sizeof(double) * (s->nk ? s->nk : 1));
    orc_ewald_terms(m, alpha, kmax, s->k, s->w, s->nk);
    structure_factor(s, n, x, y, z, q, s->sre, s->sim);
    double q2 = 0.0;
    for (uint64_t i = 0; i < n; ++i) q2 += q[i] * q[i];
    s->self_energy = -ORC_COULOMB_K * (alpha / sqrt(ORC_PI)) * q2;
    s->exclusion_energy = 0.0;
    return 0;
}

void orc_ews_free(orc_ewald_state* s) {
    free(s->k);
    free(s->w);
    free(s->sre);
    free(s->sim);
    memset(s, 0, sizeof(*s));
}

/* ewald_incremental_state.cc:85-93 */
double orc_ews_energy(const orc_ewald_state* s) {
    double sum = 0.0;
    for (uint64_t t = 0; t < s->nk; ++t) sum += s->w[t] * (s->sre[t] * s->sre[t] + s->sim[t] * s->sim[t]);
    const double reciprocal = sum * ORC_COULOMB_K * (2.0 * ORC_PI / s->volume);
    return reciprocal + s->self_energy + s->exclusion_energy;
}

/* ewald_incremental_state.cc:95-136 */
double orc_ews_delta(const orc_ewald_state* s, const double* removed, uint64_t nr,
                     const double* added, uint64_t na, double* dre, double* dim, double* dself,
                     double* dexcl) {
    const double prefactor = ORC_COULOMB_K * (2.0 * ORC_PI / s->volume);
    double wsum = 0.0;
    for (uint64_t t = 0; t < s->nk; ++t) {
        const double* k = s->k + 3 * t;
        double re = 0.0, im = 0.0;
        for (uint64_t i = 0; i < na; ++i) {
            const double* p = added + 4 * i;
            const double kr = k[0] * p[0] + k[1] * p[1] + k[2] * p[2];
            re += p[3] * cos(kr);
            im += p[3] * sin(kr);
        }
        for (uint64_t i = 0; i < nr; ++i) {
            const double* p = removed + 4 * i;
            const double kr = k[0] * p[0] + k[1] * p[1] + k[2] * p[2];
            re -= p[3] * cos(kr);
            im -= p[3] * sin(kr);
        }
        const double nre = s->sre[t] + re;
        const double nim = s->sim[t] + im;
        const double old_mag = s->sre[t] * s->sre[t] + s->sim[t] * s->sim[t];
        const double new_mag = nre * nre + nim * nim;
        wsum += s->w[t] * (new_mag - old_mag);
        if (dre) dre[t] = re;
        if (dim) dim[t] = im;
    }
    const double rec = prefactor * wsum;
    const double self_pref = -ORC_COULOMB_K * (s->alpha / sqrt(ORC_PI));
    const double self = self_pref * (sum_q2(added, na) - sum_q2(removed, nr));
    const double ax = pair_exclusion_sum(s->m, added, na, s->alpha);
    const double rx = pair_exclusion_sum(s->m, removed, nr, s->alpha);
    const double excl = -ORC_COULOMB_K * (ax - rx);
    if (dself) *dself = self;
    if (dexcl) *dexcl = excl;
    return rec + self + excl;
}

/* ewald_incremental_state.cc:138-172 */
void orc_ews_commit(orc_ewald_state* s, const double* removed, uint64_t nr, const double* added,
                    uint64_t na) {
    double* dre = (double*)malloc(sizeof(double) * (s->nk ? s->nk : 1));
    double* dim = (double*)malloc(sizeof(double) * (s->nk ? s->nk : 1));
    double dself = 0.0, dexcl = 0.0;
    orc_ews_delta(s, removed, nr, added, na, dre, dim, &dself, &dexcl);
    for (uint64_t t = 0; t < s->nk; ++t) {
        s->sre[t] += dre[t];
        s->sim[t] += dim[t];
    }
    s->self_energy += dself;
    s->exclusion_energy += dexcl;
    free(dre);
    free(dim);
}

static double molecules_exclusion(const orc_ewald_state* s, const double* x, const double* y,
                                  const double* z, const double* q, uint64_t n_mol,
                                  const uint64_t* offsets, const uint64_t* indices, int scaled) {
    double exclusion = 0.0;
    for (uint64_t k = 0; k < n_mol; ++k) {
        const uint64_t cnt = offsets[k + 1] - offsets[k];
        double* sites = (double*)malloc(sizeof(double) * 4 * (cnt ? cnt : 1));
        for (uint64_t j = 0; j < cnt; ++j) {
            const uint64_t i = indices[offsets[k] + j];
            sites[4 * j] = x[i];
            sites[4 * j + 1] = y[i];
            sites[4 * j + 2] = z[i];
            sites[4 * j + 3] = q[i];
        }
        const double e = pair_exclusion_sum(s->m, sites, cnt, s->alpha);
        exclusion += scaled ? -ORC_COULOMB_K * e : e;
        free(sites);
    }
    return exclusion;
}

/* ewald_incremental_state.cc:174-212 */
double orc_ews_recompute(const orc_ewald_state* s, uint64_t n, const double* x, const double* y,
                         const double* z, const double* q, uint64_t n_mol,
                         const uint64_t* offsets, const uint64_t* indices) {
    double rsum = 0.0;
    for (uint64_t t = 0; t < s->nk; ++t) {
        const double* k = s->k + 3 * t;
        double re = 0.0, im = 0.0;
        for (uint64_t i = 0; i < n; ++i) {
            const double kr = k[0] * x[i] + k[1] * y[i] + k[2] * z[i];
            re += q[i] * cos(kr);
            im += q[i] * sin(kr);
        }
        rsum += s->w[t] * (re * re + im * im);
    }
    const double reciprocal = rsum * ORC_COULOMB_K * (2.0 * ORC_PI / s->volume);
    double q2 = 0.0;
    for (uint64_t i = 0; i < n; ++i) q2 += q[i] * q[i];
    const double self = -ORC_COULOMB_K * (s->alpha / sqrt(ORC_PI)) * q2;
    const double exclusion = molecules_exclusion(s, x, y, z, q, n_mol, offsets, indices, 1);
    return reciprocal + self + exclusion;
}

/* ewald_incremental_state.cc:214-247 */
void orc_ews_resync(orc_ewald_state* s, uint64_t n, const double* x, const double* y,
                    const double* z, const double* q, uint64_t n_mol, const uint64_t* offsets,
                    const uint64_t* indices) {
    structure_factor(s, n, x, y, z, q, s->sre, s->sim);
    double q2 = 0.0;
    for (uint64_t i = 0; i < n; ++i) q2 += q[i] * q[i];
    s->self_energy = -ORC_COULOMB_K * (s->alpha / sqrt(ORC_PI)) * q2;
    const double e = molecules_exclusion(s, x, y, z, q, n_mol, offsets, indices, 0);
    s->exclusion_energy = -ORC_COULOMB_K * e;
}

/* ------------------------------------------------------------------ Rigid-body helpers */

/* monte_carlo_engine.cc:56-63 */
void orc_random_unit_quaternion(double u0, double u1, double u2, double q[4]) {
    const double r1 = sqrt(1.0 - u0);
    const double r2 = sqrt(u0);
    const double t1 = 2.0 * ORC_PI * u1;
    const double t2 = 2.0 * ORC_PI * u2;
    q[0] = r2 * cos(t2);
    q[1] = r1 * sin(t1);
    q[2] = r1 * cos(t1);
    q[3] = r2 * sin(t2);
}

/* monte_carlo_engine.cc:68-72 */
void orc_rotate_by_quaternion(const double v[3], const double q[4], double out[3]) {
    const double qv[3] = {q[1], q[2], q[3]};
    double c[3], t[3], c2[3];
    cross3(qv, v, c);
    for (int i = 0; i < 3; ++i) t[i] = c[i] * 2.0;
    cross3(qv, t, c2);
    for (int i = 0; i < 3; ++i) out[i] = (v[i] + t[i] * q[0]) + c2[i];
}

/* monte_carlo_engine.cc:40-44 */
void orc_rotate_about_axis(const double v[3], const double axis[3], double theta, double out[3]) {
    const double c = cos(theta);
    const double s = sin(theta);
    double cr[3];
    cross3(axis, v, cr);
    const double ad = dot3(axis, v) * (1.0 - c);
    for (int i = 0; i < 3; ++i) out[i] = (v[i] * c + cr[i] * s) + axis[i] * ad;
}

/* ------------------------------------------------------------------ Widom */

typedef struct {
    const orc_lj* lj;
    const orc_ewald_params* ew;
    const double* m;
    uint64_t n;
    double *x, *y, *z, *q; /* framework + room for guest sites */
    uint32_t* species;
    const orc_species* guest;
    const orc_ewald_state* ews;
    double temperature;
    uint64_t seed, stream, t0, t1;
    int draw_order;
    double* per_trial;
    double sum;
} widom_job;

/* monte_carlo_engine.cc:881-914 for trials [t0, t1). The draw layout is
 * counter-indexed: trial t starts at call index 3t (one site) or 6t (several). */
static void* widom_worker(void* arg) {
    widom_job* j = (widom_job*)arg;
    const orc_species* g = j->guest;
    const uint32_t ns = g->n_sites;
    const uint64_t per = ns > 1 ? 6 : 3;
    const double* m = j->m;
    uint64_t idx[64];
    double sites[4 * 64];
    double sum = 0.0;
    for (uint64_t t = j->t0; t < j->t1; ++t) {
        const uint64_t c0 = per * t;
        double u[3] = {orc_philox_uniform(j->seed, j->stream, c0),
                       orc_philox_uniform(j->seed, j->stream, c0 + 1),
                       orc_philox_uniform(j->seed, j->stream, c0 + 2)};
        if (j->draw_order == ORC_DRAWS_RIGHT_TO_LEFT) {
            const double tmp = u[0];
            u[0] = u[2];
            u[2] = tmp;
        }
        double ref[3];
        for (int c = 0; c < 3; ++c) ref[c] = (m[c] * u[0] + m[3 + c] * u[1]) + m[6 + c] * u[2];
        double quat[4] = {1.0, 0.0, 0.0, 0.0};
        if (ns > 1) {
            double v[3] = {orc_philox_uniform(j->seed, j->stream, c0 + 3),
                           orc_philox_uniform(j->seed, j->stream, c0 + 4),
                           orc_philox_uniform(j->seed, j->stream, c0 + 5)};
            if (j->draw_order == ORC_DRAWS_RIGHT_TO_LEFT) {
                const double tmp = v[0];
                v[0] = v[2];
                v[2] = tmp;
            }
            orc_random_unit_quaternion(v[0], v[1], v[2], quat);
        }
        for (uint32_t s = 0; s < ns; ++s) {
            const double local[3] = {g->x[s], g->y[s], g->z[s]};
            double rot[3];
            if (ns > 1)
                orc_rotate_by_quaternion(local, quat, rot);
            else {
                rot[0] = local[0];
                rot[1] = local[1];
                rot[2] = local[2];
            }
            const uint64_t k = j->n + s;
            j->x[k] = ref[0] + rot[0];
            j->y[k] = ref[1] + rot[1];
            j->z[k] = ref[2] + rot[2];
            j->q[k] = g->charge[s];
            j->species[k] = g->lj_species[s];
            idx[s] = k;
            sites[4 * s] = j->x[k];
            sites[4 * s + 1] = j->y[k];
            sites[4 * s + 2] = j->z[k];
            sites[4 * s + 3] = g->charge[s];
        }
        const uint64_t ntot = j->n + ns;
        double du = 0.0;
        for (uint32_t s = 0; s < ns; ++s)
            du += orc_lj_particle_energy(j->lj, m, ntot, j->x, j->y, j->z, j->species, idx[s], idx,
                                         ns);
        if (j->ew && j->ew->alpha > 0.0) {
            double e = 0.0;
            for (uint32_t s = 0; s < ns; ++s)
                e += orc_ewald_real_space_particle_energy(m, ntot, j->x, j->y, j->z, j->q,
                                                          j->ew->alpha, j->ew->rc, idx[s], idx, ns);
            du += e;
            du += orc_ews_delta(j->ews, NULL, 0, sites, ns, NULL, NULL, NULL, NULL);
        }
        if (j->per_trial) j->per_trial[t - j->t0] = du;
        sum += exp(-du / j->temperature);
    }
    j->sum = sum;
    return NULL;
}

double orc_widom(const orc_lj* lj, const orc_ewald_params* ew, const double m[9], uint64_t n,
                 const double* x, const double* y, const double* z, const double* q,
                 const uint32_t* species, const orc_species* guest, double temperature,
                 uint64_t seed, uint64_t stream, uint64_t first_trial, uint64_t n_trials,
                 int draw_order, int n_threads, double* per_trial) {
    if (guest->n_sites == 0 || guest->n_sites > 64 || n_trials == 0) return 0.0;
    orc_ewald_state ews;
    memset(&ews, 0, sizeof(ews));
    const int charged = ew && ew->alpha > 0.0;
    if (charged) orc_ews_init(&ews, m, ew->alpha, ew->kmax, n, x, y, z, q);
    if (n_threads < 1) n_threads = 1;
    if ((uint64_t)n_threads > n_trials) n_threads = (int)n_trials;
    widom_job* jobs = (widom_job*)calloc((size_t)n_threads, sizeof(widom_job));
    pthread_t* th = (pthread_t*)calloc((size_t)n_threads, sizeof(pthread_t));
    const uint64_t cap = n + guest->n_sites;
    for (int t = 0; t < n_threads; ++t) {
        widom_job* jb = &jobs[t];
        jb->lj = lj;
        jb->ew = ew;
        jb->m = m;
        jb->n = n;
        jb->x = (double*)malloc(sizeof(double) * cap);
        jb->y = (double*)malloc(sizeof(double) * cap);
        jb->z = (double*)malloc(sizeof(double) * cap);
        jb->q = (double*)malloc(sizeof(double) * cap);
        jb->species = (uint32_t*)malloc(sizeof(uint32_t) * cap);
        memcpy(jb->x, x, sizeof(double) * n);
        memcpy(jb->y, y, sizeof(double) * n);
        memcpy(jb->z, z, sizeof(double) * n);
        for (uint64_t i = 0; i < n; ++i) jb->q[i] = q ? q[i] : 0.0;
        memcpy(jb->species, species, sizeof(uint32_t) * n);
        jb->guest = guest;
        jb->ews = charged ? &ews : NULL;
        jb->temperature = temperature;
        jb->seed = seed;
        jb->stream = stream;
        jb->t0 = first_trial + n_trials * (uint64_t)t / (uint64_t)n_threads;
        jb->t1 = first_trial + n_trials * (uint64_t)(t + 1) / (uint64_t)n_threads;
        jb->draw_order = draw_order;
        jb->per_trial = per_trial ? per_trial + (jb->t0 - first_trial) : NULL;
    }
    if (n_threads == 1)
        widom_worker(&jobs[0]);
    else {
        for (int t = 0; t < n_threads; ++t) pthread_create(&th[t], NULL, widom_worker, &jobs[t]);
        for (int t = 0; t < n_threads; ++t) pthread_join(th[t], NULL);
    }
    /* With one thread this is the reference's sequential sum; with several it
     * is a per-thread partial sum (same terms, different association). */
    double sum = 0.0;
    for (int t = 0; t < n_threads; ++t) {
        sum += jobs[t].sum;
        free(jobs[t].x);
        free(jobs[t].y);
        free(jobs[t].z);
        free(jobs[t].q);
        free(jobs[t].species);
    }
    free(jobs);
    free(th);
    if (charged) orc_ews_free(&ews);
    return (sum / (double)n_trials) / temperature;
}

/* ------------------------------------------------------------------ Acceptance */

/* gcmc_acceptance.hpp:28-33 */
double orc_insertion_ratio(double f, double v, uint64_t n_before, double t, double du) {
    return (f * v / t) / (double)(n_before + 1) * exp(-du / t);
}
/* gcmc_acceptance.hpp:39-44 */
double orc_deletion_ratio(double f, double v, uint64_t n_before, double t, double du) {
    return (double)n_before / (f * v / t) * exp(-du / t);
}
/* gcmc_acceptance.hpp:49-51 */
double orc_metropolis_ratio(double t, double du) { return exp(-du / t); }
/* gcmc_acceptance.hpp:89-95 */
double orc_swap_ratio(double f_from, double f_to, uint64_t n_from, uint64_t n_to, double t,
                      double du) {
    return (f_to / f_from) * ((double)n_from / (double)(n_to + 1)) * exp(-du / t);
}
/* gcmc_acceptance.hpp:101 */
double orc_clamp_probability(double r) { return r < 1.0 ? r : 1.0; }

/* ------------------------------------------------------------------ Peng-Robinson */

/* the gas-phase Newton root shared by both forms (peng_robinson.cc:62-100, 236-276) */
static double orc_pr_root(double A, double B) {
    const double c2 = -(1.0 - B);
    const double c1 = A - 3.0 * B * B - 2.0 * B;
    const double c0 = -(A * B - B * B - B * B * B);
    double zz = 1.0;
    for (int iter = 0; iter < 100; ++iter) {
        const double fz = zz * zz * zz + c2 * zz * zz + c1 * zz + c0;
        if (fabs(fz) < 1e-14) break;
        const double fp = 3.0 * zz * zz + 2.0 * c2 * zz + c1;
        if (fp == 0.0) break;
        zz -= fz / fp;
        if (!(zz > B)) zz = B + 0.5 * (1.0 - B > 0 ? 1.0 - B : 1.0);
    }
    return zz;
}

/* PengRobinsonMixture (peng_robinson.cc:112-309): one-fluid mixing; Z from the
 * mixture's A (a_mix summed as x_i x_j a_ij, :229-235) and B; the fugacities
 * from a_mix summed as (x_i x_j sqrt(a_i a_j)) (1 - k_ij) (:288-295). */
int orc_pr_mixture(uint32_t n, const double* tc, const double* pc, const double* omega,
                   const double* kij, double t, double p, const double* x, double* z_out,
                   double* f_out) {
    const double R = 8.31446261815324;
    if (n < 2 || n > 64) return -1;
    double b[64], aa[64];
    double sum = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        if (!(tc[i] > 0.0) || !(pc[i] > 0.0) || !(x[i] >= 0.0)) return -1;
        sum += x[i];
    }
    if (fabs(sum - 1.0) > 1e-9 || !(t > 0.0) || !(p > 0.0)) return -1;
    for (uint32_t i = 0; i < n; ++i) {
        const double a = 0.45724 * R * R * tc[i] * tc[i] / pc[i];
        b[i] = 0.07780 * R * tc[i] / pc[i];
        const double kappa = 0.37464 + 1.54226 * omega[i] - 0.26992 * omega[i] * omega[i];
        const double term = 1.0 + kappa * (1.0 - sqrt(t / tc[i]));
        aa[i] = a * (term * term);
    }
    double amix_z = 0.0, amix = 0.0, bmix = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        bmix += x[i] * b[i];
        for (uint32_t j = 0; j < n; ++j) {
            const double k = kij ? kij[(size_t)i * n + j] : 0.0;
            const double aij = sqrt(aa[i] * aa[j]) * (1.0 - k);
            amix_z += x[i] * x[j] * aij;
            amix += x[i] * x[j] * sqrt(aa[i] * aa[j]) * (1.0 - k);
        }
    }
    const double B = bmix * p / (R * t);
    const double zz = orc_pr_root(amix_z * p / (R * R * t * t), B);
    const double A = amix * p / (R * R * t * t);
    const double sqrt2 = 1.41421356237309504880;
    for (uint32_t i = 0; i < n; ++i) {
        double sj = 0.0;
        for (uint32_t j = 0; j < n; ++j)
            sj += x[j] * sqrt(aa[i] * aa[j]) * (1.0 - (kij ? kij[(size_t)i * n + j] : 0.0));
        const double lnphi = (b[i] / bmix) * (zz - 1.0) - log(zz - B) -
                             (A / (2.0 * sqrt2 * B)) * ((2.0 / amix) * sj - b[i] / bmix) *
                                 log((zz + (1.0 + sqrt2) * B) / (zz + (1.0 - sqrt2) * B));
        f_out[i] = x[i] * exp(lnphi) * p;
    }
    if (z_out) *z_out = zz;
    return 0;
}

/* peng_robinson.cc:10-110 (kGasConstant peng_robinson.hpp:46) */
double orc_pr_fugacity(double tc, double pc, double omega, double t, double p) {
    const double R = 8.31446261815324;
    const double a = 0.45724 * R * R * tc * tc / pc;
    const double b = 0.07780 * R * tc / pc;
    const double kappa = 0.37464 + 1.54226 * omega - 0.26992 * omega * omega;
    const double term = 1.0 + kappa * (1.0 - sqrt(t / tc));
    const double aalpha = a * (term * term);
    const double A = aalpha * p / (R * R * t * t);
    const double B = b * p / (R * t);
    const double c2 = -(1.0 - B);
    const double c1 = A - 3.0 * B * B - 2.0 * B;
    const double c0 = -(A * B - B * B - B * B * B);
    double zz = 1.0;
    for (int iter = 0; iter < 100; ++iter) {
        const double fz = zz * zz * zz + c2 * zz * zz + c1 * zz + c0;
        if (fabs(fz) < 1e-14) break;
        const double fp = 3.0 * zz * zz + 2.0 * c2 * zz + c1;
        if (fp == 0.0) break;
        zz -= fz / fp;
        if (!(zz > B)) zz = B + 0.5 * (1.0 - B > 0 ? 1.0 - B : 1.0);
    }
    const double sqrt2 = 1.41421356237309504880;
    const double lnphi = (zz - 1.0) - log(zz - B) -
                         (A / (2.0 * sqrt2 * B)) * log((zz + (1.0 + sqrt2) * B) / (zz + (1.0 - sqrt2) * B));
    return exp(lnphi) * p;
}
