// Widom test-particle insertion on sm_103a.
//
// Reference: MonteCarloEngine::widomInsertionHenryCoefficient
// (engines/monte_carlo/monte_carlo_engine.cc:850-917). Trial t of a freshly
// seeded engine consumes Philox call indices 3t..3t+2 (position) and, for a
// multi-site species, 3t+3..3t+5 (orientation, Shoemake quaternion,
// monte_carlo_engine.cc:56-72), so each thread computes its own trial
// directly from the counter. deltaU = sum over sites of the LJ energy against
// every framework atom (lennard_jones.cc:158-182) + the real-space Ewald
// energy (ewald.cc:223-249) + EwaldIncrementalState::proposeInsertion against
// the framework's S(k) (ewald_incremental_state.cc:95-136, 152-154).
//
// One thread per trial; the framework is streamed through shared memory in
// tiles (every thread reads the same atom: a broadcast). The reciprocal delta
// walks the reference's term order row by row (n0, n1) and advances
// exp(i k.r) along n2 by one complex multiply per term and site, instead of
// one sincos per term and site. Boltzmann weights are reduced as an FP64
// log-sum-exp: per block (max, sum exp(l - max), sum exp(2(l - max))), then
// across blocks in block order.

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "ff.cuh"
#include "grid.cuh"

namespace alea {

namespace {

constexpr int WT = 128;        // trials per block
// FP32 form, charged trials: Coulomb pairs closer than 6 A are evaluated in
// double-float (ff.cuh near_coulomb_ff; closer, a pair's real-space term
// reaches 1e2-1e5 K, where FP32's ~1e-7 relative rounding would leave up to
// ~1e-2 K)
constexpr float NEAR_COULOMB_R2 = 36.0f;
constexpr int ATILE = 512;     // framework atoms per shared-memory tile
constexpr int MAXS = 8;        // sites per guest molecule
constexpr int MAXT = 64;       // LJ species
// FP32 form, uncharged trials: pairs closer than CLOSE_SIGMA x sigma (and,
// for plain truncation, pairs whose cutoff decision FP32 cannot make) are
// listed per thread, up to CLOSE_MAX per tile and site, and redone in
// double-float after the tile; the rest run on FP32 displacements from the
// atoms' FP32 positions (the image then carries up to ~ulp(L) ~ 4e-6 A, which
// beyond 1.25 sigma moves a pair energy by < 3e-4 K).
constexpr int CLOSE_MAX = 16;
// FP32 form, charged: a thread's near-Coulomb pairs (within 6 A) of one site
// and tile are listed, up to NEAR_MAX, and evaluated after the tile's loop:
// evaluated where found, a warp paid the whole double-float sequence for each
// atom that was near any one of its 32 trials.
constexpr int NEAR_MAX = 80;
constexpr float CLOSE_SIGMA2 = 1.25f * 1.25f;
constexpr float CUT_BAND = 1e-5f;  // relative band of r^2 around rc^2 redone in double-float

struct GuestSite {
    double x, y, z, q;
    uint32_t lj;
};

struct WidomParams {
    Lattice L;
    uint64_t n_atoms;
    int n_sites;
    GuestSite site[MAXS];
    uint32_t n_species;
    double rc, rc2;
    int trunc;
    double temperature;
    // electrostatics (charged == 0: none)
    int charged;
    double alpha, rc_ewald;
    uint64_t nk;
    int n_rows;
    double b[9];
    double self_pref, rec_pref;
    float lh[9], ll[9], linv[9];  // FP32 form: rows a_i as hi + lo; the inverse
};

struct KRow {
    int n0, n1, m, t0;
};

// FP32 form: a site's pair terms with one framework type: 4 eps sigma^12,
// 4 eps sigma^6, the shift terms, and sigma^2 below which the pair stays FP64.
struct PairF32W {
    float a, b, shift, dvdrc, sig2;
};

// cross(qv, v) with non-contracted arithmetic (monte_carlo_engine.cc:25-27)
__device__ __forceinline__ void cross_rn(const double* a, const double* b, double* o) {
    o[0] = sub_rn(mul_rn(a[1], b[2]), mul_rn(a[2], b[1]));
    o[1] = sub_rn(mul_rn(a[2], b[0]), mul_rn(a[0], b[2]));
    o[2] = sub_rn(mul_rn(a[0], b[1]), mul_rn(a[1], b[0]));
}

// Device data of one Widom context.
struct WidomPtrs {
    const double4* atoms;
    const float4* atoms32;  // FP32 form: per atom {x, y, z, charge} hi, then lo
    const uint32_t* types;
    const PairParams* table;
    const KRow* rows;
    const double* w;
    const double* sre;
    const double* sim;
    const float4* swk32;  // FP32 form: per term {w hi, w lo, Re S hi, lo}, {Im S hi, lo, 0, 0}
};

// One block of WT trials: trials first + block WT + threadIdx.x; writes the
// block's (max, s1, s2) to partial[3 block ..].
// Q: the context may be charged (false: an LJ-only instantiation, compiled
// without the electrostatic sums and with fewer registers).
template <typename Real, bool Q>
__device__ __forceinline__ void widom_block(const WidomParams& P, const WidomPtrs& D, uint64_t block,
                                            uint64_t seed, uint64_t stream, uint64_t first,
                                            uint64_t n, int draw_order, double* __restrict__ per_trial,
                                            double* __restrict__ partial, const ProposalTable& tab,
                                            double* __restrict__ frac_out,
                                            float* __restrict__ samples_out) {
    const double4* __restrict__ atoms = D.atoms;
    const uint32_t* __restrict__ types = D.types;
    const PairParams* __restrict__ table = D.table;
    const KRow* __restrict__ rows = D.rows;
    const double* __restrict__ w = D.w;
    const double* __restrict__ sre = D.sre;
    const double* __restrict__ sim = D.sim;
    __shared__ double4 tile[ATILE];
    __shared__ uint32_t ttype[ATILE];
    __shared__ PairParams pp[sizeof(Real) == 8 ? MAXS * MAXT : 1];
    __shared__ PairF32W ppf[sizeof(Real) == 4 ? MAXS * MAXT : 1];
    __shared__ PairCloseFF ppc[sizeof(Real) == 4 ? MAXS * MAXT : 1];
    __shared__ double red[WT];
    __shared__ uint16_t closej[sizeof(Real) == 4 ? CLOSE_MAX * WT : 1];
    __shared__ uint16_t nearj[(sizeof(Real) == 4 && Q) ? NEAR_MAX * WT : 1];

    const int ns = P.n_sites;
    for (int i = threadIdx.x; i < ns * (int)P.n_species; i += WT) {
        const int s = i / P.n_species, t = i % P.n_species;
        const PairParams q = table[(size_t)P.site[s].lj * P.n_species + t];
        if constexpr (sizeof(Real) == 8) {
            pp[s * MAXT + t] = q;
        } else {
            const double s2 = q.sigma * q.sigma, s6 = s2 * s2 * s2;
            const double sh = P.trunc != ALEA_TRUNCATED ? q.shift : 0.0;
            ppf[s * MAXT + t] = PairF32W{(float)(4.0 * q.eps * s6 * s6), (float)(4.0 * q.eps * s6),
                                         (float)sh, (float)q.dvdrc, (float)s2};
            const ff fs2 = ff_from(s2), fe4 = ff_from(4.0 * q.eps), fsh = ff_from(sh);
            ppc[s * MAXT + t] = PairCloseFF{fs2.hi, fs2.lo, fe4.hi, fe4.lo, fsh.hi, fsh.lo,
                                            (float)q.dvdrc, 0.f};
        }
    }

    const uint64_t local = block * WT + threadIdx.x;
    const bool active = local < n;
    const uint64_t trial = first + local;
    const double* M = P.L.m;

    // ---- position and orientation (monte_carlo_engine.cc:882-901)
    const uint64_t per = tab.cells > 0 ? 8 : ns > 1 ? 6 : 3;
    const uint64_t c0 = per * trial;
    double u[3];
    uint32_t cell = 0;
    if (tab.cells > 0) {
        // learned proposal: a cell from the tabulated CDF (first entry above
        // the draw), then a uniform point inside it
        const uint32_t C = (uint32_t)tab.cells;
        const double uc = philox_uniform(seed, stream, c0);
        uint32_t lo = 0, hi = C * C * C - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) / 2;
            if (__ldg(&tab.cdf[mid]) > uc) hi = mid; else lo = mid + 1;
        }
        cell = lo;
        const uint32_t ix = cell % C, iy = (cell / C) % C, iz = cell / (C * C);
        u[0] = ((double)ix + philox_uniform(seed, stream, c0 + 1)) / (double)C;
        u[1] = ((double)iy + philox_uniform(seed, stream, c0 + 2)) / (double)C;
        u[2] = ((double)iz + philox_uniform(seed, stream, c0 + 3)) / (double)C;
    } else {
        u[0] = philox_uniform(seed, stream, c0);
        u[1] = philox_uniform(seed, stream, c0 + 1);
        u[2] = philox_uniform(seed, stream, c0 + 2);
        if (draw_order == ALEA_DRAWS_RIGHT_TO_LEFT) {
            const double tmp = u[0];
            u[0] = u[2];
            u[2] = tmp;
        }
    }
    double ref[3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
        ref[c] = add_rn(add_rn(mul_rn(M[c], u[0]), mul_rn(M[3 + c], u[1])), mul_rn(M[6 + c], u[2]));
    double q[4] = {1.0, 0.0, 0.0, 0.0};
    if (ns > 1) {
        const uint64_t q0 = tab.cells > 0 ? c0 + 4 : c0 + 3;
        double v[3] = {philox_uniform(seed, stream, q0), philox_uniform(seed, stream, q0 + 1),
                       philox_uniform(seed, stream, q0 + 2)};
        if (tab.cells == 0 && draw_order == ALEA_DRAWS_RIGHT_TO_LEFT) {
            const double tmp = v[0];
            v[0] = v[2];
            v[2] = tmp;
        }
        const double r1 = __dsqrt_rn(sub_rn(1.0, v[0]));
        const double r2 = __dsqrt_rn(v[0]);
        const double t1 = mul_rn(2.0 * kPi, v[1]);
        const double t2 = mul_rn(2.0 * kPi, v[2]);
        q[0] = mul_rn(r2, cos(t2));
        q[1] = mul_rn(r1, sin(t1));
        q[2] = mul_rn(r1, cos(t1));
        q[3] = mul_rn(r2, sin(t2));
    }
    double sx[MAXS], sy[MAXS], sz[MAXS];
#pragma unroll
    for (int s = 0; s < MAXS; ++s) {
        if (s >= ns) break;
        double loc[3] = {P.site[s].x, P.site[s].y, P.site[s].z};
        double rot[3] = {loc[0], loc[1], loc[2]};
        if (ns > 1) {  // rotateByQuaternion (monte_carlo_engine.cc:68-72)
            const double qv[3] = {q[1], q[2], q[3]};
            double c[3], t[3], c2[3];
            cross_rn(qv, loc, c);
            for (int i = 0; i < 3; ++i) t[i] = mul_rn(c[i], 2.0);
            cross_rn(qv, t, c2);
            for (int i = 0; i < 3; ++i) rot[i] = add_rn(add_rn(loc[i], mul_rn(t[i], q[0])), c2[i]);
        }
        sx[s] = add_rn(ref[0], rot[0]);
        sy[s] = add_rn(ref[1], rot[1]);
        sz[s] = add_rn(ref[2], rot[2]);
    }

    // ---- LJ and real-space sums against the framework, atom tiles in smem
    double lj_site[MAXS], es_site[MAXS];
#pragma unroll
    for (int s = 0; s < MAXS; ++s) {
        lj_site[s] = 0.0;
        es_site[s] = 0.0;
    }
    for (uint64_t base = 0; base < P.n_atoms; base += ATILE) {
        __syncthreads();
        const int cnt = (int)min((uint64_t)ATILE, P.n_atoms - base);
        for (int i = threadIdx.x; i < cnt; i += WT) {
            if constexpr (sizeof(Real) == 8) {
                tile[i] = atoms[base + i];
            } else {  // {x, y, z hi, charge}, {x, y, z lo, 0}: split once at creation
                float4* t4 = reinterpret_cast<float4*>(&tile[i]);
                t4[0] = D.atoms32[2 * (base + i)];
                t4[1] = D.atoms32[2 * (base + i) + 1];
            }
            ttype[i] = types[base + i];
        }
        __syncthreads();
#pragma unroll
        for (int s = 0; s < MAXS; ++s) {
            if (s >= ns) break;
            Real lj_acc = 0, es_acc = 0;
            double lj_close = 0.0, es_near = 0.0;
            if constexpr (sizeof(Real) == 8) {
                for (int j = 0; j < cnt; ++j) {
                    const double4 a = tile[j];
                    double dx, dy, dz;
                    min_image(P.L, a.x - sx[s], a.y - sy[s], a.z - sz[s], dx, dy, dz);
                    const double r2 = dx * dx + dy * dy + dz * dz;
                    const double r = sqrt(r2);
                    lj_acc += lj_pair_rt(P.trunc, r, P.rc, pp[s * MAXT + ttype[j]]);
                    if ((Q && P.charged) && r <= P.rc_ewald) es_acc += a.w * (erfc(P.alpha * r) / r);
                }
            } else if (!(Q && P.charged)) {
                // FP32 displacement (hi and lo parts subtracted apart: exact
                // for nearby atoms) and image on the FP32 pipe; close pairs and
                // cutoff-ambiguous ones listed and redone in double-float
                const ff px = ff_from(sx[s]), py = ff_from(sy[s]), pz = ff_from(sz[s]);
                const float rc2f = (float)P.rc2, rcf = (float)P.rc;
                const float band = P.trunc == ALEA_TRUNCATED ? CUT_BAND * rc2f : 0.f;
                const PairF32W* rowf = ppf + s * MAXT;
                ff close_acc{0.f, 0.f};
                uint16_t* mine = closej + threadIdx.x;  // stride WT: bank-conflict free
                int nclose = 0;
                // double-float energy of pair j (its cutoff decided in double-float)
                auto redo = [&](int j) {
                    const float4* t4 = reinterpret_cast<const float4*>(&tile[j]);
                    const float4 ah = t4[0], al = t4[1];
                    ff dx = ff_add(ff{ah.x, al.x}, ff{-px.hi, -px.lo});
                    ff dy = ff_add(ff{ah.y, al.y}, ff{-py.hi, -py.lo});
                    ff dz = ff_add(ff{ah.z, al.z}, ff{-pz.hi, -pz.lo});
                    ff_min_image(P.lh, P.ll, P.linv, P.L.ortho, dx, dy, dz);
                    const ff rr = ff_add(ff_add(ff_mul(dx, dx), ff_mul(dy, dy)), ff_mul(dz, dz));
                    const ff over = ff_add(rr, ff_from(-P.rc2));
                    if (over.hi > 0.f || (over.hi == 0.f && over.lo > 0.f)) return;
                    close_acc = ff_add(close_acc, lj_close_ff(ppc[s * MAXT + ttype[j]], rr, rcf, P.trunc));
                };
                for (int j = 0; j < cnt; ++j) {
                    // hi parts only: a far pair tolerates the ~ulp(L) this leaves
                    const float4 ah = reinterpret_cast<const float4*>(&tile[j])[0];
                    float dx = __fsub_rn(__fsub_rn(ah.x, px.hi), px.lo);
                    float dy = __fsub_rn(__fsub_rn(ah.y, py.hi), py.lo);
                    float dz = __fsub_rn(__fsub_rn(ah.z, pz.hi), pz.lo);
                    if (P.L.ortho) {
                        dx = fmaf(-rintf(dx * P.linv[0]), P.lh[0], dx);
                        dy = fmaf(-rintf(dy * P.linv[4]), P.lh[4], dy);
                        dz = fmaf(-rintf(dz * P.linv[8]), P.lh[8], dz);
                    } else {
                        float n[3];
#pragma unroll
                        for (int a = 0; a < 3; ++a)
                            n[a] = rintf(fmaf(dx, P.linv[a], fmaf(dy, P.linv[3 + a], dz * P.linv[6 + a])));
                        const float ex = fmaf(-n[0], P.lh[0], fmaf(-n[1], P.lh[3], -n[2] * P.lh[6]));
                        const float ey = fmaf(-n[0], P.lh[1], fmaf(-n[1], P.lh[4], -n[2] * P.lh[7]));
                        const float ez = fmaf(-n[0], P.lh[2], fmaf(-n[1], P.lh[5], -n[2] * P.lh[8]));
                        dx += ex;
                        dy += ey;
                        dz += ez;
                    }
                    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    const PairF32W q = rowf[ttype[j]];
                    const bool close = r2 < CLOSE_SIGMA2 * q.sig2 || fabsf(r2 - rc2f) <= band;
                    if (close) {  // rare: listed
                        if (nclose < CLOSE_MAX) mine[WT * nclose++] = (uint16_t)j;
                        else redo(j);  // a crowded trial: at once
                    }
                    // every lane evaluates the term (no divergence); kept inside rc
                    const float ir2 = __frcp_rn(r2);
                    const float ir6 = ir2 * ir2 * ir2;
                    float e = ir6 * fmaf(q.a, ir6, -q.b) - q.shift;
                    if (P.trunc == ALEA_LINEAR_FORCE_SHIFTED) e -= (sqrtf(r2) - rcf) * q.dvdrc;
                    lj_acc += (!close && r2 <= rc2f) ? e : 0.f;
                }
                for (int k = 0; k < nclose; ++k) redo(mine[WT * k]);
                lj_close = (double)close_acc.hi + (double)close_acc.lo;
            } else {
                // the displacement formed and brought to its image in
                // double-float, rounded to FP32 once; FP32 pair terms
                const ff px = ff_from(sx[s]), py = ff_from(sy[s]), pz = ff_from(sz[s]);
                const float rc2f = (float)P.rc2, rcf = (float)P.rc, alphaf = (float)P.alpha,
                            rce2f = (float)(P.rc_ewald * P.rc_ewald);
                const PairF32W* rowf = ppf + s * MAXT;
                ff close_acc{0.f, 0.f};
                const ff alpha_ff = ff_from(P.alpha);
                // the term of a near pair from the double-float displacement
                // and charge, in double-float (FP64 beyond the erfc series)
                auto near_term = [&](int j) -> double {
                    const float4* t4 = reinterpret_cast<const float4*>(&tile[j]);
                    const float4 ah = t4[0], al = t4[1];
                    ff dx = ff_add(ff{ah.x, al.x}, ff{-px.hi, -px.lo});
                    ff dy = ff_add(ff{ah.y, al.y}, ff{-py.hi, -py.lo});
                    ff dz = ff_add(ff{ah.z, al.z}, ff{-pz.hi, -pz.lo});
                    ff_min_image(P.lh, P.ll, P.linv, P.L.ortho, dx, dy, dz);
                    double v;
                    if (near_coulomb_ff(dx, dy, dz, ff{ah.w, al.w}, alpha_ff, v)) return v;
                    const double ddx = (double)dx.hi + dx.lo, ddy = (double)dy.hi + dy.lo,
                                 ddz = (double)dz.hi + dz.lo;
                    const double rd = fmax(sqrt(ddx * ddx + ddy * ddy + ddz * ddz), 1e-6);
                    return ((double)ah.w + (double)al.w) * (erfc(P.alpha * rd) / rd);
                };
                uint16_t* nl = nearj + threadIdx.x;  // stride WT: bank-conflict free
                int nnear = 0;
                for (int j = 0; j < cnt; ++j) {
                    const float4* t4 = reinterpret_cast<const float4*>(&tile[j]);
                    const float4 ah = t4[0], al = t4[1];
                    ff dx = ff_add(ff{ah.x, al.x}, ff{-px.hi, -px.lo});
                    ff dy = ff_add(ff{ah.y, al.y}, ff{-py.hi, -py.lo});
                    ff dz = ff_add(ff{ah.z, al.z}, ff{-pz.hi, -pz.lo});
                    ff_min_image(P.lh, P.ll, P.linv, P.L.ortho, dx, dy, dz);
                    const float r2 = fmaf(dx.hi, dx.hi, fmaf(dy.hi, dy.hi, dz.hi * dz.hi));
                    const uint32_t ty = ttype[j];
                    const PairF32W q = rowf[ty];
                    if (r2 < q.sig2) {
                        // close pair (r < sigma): its repulsive term reaches 1e4 K,
                        // in double-float so its rounding stays below 1e-6 K
                        const ff rr = ff_add(ff_add(ff_mul(dx, dx), ff_mul(dy, dy)), ff_mul(dz, dz));
                        close_acc = ff_add(close_acc, lj_close_ff(ppc[s * MAXT + ty], rr, rcf, P.trunc));
                    } else if (r2 <= rc2f) {
                        const float ir2 = 1.0f / r2;
                        const float ir6 = ir2 * ir2 * ir2;
                        float e = ir6 * fmaf(q.a, ir6, -q.b) - q.shift;
                        if (P.trunc == ALEA_LINEAR_FORCE_SHIFTED) e -= (sqrtf(r2) - rcf) * q.dvdrc;
                        lj_acc += e;
                    }
                    if ((Q && P.charged) && r2 <= rce2f) {
                        if (r2 < NEAR_COULOMB_R2) {  // a near pair: listed
                            if (nnear < NEAR_MAX) nl[WT * nnear++] = (uint16_t)j;
                            else es_near += near_term(j);  // a crowded trial: at once
                        } else {
                            const float rf = sqrtf(r2);
                            es_acc += ah.w * (erfcf(alphaf * rf) / rf);
                        }
                    }
                }
                for (int k = 0; k < nnear; ++k) es_near += near_term(nl[WT * k]);
                lj_close = (double)close_acc.hi + (double)close_acc.lo;
            }
            lj_site[s] += (double)lj_acc + lj_close;
            es_site[s] += (double)es_acc + es_near;
        }
    }
    double du = 0.0;
#pragma unroll
    for (int s = 0; s < MAXS; ++s)
        if (s < ns) du += lj_site[s];

    if ((Q && P.charged)) {
        double e = 0.0;
#pragma unroll
        for (int s = 0; s < MAXS; ++s)
            if (s < ns) e += (P.site[s].q * es_site[s]) * kCoulomb;
        du += e;
        // ---- reciprocal delta against the framework S(k)
        double acc = 0.0;
        if constexpr (sizeof(Real) == 4) {
            // FP32 form: the trial's phases, the framework's S(k) and the
            // weights as double-float (hi + lo FP32 pairs, ~48 bits) on the FP32
            // pipe: each row's start phase and the step e^{i theta_2} from an
            // FP64 sincos, one double-float complex rotation per term and site
            // along the row; each row's terms summed in double-float, the rows
            // in FP64. (Plain FP32 phases leave ~1e-7 relative per term, which
            // the strongly charged frameworks' |S(k)| turns into ~1e-2 K.)
            double th[MAXS][3];
            ff qf[MAXS], c1f[MAXS], s1f[MAXS], c2f[MAXS], s2f[MAXS];
            ff rc[MAXS], rs[MAXS];  // the previous row's start phase
            const float4* __restrict__ swk = D.swk32;
#pragma unroll
            for (int s = 0; s < MAXS; ++s) {
                if (s >= ns) break;
                for (int i = 0; i < 3; ++i)
                    th[s][i] = P.b[3 * i] * sx[s] + P.b[3 * i + 1] * sy[s] + P.b[3 * i + 2] * sz[s];
                double sn, cs;
                sincos(th[s][2], &sn, &cs);
                s2f[s] = ff_from(sn);
                c2f[s] = ff_from(cs);
                sincos(th[s][1], &sn, &cs);
                s1f[s] = ff_from(sn);
                c1f[s] = ff_from(cs);
                qf[s] = ff_from(P.site[s].q);
            }
            // (c, s) *= e^{i sign theta}, theta given by its (cos, sin)
            auto rotate = [](ff& c, ff& s, const ff& ct, const ff& st, bool neg) {
                const ff a = ff_mul(s, st), b = ff_mul(c, st);
                const ff cc = ff_mul(c, ct), sc = ff_mul(s, ct);
                c = neg ? ff_add(cc, a) : ff_add(cc, ff{-a.hi, -a.lo});
                s = neg ? ff_add(sc, ff{-b.hi, -b.lo}) : ff_add(sc, b);
            };
            int prev_n0 = -(1 << 30), prev_n1 = 0, prev_m = 0;
            for (int r = 0; r < P.n_rows; ++r) {
                const KRow kr = rows[r];
                ff pc[MAXS], ps[MAXS];
                // the row's start phase n0 th0 + n1 th1 - m th2: from an FP64 sincos
                // at the first row of each n0, else the previous row's advanced by
                // e^{i th1} and (m - m_prev) steps of e^{-i th2}, in double-float
                const bool chain = kr.n0 == prev_n0 && kr.n1 == prev_n1 + 1;
#pragma unroll
                for (int s = 0; s < MAXS; ++s) {
                    if (s >= ns) break;
                    if (!chain) {
                        double sn, cs;
                        sincos(kr.n0 * th[s][0] + kr.n1 * th[s][1] - kr.m * th[s][2], &sn, &cs);
                        rs[s] = ff_from(sn);
                        rc[s] = ff_from(cs);
                    } else {
                        rotate(rc[s], rs[s], c1f[s], s1f[s], false);
                        for (int d = prev_m; d < kr.m; ++d) rotate(rc[s], rs[s], c2f[s], s2f[s], true);
                        for (int d = kr.m; d < prev_m; ++d) rotate(rc[s], rs[s], c2f[s], s2f[s], false);
                    }
                    pc[s] = rc[s];
                    ps[s] = rs[s];
                }
                prev_n0 = kr.n0;
                prev_n1 = kr.n1;
                prev_m = kr.m;
                int t = kr.t0;
                ff racc{0.f, 0.f};
                for (int n2 = -kr.m; n2 <= kr.m; ++n2) {
                    if (!(kr.n0 == 0 && kr.n1 == 0 && n2 == 0)) {
                        ff re{0.f, 0.f}, im{0.f, 0.f};
#pragma unroll
                        for (int s = 0; s < MAXS; ++s) {
                            if (s >= ns) break;
                            re = ff_add(re, ff_mul(qf[s], pc[s]));
                            im = ff_add(im, ff_mul(qf[s], ps[s]));
                        }
                        const float4 o1 = __ldg(&swk[2 * t]);      // {w, Re S} hi, lo
                        const float4 o2 = __ldg(&swk[2 * t + 1]);  // {Im S} hi, lo
                        const ff dot = ff_add(ff_mul(ff{o1.z, o1.w}, re), ff_mul(ff{o2.x, o2.y}, im));
                        const ff d2 = ff_add(ff_mul(re, re), ff_mul(im, im));
                        racc = ff_add(racc, ff_mul(ff{o1.x, o1.y}, ff_add(ff_add(dot, dot), d2)));
                        ++t;
                    }
#pragma unroll
                    for (int s = 0; s < MAXS; ++s) {
                        if (s >= ns) break;
                        const ff a = ff_mul(ps[s], s2f[s]);
                        const ff c = ff_add(ff_mul(pc[s], c2f[s]), ff{-a.hi, -a.lo});
                        ps[s] = ff_add(ff_mul(ps[s], c2f[s]), ff_mul(pc[s], s2f[s]));
                        pc[s] = c;
                    }
                }
                acc += (double)racc.hi + (double)racc.lo;
            }
        } else {
        double th[MAXS][3], cs2[MAXS], sn2[MAXS];
#pragma unroll
        for (int s = 0; s < MAXS; ++s) {
            if (s >= ns) break;
            for (int i = 0; i < 3; ++i)
                th[s][i] = P.b[3 * i] * sx[s] + P.b[3 * i + 1] * sy[s] + P.b[3 * i + 2] * sz[s];
            sincos(th[s][2], &sn2[s], &cs2[s]);
        }
        for (int r = 0; r < P.n_rows; ++r) {
            const KRow kr = rows[r];
            double pc[MAXS], ps[MAXS];
#pragma unroll
            for (int s = 0; s < MAXS; ++s) {
                if (s >= ns) break;
                const double ph = kr.n0 * th[s][0] + kr.n1 * th[s][1] - kr.m * th[s][2];
                sincos(ph, &ps[s], &pc[s]);
            }
            int t = kr.t0;
            for (int n2 = -kr.m; n2 <= kr.m; ++n2) {
                if (!(kr.n0 == 0 && kr.n1 == 0 && n2 == 0)) {
                    double re = 0.0, im = 0.0;
#pragma unroll
                    for (int s = 0; s < MAXS; ++s) {
                        if (s >= ns) break;
                        re += P.site[s].q * pc[s];
                        im += P.site[s].q * ps[s];
                    }
                    const double o_re = __ldg(&sre[t]), o_im = __ldg(&sim[t]);
                    const double n_re = o_re + re, n_im = o_im + im;
                    acc += __ldg(&w[t]) * ((n_re * n_re + n_im * n_im) - (o_re * o_re + o_im * o_im));
                    ++t;
                }
#pragma unroll
                for (int s = 0; s < MAXS; ++s) {
                    if (s >= ns) break;
                    const double c = pc[s] * cs2[s] - ps[s] * sn2[s];
                    ps[s] = ps[s] * cs2[s] + pc[s] * sn2[s];
                    pc[s] = c;
                }
            }
        }
        }  // FP64 form
        double q2 = 0.0, ex = 0.0;
        for (int i = 0; i < ns; ++i) {
            q2 += P.site[i].q * P.site[i].q;
            for (int j = i + 1; j < ns; ++j) {
                double dx, dy, dz;
                min_image(P.L, sx[j] - sx[i], sy[j] - sy[i], sz[j] - sz[i], dx, dy, dz);
                const double r = sqrt(dx * dx + dy * dy + dz * dz);
                ex += P.site[i].q * P.site[j].q *
                      (r < 1e-8 ? 2.0 * P.alpha / sqrt(kPi) : erf(P.alpha * r) / r);
            }
        }
        du += (P.rec_pref * acc + P.self_pref * q2) + (-kCoulomb * ex);
    }

    if (active && per_trial) per_trial[local] = du;
    if (active && frac_out)
        for (int a = 0; a < 3; ++a) frac_out[3 * local + a] = u[a];
    if (active && samples_out) {
        float* o = samples_out + ALEA_SAMPLE_ROW * local;
        for (int a = 0; a < 3; ++a) o[a] = (float)u[a];
        o[3] = (float)((-du) / P.temperature);
        o[4] = tab.cells > 0 ? (float)__ldg(&tab.logp[cell]) : 0.f;
    }

    // ---- log-sum-exp of -du/T (minus log p(s) for the learned proposal)
    // over the block (fixed order)
    double lw = active ? (-du) / P.temperature : -INFINITY;
    if (active && tab.cells > 0) lw -= __ldg(&tab.logp[cell]);
    red[threadIdx.x] = lw;
    __syncthreads();
    for (int s = WT / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    const double mx = red[0];
    __syncthreads();
    const bool finite = mx > -INFINITY;
    red[threadIdx.x] = (active && finite) ? exp(lw - mx) : 0.0;
    __syncthreads();
    for (int s = WT / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    const double s1 = red[0];
    __syncthreads();
    red[threadIdx.x] = (active && finite) ? exp(2.0 * (lw - mx)) : 0.0;
    __syncthreads();
    for (int s = WT / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[3 * block] = mx;
        partial[3 * block + 1] = s1;
        partial[3 * block + 2] = red[0];
    }
    __syncthreads();  // shared memory is reused by the next block of trials
}


// The per-block (max, s1, s2) combined in block order into {max, S1, S2},
// every operation explicitly rounded so that every kernel calling it gives
// the same bits.
__device__ __forceinline__ void combine_partials(const double* __restrict__ partial,
                                                 uint64_t nblocks, double* __restrict__ out) {
    double mx = -INFINITY;
    for (uint64_t b = 0; b < nblocks; ++b) mx = fmax(mx, partial[3 * b]);
    double s1 = 0.0, s2 = 0.0;
    if (mx > -INFINITY)
        for (uint64_t b = 0; b < nblocks; ++b) {
            const double m = partial[3 * b];
            if (!(m > -INFINITY)) continue;
            const double f = exp(__dsub_rn(m, mx));
            s1 = __dadd_rn(s1, __dmul_rn(partial[3 * b + 1], f));
            s2 = __dadd_rn(s2, __dmul_rn(partial[3 * b + 2], __dmul_rn(f, f)));
        }
    out[0] = mx;
    out[1] = s1;
    out[2] = s2;
}


// ---- the Widom kernel: one or many contexts in one launch
// One CTA per work item (context, block of WT trials), found by binary search
// over the contexts' first items (the hardware schedules the uneven blocks);
// each CTA copies the context's parameters into shared memory and runs the
// block. A single context is a batch of one, so a framework's result in a
// batch is its own alea_widom_run's, bit for bit (the same instructions).
struct WidomItem {
    WidomParams P;
    WidomPtrs D;
    uint64_t seed, stream, first, n;
    double* partial;  // 3 per block of this context
    double* result;   // combined {max, S1, S2}
    uint64_t block0;  // first work item
    uint64_t nblocks;
    // optional per-trial outputs (single contexts) and the learned proposal
    double* per_trial;
    double* frac_out;
    float* samples_out;
    ProposalTable tab;
};

// FP32: 3 CTAs per SM when charged (at most 170 registers a thread), 4 for LJ only
template <typename Real, bool Q>
__global__ void __launch_bounds__(WT, sizeof(Real) == 4 ? (Q ? 3 : 4) : 1)
widom_batch_kernel(const WidomItem* __restrict__ items, int n_items, int draw_order) {
    __shared__ WidomParams Ps;
    __shared__ int item;
    static_assert(sizeof(WidomParams) % 4 == 0, "parameters copied as words");
    const uint64_t work = blockIdx.x;
    if (threadIdx.x == 0) {
        int lo = 0, hi = n_items - 1;  // last context with block0 <= work
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (items[mid].block0 <= work) lo = mid; else hi = mid - 1;
        }
        item = lo;
    }
    __syncthreads();
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&items[item].P);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&Ps);
    for (int i = threadIdx.x; i < (int)(sizeof(WidomParams) / 4); i += WT) dst[i] = src[i];
    __syncthreads();
    const WidomItem& it = items[item];
    widom_block<Real, Q>(Ps, it.D, work - it.block0, it.seed, it.stream, it.first, it.n, draw_order,
                      it.per_trial, it.partial, it.tab, it.frac_out, it.samples_out);
}

// One thread per framework: its blocks' partials combined in block order.
__global__ void widom_batch_combine_kernel(const WidomItem* __restrict__ items, int n_items) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_items) return;
    combine_partials(items[i].partial, items[i].nblocks, items[i].result);
}

// The instantiation for a launch: FP32 or FP64, charged or LJ-only contexts.
using WidomKernel = void (*)(const WidomItem*, int, int);
WidomKernel widom_kernel_for(int precision, bool charged) {
    if (precision == ALEA_FP32)
        return charged ? widom_batch_kernel<float, true> : widom_batch_kernel<float, false>;
    return charged ? widom_batch_kernel<double, true> : widom_batch_kernel<double, false>;
}

}  // namespace

struct WidomImpl {
    WidomParams P{};
    int precision = ALEA_FP64;
    DevBuf<double4> atoms;
    DevBuf<float4> atoms32;
    DevBuf<uint32_t> types;
    DevBuf<PairParams> table;
    DevBuf<KRow> rows;
    EwaldStateImpl* ews = nullptr;
    DevBuf<float4> swk32;            // FP32 form: per term {w, Re S} and {Im S} as hi, lo
    DevBuf<double> partial, result, per_trial, per_trial_frac;
    WidomItem item_h{};
    DevBuf<WidomItem> item;          // the context as a batch of one
    // opt-in (no counterpart in the reference engine): every trial's deltaU
    // gains U_tail(framework + molecule) - U_tail(framework), a constant of
    // the context (tailEnergyCorrection, lennard_jones.cc:246-257)
    bool tail = false;
    double tail_du = 0.0;
    ~WidomImpl() {
        if (ews) ewald_state_destroy(ews);
    }
};

WidomImpl* widom_create(const alea_lennard_jones& lj, const alea_ewald* ew,
                        const alea_particles& fw, const alea_lattice& lat,
                        const alea_molecule_species& guest, double temperature, int precision) {
    require(temperature > 0.0, ALEA_ERR_INVALID_ARGUMENT,
            "MonteCarloEngine: temperatureKelvin must be positive");
    require(guest.n_sites >= 1 && guest.n_sites <= MAXS, ALEA_ERR_INVALID_ARGUMENT,
            "Widom: the guest species needs 1..8 sites");
    require(lj.n_species >= 1 && lj.n_species <= MAXT, ALEA_ERR_INVALID_ARGUMENT,
            "Widom: 1..64 LJ species supported");
    require(lj.cutoff > 0.0, ALEA_ERR_INVALID_ARGUMENT, "LennardJones: cutoff must be positive");
    require(precision == ALEA_FP64 || precision == ALEA_FP32, ALEA_ERR_INVALID_ARGUMENT,
            "Widom: precision must be ALEA_FP64 or ALEA_FP32");
    require(fw.n == 0 || (fw.x && fw.y && fw.z), ALEA_ERR_INVALID_ARGUMENT,
            "Widom: framework coordinates missing");
    auto* w = new WidomImpl();
    try {
        WidomParams& P = w->P;
        P.L = make_lattice(lat.m);
        for (int i = 0; i < 9; ++i) {
            const ff m = ff_from(P.L.m[i]);
            P.lh[i] = m.hi;
            P.ll[i] = m.lo;
            P.linv[i] = (float)P.L.inv[i];
        }
        validate_cutoff(P.L, lj.cutoff, "MonteCarloEngine (LJ)");
        P.n_atoms = fw.n;
        P.n_sites = (int)guest.n_sites;
        for (uint32_t s = 0; s < guest.n_sites; ++s) {
            require(guest.lj_species[s] < lj.n_species, ALEA_ERR_OUT_OF_RANGE,
                    "Widom: guest site LJ species out of range");
            P.site[s] = GuestSite{guest.x[s], guest.y[s], guest.z[s],
                                  guest.charge ? guest.charge[s] : 0.0, guest.lj_species[s]};
        }
        {  // the tail-correction change of one insertion into the framework
            std::vector<double> cnt(lj.n_species, 0.0), mol(lj.n_species, 0.0);
            for (uint64_t i = 0; i < fw.n; ++i) {
                const uint32_t t = fw.species ? fw.species[i] : 0u;
                require(t < lj.n_species, ALEA_ERR_OUT_OF_RANGE, "Widom: framework species out of range");
                cnt[t] += 1.0;
            }
            for (uint32_t s = 0; s < guest.n_sites; ++s) mol[guest.lj_species[s]] += 1.0;
            std::vector<PairParams> tab((size_t)lj.n_species * lj.n_species);
            mixed_table(lj, tab.data());
            const double rc3 = lj.cutoff * lj.cutoff * lj.cutoff;
            auto u_tail = [&](const std::vector<double>& n) {
                double total = 0.0;
                for (uint32_t a = 0; a < lj.n_species; ++a) {
                    if (n[a] == 0.0) continue;
                    for (uint32_t b = 0; b < lj.n_species; ++b) {
                        if (n[b] == 0.0) continue;
                        const PairParams& pp = tab[(size_t)a * lj.n_species + b];
                        const double sr3 = pp.sigma * pp.sigma * pp.sigma;
                        const double sr9 = sr3 * sr3 * sr3 / (rc3 * rc3 * rc3);
                        total += n[a] * n[b] *
                                 (pp.eps * sr3 * ((4.0 / 9.0) * sr9 - (4.0 / 3.0) * (sr3 / rc3)));
                    }
                }
                return (2.0 * kPi / std::fabs(P.L.volume)) * total;
            };
            std::vector<double> after(cnt);
            for (uint32_t t = 0; t < lj.n_species; ++t) after[t] += mol[t];
            w->tail_du = u_tail(after) - u_tail(cnt);
        }
        P.n_species = lj.n_species;
        P.rc = lj.cutoff;
        P.rc2 = lj.cutoff * lj.cutoff;
        P.trunc = lj.truncation;
        P.temperature = temperature;
        w->precision = precision;
        if (ew) {  // engine ctor checks (monte_carlo_engine.cc:273-293), before any device work
            double qs = 0.0;
            for (uint32_t s = 0; s < guest.n_sites; ++s) qs += guest.charge ? guest.charge[s] : 0.0;
            require(std::fabs(qs) <= 1e-8, ALEA_ERR_INVALID_ARGUMENT,
                    "MonteCarloEngine: GCMC species 0 is not individually charge-neutral (total "
                    "site charge = " + std::to_string(qs) +
                        " e); every insertion/deletion/swap would drift the system away from "
                        "neutrality, which electrostatics requires");
            double qf = 0.0;
            for (uint64_t i = 0; i < fw.n; ++i) qf += fw.charge ? fw.charge[i] : 0.0;
            require(std::fabs(qf) <= 1e-8, ALEA_ERR_INVALID_ARGUMENT,
                    "MonteCarloEngine: framework is not charge-neutral (total charge = " +
                        std::to_string(qf) + " e)");
        }
        require_device();
        std::vector<double4> packed(fw.n);
        std::vector<uint32_t> types(fw.n, 0);
        for (uint64_t i = 0; i < fw.n; ++i) {
            packed[i] = make_double4(fw.x[i], fw.y[i], fw.z[i], fw.charge ? fw.charge[i] : 0.0);
            if (fw.species) {
                require(fw.species[i] < lj.n_species, ALEA_ERR_OUT_OF_RANGE,
                        "Widom: framework species out of range");
                types[i] = fw.species[i];
            }
        }
        w->atoms.alloc(std::max<size_t>(fw.n, 1));
        w->types.alloc(std::max<size_t>(fw.n, 1));
        w->atoms.upload(packed.data(), fw.n);
        if (precision == ALEA_FP32) {  // the atoms as double-float, split here once
            std::vector<float4> split(2 * fw.n);
            for (uint64_t i = 0; i < fw.n; ++i) {
                const ff x = ff_from(packed[i].x), y = ff_from(packed[i].y), z = ff_from(packed[i].z),
                         q = ff_from(packed[i].w);
                split[2 * i] = make_float4(x.hi, y.hi, z.hi, q.hi);
                split[2 * i + 1] = make_float4(x.lo, y.lo, z.lo, q.lo);
            }
            w->atoms32.alloc(std::max<size_t>(2 * fw.n, 2));
            w->atoms32.upload(split.data(), 2 * fw.n);
        }
        w->types.upload(types.data(), fw.n);
        std::vector<PairParams> table((size_t)lj.n_species * lj.n_species);
        mixed_table(lj, table.data());
        w->table.alloc(table.size());
        w->table.upload(table.data(), table.size());
        std::vector<KRow> rows;
        if (ew) {
            validate_cutoff(P.L, ew->real_space_cutoff, "MonteCarloEngine (Ewald real space)");
            w->ews = ewald_state_create(*ew, fw, lat);
            const EwaldDeviceView v = ewald_state_view(w->ews);
            P.charged = 1;
            P.alpha = ew->alpha;
            P.rc_ewald = ew->real_space_cutoff;
            P.nk = v.nk;
            for (int i = 0; i < 9; ++i) P.b[i] = v.b[i];
            P.self_pref = v.self_pref;
            P.rec_pref = v.rec_pref;
            const int K = ew->kmax;
            const int bound = K * K + 2;
            int t = 0;
            for (int n0 = -K; n0 <= K; ++n0)
                for (int n1 = -K; n1 <= K; ++n1) {
                    const int rem = bound - n0 * n0 - n1 * n1;  // n2^2 < rem
                    if (rem <= 0) continue;
                    int m = 0;
                    while ((m + 1) * (m + 1) < rem) ++m;
                    rows.push_back(KRow{n0, n1, m, t});
                    t += 2 * m + 1 - ((n0 == 0 && n1 == 0) ? 1 : 0);
                }
            require((uint64_t)t == v.nk, ALEA_ERR_RUNTIME, "Widom: k-row table mismatch");
            P.n_rows = (int)rows.size();
            if (precision == ALEA_FP32 && v.nk) {
                std::vector<double> hw(v.nk), hre(v.nk), him(v.nk);
                ALEA_CUDA(cudaMemcpy(hw.data(), v.w, v.nk * sizeof(double), cudaMemcpyDeviceToHost));
                ALEA_CUDA(cudaMemcpy(hre.data(), v.sre, v.nk * sizeof(double), cudaMemcpyDeviceToHost));
                ALEA_CUDA(cudaMemcpy(him.data(), v.sim, v.nk * sizeof(double), cudaMemcpyDeviceToHost));
                std::vector<float4> pk(2 * v.nk);
                for (uint64_t i = 0; i < v.nk; ++i) {
                    const ff a = ff_from(hw[i]), b = ff_from(hre[i]), c = ff_from(him[i]);
                    pk[2 * i] = make_float4(a.hi, a.lo, b.hi, b.lo);
                    pk[2 * i + 1] = make_float4(c.hi, c.lo, 0.f, 0.f);
                }
                w->swk32.alloc(2 * v.nk);
                w->swk32.upload(pk.data(), 2 * v.nk);
            }
        }
        w->rows.alloc(std::max<size_t>(rows.size(), 1));
        w->rows.upload(rows.data(), rows.size());
        w->result.alloc(3);
        w->item.alloc(1);
    } catch (...) {
        delete w;
        throw;
    }
    return w;
}

// K_H, log mean weight and relative standard error from the combined
// {max, S1 = sum e^(l - max), S2 = sum e^(2 (l - max))} of n trials.
static void summarise(const double* r, uint64_t n, double temperature, float ms,
                      alea_widom_result* out) {
    const double nn = (double)n;
    const double mean_scaled = r[1] / nn;  // mean(exp(l - max))
    out->n_trials = n;
    out->kernel_ms = ms;
    if (r[1] > 0.0) {
        out->log_mean_weight = r[0] + std::log(mean_scaled);
        out->henry = std::exp(out->log_mean_weight) / temperature;
        const double var = r[2] / nn - mean_scaled * mean_scaled;  // in units of exp(2 max)
        out->rel_std_error = std::sqrt(std::max(var, 0.0) / nn) / mean_scaled;
    } else {
        out->log_mean_weight = -INFINITY;
        out->henry = 0.0;
        out->rel_std_error = INFINITY;
    }
}

static void widom_launch(WidomImpl* w, uint64_t seed, uint64_t stream, uint64_t first, uint64_t n,
                         int draw_order, bool per_trial, const ProposalTable& tab,
                         double* frac_dev, float* samples_dev) {
    const uint64_t nblocks = (n + WT - 1) / WT;
    WidomItem& it = w->item_h;
    it.P = w->P;
    const double* wk = nullptr;
    const double *sre = nullptr, *sim = nullptr;
    if (w->ews) {
        const EwaldDeviceView v = ewald_state_view(w->ews);
        wk = v.w;
        sre = v.sre;
        sim = v.sim;
    }
    it.D = WidomPtrs{w->atoms.p, w->atoms32.p, w->types.p, w->table.p, w->rows.p, wk, sre, sim,
                     w->swk32.p};
    it.seed = seed;
    it.stream = stream;
    it.first = first;
    it.n = n;
    it.partial = w->partial.p;
    it.result = w->result.p;
    it.block0 = 0;
    it.nblocks = nblocks;
    it.per_trial = per_trial ? w->per_trial.p : nullptr;
    it.frac_out = frac_dev;
    it.samples_out = samples_dev;
    it.tab = tab;
    ALEA_CUDA(cudaMemcpy(w->item.p, &it, sizeof(WidomItem), cudaMemcpyHostToDevice));
    const WidomKernel kern = widom_kernel_for(w->precision, it.P.charged != 0);
    kern<<<(unsigned)nblocks, WT>>>(w->item.p, 1, draw_order);
    ALEA_CUDA(cudaGetLastError());
    widom_batch_combine_kernel<<<1, 32>>>(w->item.p, 1);
    ALEA_CUDA(cudaGetLastError());
}

void widom_samples(WidomImpl* w, uint64_t seed, uint64_t stream, uint64_t first, uint64_t n,
                   int draw_order, float* samples_dev, const ProposalTable* proposal) {
    require(draw_order == ALEA_DRAWS_RIGHT_TO_LEFT || draw_order == ALEA_DRAWS_LEFT_TO_RIGHT,
            ALEA_ERR_INVALID_ARGUMENT, "Widom: unknown draw order");
    if (n == 0) return;
    const uint64_t chunk = (uint64_t)WT << 20;  // trials per launch
    for (uint64_t a = 0; a < n; a += chunk) {
        const uint64_t m = std::min(chunk, n - a);
        const uint64_t nblocks = (m + WT - 1) / WT;
        if (w->partial.n < 3 * nblocks) w->partial.alloc(3 * nblocks);
        widom_launch(w, seed, stream, first + a, m, draw_order, false,
                     proposal ? *proposal : ProposalTable{0, nullptr, nullptr}, nullptr,
                     samples_dev + ALEA_SAMPLE_ROW * a);
    }
    ALEA_CUDA(cudaDeviceSynchronize());
}

void widom_run(WidomImpl* w, uint64_t seed, uint64_t stream, uint64_t first, uint64_t n,
               int draw_order, alea_widom_result* out, double* per_trial,
               const ProposalTable* proposal, double* per_trial_frac) {
    require(n > 0, ALEA_ERR_INVALID_ARGUMENT, "Widom: numTrials must be positive");
    require(draw_order == ALEA_DRAWS_RIGHT_TO_LEFT || draw_order == ALEA_DRAWS_LEFT_TO_RIGHT,
            ALEA_ERR_INVALID_ARGUMENT, "Widom: unknown draw order");
    const uint64_t nblocks = (n + WT - 1) / WT;
    require(nblocks < (1ull << 31), ALEA_ERR_INVALID_ARGUMENT, "Widom: too many trials per call");
    if (w->partial.n < 3 * nblocks) w->partial.alloc(3 * nblocks);
    if (per_trial && w->per_trial.n < n) w->per_trial.alloc(n);
    if (per_trial_frac && w->per_trial_frac.n < 3 * n) w->per_trial_frac.alloc(3 * n);
    const ProposalTable tab = proposal ? *proposal : ProposalTable{0, nullptr, nullptr};
    cudaEvent_t e0, e1;
    ALEA_CUDA(cudaEventCreate(&e0));
    ALEA_CUDA(cudaEventCreate(&e1));
    ALEA_CUDA(cudaEventRecord(e0));
    widom_launch(w, seed, stream, first, n, draw_order, per_trial != nullptr, tab,
                 per_trial_frac ? w->per_trial_frac.p : nullptr, nullptr);
    ALEA_CUDA(cudaEventRecord(e1));
    ALEA_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    ALEA_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    double r[3];
    ALEA_CUDA(cudaMemcpy(r, w->result.p, sizeof r, cudaMemcpyDeviceToHost));
    if (per_trial) {
        ALEA_CUDA(cudaMemcpy(per_trial, w->per_trial.p, n * sizeof(double), cudaMemcpyDeviceToHost));
    }
    if (per_trial_frac) {
        ALEA_CUDA(cudaMemcpy(per_trial_frac, w->per_trial_frac.p, 3 * n * sizeof(double),
                             cudaMemcpyDeviceToHost));
    }
    summarise(r, n, w->P.temperature, ms, out);
    if (w->tail) {  // a constant added to every trial's deltaU
        const double shift = -w->tail_du / w->P.temperature;
        out->log_mean_weight += shift;
        out->henry *= std::exp(shift);
        if (per_trial)
            for (uint64_t i = 0; i < n; ++i) per_trial[i] += w->tail_du;
    }
}

void widom_set_tail_correction(WidomImpl* w, int on) { w->tail = on != 0; }
double widom_tail_change(const WidomImpl* w) { return w->tail_du; }

void widom_destroy(WidomImpl* w) { delete w; }

// ---- batch of Widom contexts
struct WidomBatchImpl {
    std::vector<WidomImpl*> ctx;
    int precision = ALEA_FP64;
    std::vector<WidomItem> items_h;
    DevBuf<WidomItem> items;
    DevBuf<double> partial, result;
    cudaStream_t own = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t graph_total = 0;  // the work the captured graph was made for
    int graph_order = -1;
    int sms = 0;
    ~WidomBatchImpl() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (own) cudaStreamDestroy(own);
        for (auto* c : ctx) delete c;
    }
};

WidomBatchImpl* widom_batch_create(uint32_t n, const alea_lennard_jones* lj, const alea_ewald* ew,
                                   const alea_particles* fw, const alea_lattice* lat,
                                   const alea_molecule_species* guest, double temperature,
                                   int precision) {
    require(n >= 1, ALEA_ERR_INVALID_ARGUMENT, "alea_widom_batch_create: at least one framework");
    auto* b = new WidomBatchImpl();
    try {
        for (uint32_t i = 0; i < n; ++i)
            b->ctx.push_back(widom_create(lj[i], ew ? &ew[i] : nullptr, fw[i], lat[i], guest[i],
                                          temperature, precision));
        b->precision = precision;
        b->items.alloc(n);
        b->result.alloc(3 * (size_t)n);
        ALEA_CUDA(cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking));
        int dev = 0;
        ALEA_CUDA(cudaGetDevice(&dev));
        ALEA_CUDA(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev));
    } catch (...) {
        delete b;
        throw;
    }
    return b;
}

// Trials [first, first + n) of every framework (framework i on stream
// (seeds[i], streams[i])), one persistent launch and the per-framework
// combination replayed from a CUDA graph (captured again only when the total
// work or the draw order changes).
void widom_batch_run(WidomBatchImpl* b, const uint64_t* seeds, const uint64_t* streams,
                     uint64_t first, uint64_t n, int draw_order, alea_widom_result* out,
                     cudaStream_t s) {
    require(n > 0, ALEA_ERR_INVALID_ARGUMENT, "Widom: numTrials must be positive");
    require(draw_order == ALEA_DRAWS_RIGHT_TO_LEFT || draw_order == ALEA_DRAWS_LEFT_TO_RIGHT,
            ALEA_ERR_INVALID_ARGUMENT, "Widom: unknown draw order");
    const uint32_t m = (uint32_t)b->ctx.size();
    const uint64_t nb = (n + WT - 1) / WT;
    const uint64_t total = nb * m;
    if (b->partial.n < 3 * total) b->partial.alloc(3 * total);
    b->items_h.resize(m);
    for (uint32_t i = 0; i < m; ++i) {
        WidomImpl* w = b->ctx[i];
        const double* wk = nullptr;
        const double *sre = nullptr, *sim = nullptr;
        if (w->ews) {
            const EwaldDeviceView v = ewald_state_view(w->ews);
            wk = v.w;
            sre = v.sre;
            sim = v.sim;
        }
        WidomItem& it = b->items_h[i];
        it.P = w->P;
        it.D = WidomPtrs{w->atoms.p, w->atoms32.p, w->types.p, w->table.p, w->rows.p, wk, sre, sim,
                     w->swk32.p};
        it.seed = seeds[i];
        it.stream = streams[i];
        it.first = first;
        it.n = n;
        it.partial = b->partial.p + 3 * nb * i;
        it.result = b->result.p + 3 * (size_t)i;
        it.block0 = nb * i;
        it.nblocks = nb;
        it.per_trial = nullptr;
        it.frac_out = nullptr;
        it.samples_out = nullptr;
        it.tab = ProposalTable{0, nullptr, nullptr};
    }
    cudaStream_t run = s ? s : b->own;
    ALEA_CUDA(cudaMemcpyAsync(b->items.p, b->items_h.data(), m * sizeof(WidomItem),
                              cudaMemcpyHostToDevice, run));
    if (!b->exec || b->graph_total != total || b->graph_order != draw_order) {
        if (b->exec) cudaGraphExecDestroy(b->exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        b->exec = nullptr;
        b->graph = nullptr;
        bool charged = false;
        for (size_t i = 0; i < m; ++i) charged |= b->items_h[i].P.charged != 0;
        const WidomKernel kern = widom_kernel_for(b->precision, charged);
        require(total < (1ull << 31), ALEA_ERR_INVALID_ARGUMENT, "Widom batch: too many trials");
        ALEA_CUDA(cudaStreamSynchronize(run));
        ALEA_CUDA(cudaStreamBeginCapture(b->own, cudaStreamCaptureModeThreadLocal));
        kern<<<(unsigned)total, WT, 0, b->own>>>(b->items.p, (int)m, draw_order);
        widom_batch_combine_kernel<<<(m + 127) / 128, 128, 0, b->own>>>(b->items.p, (int)m);
        ALEA_CUDA(cudaStreamEndCapture(b->own, &b->graph));
        ALEA_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
        b->graph_total = total;
        b->graph_order = draw_order;
    }
    cudaEvent_t e0, e1;
    ALEA_CUDA(cudaEventCreate(&e0));
    ALEA_CUDA(cudaEventCreate(&e1));
    ALEA_CUDA(cudaEventRecord(e0, run));
    ALEA_CUDA(cudaGraphLaunch(b->exec, run));
    ALEA_CUDA(cudaEventRecord(e1, run));
    ALEA_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    ALEA_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::vector<double> r(3 * (size_t)m);
    ALEA_CUDA(cudaMemcpy(r.data(), b->result.p, r.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (uint32_t i = 0; i < m; ++i) summarise(&r[3 * (size_t)i], n, b->ctx[i]->P.temperature, ms, &out[i]);
}

void widom_batch_destroy(WidomBatchImpl* b) { delete b; }

}  // namespace alea
