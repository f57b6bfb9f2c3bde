// GCMC chains (one rigid species, or a mixture of up to four) on sm_103a, one
// 512-thread CTA per chain, every move of a launch in one persistent loop.
//
// Reference: MonteCarloEngine (engines/monte_carlo/monte_carlo_engine.cc):
//   run                      :405-439   25 % each translate / rotate / insert / delete
//   attemptTranslation       :441-484
//   attemptRotation          :486-554   (rotateAboutAxis :40-44)
//   attemptInsertion         :556-619   (randomUnitQuaternion :56-63, rotateByQuaternion :68-72)
//   attemptDeletion          :621-671   (removeMolecule :814-823, removeParticleIndices :825-848)
//   moleculeDispersionEnergy :341-374   (direct scan form; the guest-guest cell-list
//                                        candidates are a superset visited in ascending order)
//   moleculeElectrostaticRealSpaceEnergy :299-314
//   maybeResyncEwald         :380-403   (every 100 accepted moves)
// and EwaldIncrementalState's propose / commit / resync
// (forcefield/electrostatics/ewald_incremental_state.cc:95-247).
//
// Per move: thread 0 draws from the chain's Philox stream in the reference's
// order and builds the trial sites; the block sums the LJ and real-space
// Ewald energies of the old and new sites against every particle in one pass
// (FP64); the reciprocal delta runs one thread per k-term, each site's phase
// exp(i k.r) assembled from per-site tables of exp(i n theta_a) in shared
// memory (two complex products per term and site instead of an FP64 sincos),
// and the per-term delta is kept for the commit; thread 0 applies the
// acceptance rule and the bookkeeping (molecule erase, swap-with-last
// removal). Every 100 accepted moves S(k) is rebuilt as the framework's S(k)
// plus the guest sites in index order, the reference's summation order.
//
// The FP32 form (alea_gcmc_set_precision) keeps that draw order and
// bookkeeping and moves the per-pair and per-term work to the FP32 pipe:
// pair terms in FP32 from double-float displacements; Coulomb pairs within
// 6 A deferred to per-warp lists and evaluated after the pair loop, one a
// thread, in double-float (ff.cuh near_coulomb_ff); S(k) committed as
// double-float. An orientation-biased insertion or deletion (no reference
// counterpart) evaluates its k <= 8 trials in one pass in this form, one pass
// a trial in the FP64 form; both take the same draws.
//
// Layout in HBM: read-only framework (x, y, z, q as double4 + LJ type), mixed
// LJ table, k-term table (k, weight, index triple, framework S(k)); per chain:
// guest sites SoA (x, y, z, q, type), molecule -> particle index table, the
// committed S(k), a per-term delta scratch, and a ChainState record.

#include <cmath>
#include <vector>

#include "common.cuh"
#include "ff.cuh"
#include "gcmc.cuh"
#include "grid.cuh"

namespace alea {

namespace {

constexpr int GT = 512;     // threads per chain
constexpr int MAXS = 8;     // sites per molecule
constexpr int KMAXC = 64;   // largest kMax the per-site phase tables hold
// the FP32 form's (n0, n1) product table is used while it fits this budget
// of dynamic shared memory; beyond, the products are formed per term
constexpr size_t AB_TABLE_BUDGET = 160 * 1024;
constexpr int RSTRIDE = 4 * MAXS + 1;
constexpr int TU = 4;  // FP32 form: reciprocal terms per turn of a thread's loop

constexpr int MAXGS = GCMC_MAX_SPECIES;
// FP32 form: pairs closer than NEAR_R (A) take the double-float displacement;
// beyond, a pair energy (<= ~100 K of Coulomb at 6 A) moves by < 1e-4 K with
// the FP32 one. Under plain truncation, pairs within CUT_BAND (relative, on
// r^2) of the cutoff are decided in double-float too.
constexpr float NEAR_R2 = 6.0f * 6.0f;
// the near sphere under 1 % of the cell: 100 x (4/3) pi 6^3 A^3
constexpr double FIXED_FAR_VOLUME = 100.0 * 4.0 / 3.0 * 3.14159265358979 * 216.0;
constexpr float CUT_BAND = 1e-5f;
// FP32 form: Coulomb pairs closer than 6 A in double-float (ff.cuh
// near_coulomb_ff; closer, a pair's real-space term reaches 1e2-1e5 K, where
// FP32 rounding would leave up to ~1e-2 K)
constexpr float NEAR_COULOMB_R2 = 36.0f;
constexpr int NEAR_W = 128;  // FP32 form: near-Coulomb pairs a warp defers in one energy pass
constexpr int MAXROWS = 8;  // distinct LJ species among the guest sites
constexpr int MAXCB = 16;   // orientation trials of a biased insertion or deletion
// FP32 form: up to FUSE_MAX orientation trials are evaluated in one energy
// pass (all trial sites against every atom and reciprocal term at once);
// more, one pass each as in the FP64 form
constexpr int FUSE_MAX = 8;

struct GcmcConst {
    Lattice L;
    int ns;     // sites of the largest guest species (the kernel's NS)
    int n_gsp;  // guest species (1: the single-species engine)
    int sp_ns[MAXGS];
    double spx[MAXGS][MAXS], spy[MAXGS][MAXS], spz[MAXGS][MAXS], spq[MAXGS][MAXS];
    uint32_t splj[MAXGS][MAXS];
    int sprow[MAXGS][MAXS];  // the site's row of the pair tables
    int n_rows;
    uint32_t row_lj[MAXROWS];  // distinct guest LJ species, one pair-table row each
    uint32_t n_species;
    double rc, rc2;
    int trunc;
    double temperature;
    double max_trans, max_rot;
    int draw_order;
    uint64_t n_fw;
    uint32_t max_mol, max_sites;
    double volume;
    int charged;
    double alpha, rc_ew, rc_ew2;
    int kmax;
    uint64_t nk;
    double b[9];
    double self_pref, rec_pref;
    double fw_q2;
    // learned insertion proposal (prop_cells == 0: the reference's uniform
    // insertion): the template centred on its centroid, and the table size
    int prop_cells;
    double tc[MAXGS][MAXS][3];
    int f32;  // ALEA_FP32 form: FP32 pair and real-space terms, FP32 per-term S(k) deltas
    // FP32 form: far pairs on the fixed-point displacement (cells above
    // FIXED_FAR_VOLUME, where under 1 % of pairs are near, so that a warp
    // rarely takes both paths)
    int fixed_far;
    float lh[9], ll[9], linv[9];  // FP32 form: rows a_i as hi + lo; the inverse (f = d . inv)
    double excl_tmpl[MAXGS];  // FP32 form: pairExclusionSum of each rigid template
    // the engine's frameworkEnergyGrid (grid == 0: none): a site's dispersion
    // is its species' interpolated table plus the LJ with the guests
    int grid, grid_fast;
    int gn[3];
    // opt-in tail correction of insertions, deletions and swaps (no
    // counterpart in the reference engine): with T_b the particle count of LJ
    // species b, U_tail = K sum_ab f_ab T_a T_b (lennard_jones.cc:217-257,
    // K = 2 pi / V) is quadratic in the molecule counts n_s, so
    //   U(n + e_s) - U(n) = lin(s) + tail_self[s],
    //   lin(s) = tail_fw[s] + sum_s' n_s' tail_x[s][s']
    int tail;
    // orientation-biased insertion and deletion of multi-site molecules (no
    // counterpart in the reference engine; 1: its single random orientation)
    int orient;
    double tail_fw[MAXGS];         // 2K sum_ab f_ab d^s_a F_b (F: framework counts)
    double tail_x[MAXGS][MAXGS];   // 2K sum_ab f_ab d^s_a d^s'_b
    double tail_self[MAXGS];       // K sum_ab f_ab d^s_a d^s_b
};

struct GcmcPtrs {
    const double4* fw;
    const uint32_t* fw_type;
    const PairParams* table;
    const double* k;
    const double* w;
    const int* nidx;
    const double* sfw_re;
    const double* sfw_im;
    ChainState* st;
    double *gx, *gy, *gz, *gq;
    uint32_t* gt;
    uint32_t* mol;
    double *sre, *sim, *dre, *dim;
    unsigned* flags;
    const double* pcdf;   // proposal cell CDF
    const double* plogp;  // log of the cell density relative to uniform
    // FP32 form: positions as double-float, {x, y, z hi, charge} and {x, y, z lo, 0}
    const float4* fwh;
    const float4* fwl;
    float4 *ghi, *glo;
    // FP32 form: fractional positions in 32-bit fixed point (x, y, z, 0): the
    // wrapped displacement of a pair is an exact integer difference
    const uint4* fwq;
    uint4* gq4;
    // FP32 form: FP32 copies of the weights and of each chain's committed
    // S(k) (refreshed on every commit and resync), FP32 per-term deltas
    const float* w32;
    // FP32 form: each chain's committed S(k) as double-float, {re, im} hi and
    // lo per term (the term loop reads the hi pair), and the terms' (n0, n1, n2)
    // packed as (n0+K) | (n1+K) << 8 | (n2+K) << 16
    float2 *sk_hi, *sk_lo;
    const float2 *sfw_hi, *sfw_lo;  // FP32 form: the framework's S(k) as double-float
    const uint32_t* npack;
    const double* gtab[MAXROWS];  // per pair-table row: its LJ species' grid table
    uint32_t* msp;                // per chain, per molecule: its species
};

struct StepShared {
    int move, valid, accept, do_resync;
    int sp_old, sp_new;       // species of the old and the new sites
    double sq_slot[2 * MAXS];  // charge per slot (old sites, then new)
    float sq32[2 * MAXS];      // the same in FP32 (the FP32 form's phase products)
    int row_slot[2 * MAXS];    // pair-table row per slot
    uint32_t mi;
    int n_old, n_new;
    uint64_t ng;        // guest sites while the move is evaluated
    uint64_t ng_after;  // guest sites after the bookkeeping
    double op[MAXS][3];
    double np_[MAXS][3];
    uint32_t ex[MAXS];
    double e_lj[2 * MAXS], e_el[2 * MAXS];
    double rec_sum, dself, dexcl;
    double lq;  // learned proposal: log density at the inserted / deleted centroid
    // orientation bias (C.orient > 1): cb 1 for an insertion, 2 for a
    // deletion; cb_pass the energy pass being evaluated; cb_q the trial
    // orientations about the centroid cb_ref; cb_lw their log weights -U/T;
    // cb_logw log(W / k) of the trials (insertion) or of the molecule's own
    // orientation and its k - 1 alternatives (deletion)
    int cb, cb_pass, cb_more;
    double cb_ref[3];
    double cb_q[MAXCB][4];
    double cb_lw[MAXCB];
    double cb_u0, cb_logw, cb_du;
    // trial orientations 1..cb_ndraw drawn by warp 0's lanes at once, from
    // the consecutive Philox calls that begin at cb_call0 (three each)
    uint64_t cb_call0;
    int cb_ndraw;
    double cb_e[MAXCB];  // exp(lw_j - max lw), formed by warp 0's lanes
};

// FP32 form: a guest site's pair terms with one framework or guest type:
// 4 eps sigma^12, 4 eps sigma^6, the shift terms, and sigma^2 below which the
// pair stays in FP64 (its repulsive term reaches 1e4 K there).
struct PairF32 {
    float a, b, shift, dvdrc, sig2;
};


// Block sum of n double-float values per thread (n <= 4*MAXS), in a fixed
// order on the FP32 pipe (a warp tree, then the warps in order), rounded to
// double: out[i] (shared memory, read after the call).
__device__ void block_sum_ff(ff* v, int n, double* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    ff* rf = reinterpret_cast<ff*>(red);
    for (int i = 0; i < n; ++i) {
        ff x = v[i];
        for (int o = 16; o > 0; o >>= 1)
            x = ff_add(x, ff{__shfl_down_sync(0xffffffffu, x.hi, o), __shfl_down_sync(0xffffffffu, x.lo, o)});
        if (lane == 0) rf[wid * RSTRIDE + i] = x;
    }
    __syncthreads();
    if (threadIdx.x < n) {
        ff t{0.f, 0.f};
        for (int w = 0; w < GT / 32; ++w) t = ff_add(t, rf[w * RSTRIDE + threadIdx.x]);
        red[(GT / 32) * RSTRIDE + threadIdx.x] = (double)t.hi + (double)t.lo;
    }
    __syncthreads();
}

__device__ __forceinline__ double u01(ChainState& c) {
    return philox_uniform(c.seed, c.stream, c.call++);
}

// Fixed-order block sum of n values per thread (n <= 4*MAXS).
__device__ void block_sum_n(double* v, int n, double* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int i = 0; i < n; ++i) {
        double x = v[i];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[wid * RSTRIDE + i] = x;
    }
    __syncthreads();
    if (threadIdx.x < n) {
        double s = 0.0;
        for (int w = 0; w < GT / 32; ++w) s += red[w * RSTRIDE + threadIdx.x];
        red[(GT / 32) * RSTRIDE + threadIdx.x] = s;
    }
    __syncthreads();
    for (int i = 0; i < n; ++i) v[i] = red[(GT / 32) * RSTRIDE + i];
    __syncthreads();
}

__device__ __forceinline__ double erf_over_r_d(double r, double alpha) {
    if (r < 1e-8) return 2.0 * alpha / sqrt(kPi);
    return erf(alpha * r) / r;
}

// pairExclusionSum (ewald_incremental_state.cc:32-43)
__device__ double exclusion_sum(const Lattice& L, const double (*p)[3], const double* q, int n,
                                double alpha) {
    double s = 0.0;
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) {
            double dx, dy, dz;
            min_image(L, p[j][0] - p[i][0], p[j][1] - p[i][1], p[j][2] - p[i][2], dx, dy, dz);
            s += q[i] * q[j] * erf_over_r_d(sqrt(dx * dx + dy * dy + dz * dz), alpha);
        }
    return s;
}

// rotateAboutAxis (monte_carlo_engine.cc:40-44)
__device__ void rotate_about_axis(const double* v, const double* a, double th, double* o) {
    double s, c;
    sincos(th, &s, &c);
    const double cr[3] = {sub_rn(mul_rn(a[1], v[2]), mul_rn(a[2], v[1])),
                          sub_rn(mul_rn(a[2], v[0]), mul_rn(a[0], v[2])),
                          sub_rn(mul_rn(a[0], v[1]), mul_rn(a[1], v[0]))};
    const double ad = mul_rn(add_rn(add_rn(mul_rn(a[0], v[0]), mul_rn(a[1], v[1])), mul_rn(a[2], v[2])),
                             sub_rn(1.0, c));
    for (int i = 0; i < 3; ++i) o[i] = add_rn(add_rn(mul_rn(v[i], c), mul_rn(cr[i], s)), mul_rn(a[i], ad));
}

// Proposal cell of a fractional position (wrapped into [0, 1)).
__device__ __forceinline__ uint32_t proposal_cell(int cells, const double* f) {
    uint32_t idx[3];
    for (int a = 0; a < 3; ++a) {
        const double w = f[a] - floor(f[a]);
        const int i = (int)(w * cells);
        idx[a] = (uint32_t)min(max(i, 0), cells - 1);
    }
    return (idx[2] * (uint32_t)cells + idx[1]) * (uint32_t)cells + idx[0];
}

// A rotation q of a species' site (rotateByQuaternion, monte_carlo_engine.cc:
// 68-72, non-contracted) about the origin of its template frame.
__device__ __forceinline__ void rotate_site(const double* loc, const double* q, double* rot) {
    const double qv[3] = {q[1], q[2], q[3]};
    const double cr[3] = {sub_rn(mul_rn(qv[1], loc[2]), mul_rn(qv[2], loc[1])),
                          sub_rn(mul_rn(qv[2], loc[0]), mul_rn(qv[0], loc[2])),
                          sub_rn(mul_rn(qv[0], loc[1]), mul_rn(qv[1], loc[0]))};
    const double t[3] = {mul_rn(cr[0], 2.0), mul_rn(cr[1], 2.0), mul_rn(cr[2], 2.0)};
    const double c2[3] = {sub_rn(mul_rn(qv[1], t[2]), mul_rn(qv[2], t[1])),
                          sub_rn(mul_rn(qv[2], t[0]), mul_rn(qv[0], t[2])),
                          sub_rn(mul_rn(qv[0], t[1]), mul_rn(qv[1], t[0]))};
    for (int i = 0; i < 3; ++i) rot[i] = add_rn(add_rn(loc[i], mul_rn(t[i], q[0])), c2[i]);
}

// randomUnitQuaternion (monte_carlo_engine.cc:56-63) over three draws taken
// in the engine's argument order.
__device__ __forceinline__ void quaternion_from(const double* v, double* q);
__device__ __forceinline__ void draw_quaternion(const GcmcConst& C, ChainState& c, double* q,
                                                bool swap_order) {
    double v[3];
    v[0] = u01(c);
    v[1] = u01(c);
    v[2] = u01(c);
    if (swap_order) {
        const double t = v[0];
        v[0] = v[2];
        v[2] = t;
    }
    quaternion_from(v, q);
}
// The quaternion of three draws (already in the engine's argument order).
__device__ __forceinline__ void quaternion_from(const double* v, double* q) {
    const double r1 = __dsqrt_rn(sub_rn(1.0, v[0])), r2 = __dsqrt_rn(v[0]);
    const double t1 = mul_rn(2.0 * kPi, v[1]), t2 = mul_rn(2.0 * kPi, v[2]);
    double s1, c1, s2, c2;
    sincos(t1, &s1, &c1);
    sincos(t2, &s2, &c2);
    q[0] = mul_rn(r2, c2);
    q[1] = mul_rn(r1, s1);
    q[2] = mul_rn(r1, c1);
    q[3] = mul_rn(r2, s2);
}

// The new sites of species k at ref: the template (about its own origin, or
// about its centroid when `centred`) rotated by q when it has several sites.
__device__ __forceinline__ void place_new(const GcmcConst& C, int k, const double* ref,
                                          const double* q, bool centred, StepShared& S) {
    const int ns = C.sp_ns[k];
    for (int s = 0; s < ns; ++s) {
        const double loc[3] = {centred ? C.tc[k][s][0] : C.spx[k][s],
                               centred ? C.tc[k][s][1] : C.spy[k][s],
                               centred ? C.tc[k][s][2] : C.spz[k][s]};
        double rot[3] = {loc[0], loc[1], loc[2]};
        if (ns > 1) rotate_site(loc, q, rot);
        for (int i = 0; i < 3; ++i) S.np_[s][i] = add_rn(ref[i], rot[i]);
    }
    S.n_new = ns;
    S.sp_new = k;
}

// Learned-proposal insertion of species k: the centroid from the tabulated
// density (a cell from the CDF, a uniform point inside it; draws 1 and 2..4),
// a uniform orientation (draws 5..7, in order), the template centred on its
// centroid.
__device__ void plan_biased_insertion(const GcmcConst& C, const GcmcPtrs& P, ChainState& c,
                                      StepShared& S, int k) {
    const uint32_t cells = (uint32_t)C.prop_cells;
    const double uc = u01(c);
    uint32_t lo = 0, hi = cells * cells * cells - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) / 2;
        if (P.pcdf[mid] > uc) hi = mid; else lo = mid + 1;
    }
    const uint32_t idx[3] = {lo % cells, (lo / cells) % cells, lo / (cells * cells)};
    double u[3];
    for (int a = 0; a < 3; ++a) u[a] = ((double)idx[a] + u01(c)) / (double)cells;
    S.lq = P.plogp[lo];
    const double* M = C.L.m;
    double ref[3];
    for (int i = 0; i < 3; ++i)
        ref[i] = add_rn(add_rn(mul_rn(M[i], u[0]), mul_rn(M[3 + i], u[1])), mul_rn(M[6 + i], u[2]));
    double q[4] = {1.0, 0.0, 0.0, 0.0};
    if (C.sp_ns[k] > 1) draw_quaternion(C, c, q, false);
    place_new(C, k, ref, q, true, S);
    for (int i = 0; i < 3; ++i) S.cb_ref[i] = ref[i];
    for (int i = 0; i < 4; ++i) S.cb_q[0][i] = q[i];
}

// The molecule `mi`'s sites as the old ones.
__device__ __forceinline__ void take_old(const GcmcConst& C, const GcmcPtrs& P, const double* gx,
                                         const double* gy, const double* gz, const uint32_t* mol,
                                         const uint32_t* msp, uint32_t mi, StepShared& S) {
    const int k = (int)msp[mi];
    const int ns = C.sp_ns[k];
    S.mi = mi;
    S.sp_old = k;
    for (int s = 0; s < ns; ++s) {
        const uint32_t gi = mol[(size_t)mi * C.ns + s];
        S.ex[s] = gi;
        const uint32_t slot = gi - (uint32_t)C.n_fw;
        S.op[s][0] = gx[slot];
        S.op[s][1] = gy[slot];
        S.op[s][2] = gz[slot];
    }
    S.n_old = ns;
}

// The pick-th molecule of species k (index order): the engine's
// moleculeIndicesOfSpecies(k)[pick].
__device__ __forceinline__ uint32_t nth_of_species(const uint32_t* msp, uint64_t n_mol, int k,
                                                   uint64_t pick) {
    uint64_t seen = 0;
    for (uint64_t m = 0; m < n_mol; ++m)
        if ((int)msp[m] == k && seen++ == pick) return (uint32_t)m;
    return 0;
}

// Thread 0: the draws and trial geometry of one move (run, monte_carlo_engine.cc:
// 405-439: 25 % each of translate, rotate, insert, delete for one species; 20 %
// each plus identity swap for several).
__device__ void plan_move(const GcmcConst& C, const GcmcPtrs& P, ChainState& c, const double* gx,
                          const double* gy, const double* gz, const uint32_t* mol,
                          const uint32_t* msp, StepShared& S) {
    const double pick = u01(c);
    const bool mixture = C.n_gsp >= 2;
    if (!mixture)
        S.move = pick < 0.25 ? 0 : pick < 0.5 ? 1 : pick < 0.75 ? 2 : 3;
    else
        S.move = pick < 0.2 ? 0 : pick < 0.4 ? 1 : pick < 0.6 ? 2 : pick < 0.8 ? 3 : 4;
    S.valid = 1;
    S.accept = 0;
    S.do_resync = 0;
    S.n_old = S.n_new = 0;
    S.sp_old = S.sp_new = 0;
    S.ng = c.n_guest;
    S.lq = 0.0;
    for (int s = 0; s < MAXS; ++s) S.ex[s] = 0xffffffffu;
    const bool rl = C.draw_order == ALEA_DRAWS_RIGHT_TO_LEFT;
    if (S.move == 2) {  // attemptInsertion (monte_carlo_engine.cc:556-619)
        const int k = mixture ? (int)(u01(c) * (double)C.n_gsp) : 0;
        if (C.prop_cells > 0) {
            plan_biased_insertion(C, P, c, S, k);
            return;
        }
        double u[3];
        u[0] = u01(c);
        u[1] = u01(c);
        u[2] = u01(c);
        if (rl) {
            const double t = u[0];
            u[0] = u[2];
            u[2] = t;
        }
        const double* M = C.L.m;
        double ref[3];
        for (int i = 0; i < 3; ++i)
            ref[i] = add_rn(add_rn(mul_rn(M[i], u[0]), mul_rn(M[3 + i], u[1])), mul_rn(M[6 + i], u[2]));
        double q[4] = {1.0, 0.0, 0.0, 0.0};
        if (C.sp_ns[k] > 1) draw_quaternion(C, c, q, rl);
        // with orientation trials the drawn point is the molecule's centroid
        // (the deletion's reverse move uses the centroid)
        place_new(C, k, ref, q, C.orient > 1 && C.sp_ns[k] > 1, S);
        for (int i = 0; i < 3; ++i) S.cb_ref[i] = ref[i];
        for (int i = 0; i < 4; ++i) S.cb_q[0][i] = q[i];
        return;
    }
    if (c.n_mol == 0) {  // nothing to act on: no further draws
        S.valid = 0;
        return;
    }
    if (S.move == 1 && !mixture && C.sp_ns[0] < 2) {  // single species, single site: no draw
        S.valid = 0;
        return;
    }
    if (S.move == 3) {  // attemptDeletion (:621-671)
        uint32_t mi;
        if (!mixture) {
            mi = (uint32_t)(u01(c) * (double)c.n_mol);
        } else {
            const int k = (int)(u01(c) * (double)C.n_gsp);
            if (c.n_of[k] == 0) {
                S.valid = 0;
                return;
            }
            mi = nth_of_species(msp, c.n_mol, k, (uint64_t)(u01(c) * (double)c.n_of[k]));
        }
        take_old(C, P, gx, gy, gz, mol, msp, mi, S);
        if (C.prop_cells > 0) {  // the proposal's density at the molecule's centroid
            double cen[3] = {0.0, 0.0, 0.0};
            for (int s = 0; s < S.n_old; ++s)
                for (int i = 0; i < 3; ++i) cen[i] += S.op[s][i];
            for (int i = 0; i < 3; ++i) cen[i] /= (double)S.n_old;
            double f[3];
            for (int a = 0; a < 3; ++a)
                f[a] = cen[0] * C.L.inv[a] + cen[1] * C.L.inv[3 + a] + cen[2] * C.L.inv[6 + a];
            S.lq = P.plogp[proposal_cell(C.prop_cells, f)];
        }
        return;
    }
    if (S.move == 4) {  // attemptSwap (:673-792)
        const int from = (int)(u01(c) * (double)C.n_gsp);
        if (c.n_of[from] == 0) {
            S.valid = 0;
            return;
        }
        const uint32_t mi = nth_of_species(msp, c.n_mol, from, (uint64_t)(u01(c) * (double)c.n_of[from]));
        int to = (int)(u01(c) * (double)(C.n_gsp - 1));
        if (to >= from) ++to;
        take_old(C, P, gx, gy, gz, mol, msp, mi, S);
        // moleculeCentroid (:74-80)
        double cen[3] = {0.0, 0.0, 0.0};
        for (int s = 0; s < S.n_old; ++s)
            for (int i = 0; i < 3; ++i) cen[i] = add_rn(cen[i], S.op[s][i]);
        const double inv = 1.0 / (double)S.n_old;
        for (int i = 0; i < 3; ++i) cen[i] = mul_rn(cen[i], inv);
        double q[4] = {1.0, 0.0, 0.0, 0.0};
        if (C.sp_ns[to] > 1) draw_quaternion(C, c, q, rl);
        place_new(C, to, cen, q, false, S);
        return;
    }
    // translate or rotate: any molecule
    const uint32_t mi = (uint32_t)(u01(c) * (double)c.n_mol);
    take_old(C, P, gx, gy, gz, mol, msp, mi, S);
    const int ns = S.n_old;
    if (S.move == 1 && ns < 2) {  // this molecule's species is single-site
        S.valid = 0;
        return;
    }
    S.sp_new = S.sp_old;
    if (S.move == 0) {  // braced initializer: left-to-right draws (:454-456)
        double d[3];
        for (int i = 0; i < 3; ++i) d[i] = mul_rn(sub_rn(mul_rn(2.0, u01(c)), 1.0), C.max_trans);
        for (int s = 0; s < ns; ++s)
            for (int i = 0; i < 3; ++i) S.np_[s][i] = add_rn(S.op[s][i], d[i]);
    } else {  // :512-532
        double cen[3] = {0.0, 0.0, 0.0};
        for (int s = 0; s < ns; ++s)
            for (int i = 0; i < 3; ++i) cen[i] = add_rn(cen[i], S.op[s][i]);
        const double inv = 1.0 / (double)ns;
        for (int i = 0; i < 3; ++i) cen[i] = mul_rn(cen[i], inv);
        const double ct = sub_rn(mul_rn(2.0, u01(c)), 1.0);
        const double st = __dsqrt_rn(fmax(0.0, sub_rn(1.0, mul_rn(ct, ct))));
        const double phi = mul_rn(2.0 * kPi, u01(c));
        double sp, cp;
        sincos(phi, &sp, &cp);
        const double axis[3] = {mul_rn(st, cp), mul_rn(st, sp), ct};
        const double ang = mul_rn(sub_rn(mul_rn(2.0, u01(c)), 1.0), C.max_rot);
        for (int s = 0; s < ns; ++s) {
            const double v[3] = {sub_rn(S.op[s][0], cen[0]), sub_rn(S.op[s][1], cen[1]),
                                 sub_rn(S.op[s][2], cen[2])};
            double r[3];
            rotate_about_axis(v, axis, ang, r);
            for (int i = 0; i < 3; ++i) S.np_[s][i] = add_rn(cen[i], r[i]);
        }
    }
    S.n_new = ns;
}

// A position's fractional coordinates in 32-bit fixed point (f wrapped into
// [0, 1), times 2^32, rounded; 1 wraps to 0).
__host__ __device__ __forceinline__ uint4 fixed_frac(const Lattice& L, double x, double y, double z) {
    uint32_t q[3];
    for (int a = 0; a < 3; ++a) {
        double f = x * L.inv[a] + y * L.inv[3 + a] + z * L.inv[6 + a];
        f -= floor(f);
        q[a] = (uint32_t)(uint64_t)(f * 4294967296.0 + 0.5);
    }
    return make_uint4(q[0], q[1], q[2], 0u);
}

// The double-float and fixed-point copies of a guest site's position (the FP32
// form's inputs).
__device__ __forceinline__ void put_hilo(const Lattice& L, float4* ghi, float4* glo, uint4* gq4,
                                         uint32_t slot, const double* p, double q) {
    const ff x = ff_from(p[0]), y = ff_from(p[1]), z = ff_from(p[2]), qq = ff_from(q);
    ghi[slot] = make_float4(x.hi, y.hi, z.hi, qq.hi);
    glo[slot] = make_float4(x.lo, y.lo, z.lo, qq.lo);
    gq4[slot] = fixed_frac(L, p[0], p[1], p[2]);
}

// Per slot (old sites, then new): charge and pair-table row of its species' site.
__device__ __forceinline__ void slot_tables(const GcmcConst& C, StepShared& S) {
    for (int e = 0; e < 2 * MAXS; ++e) {
        S.sq_slot[e] = 0.0;
        S.row_slot[e] = 0;
    }
    for (int s = 0; s < S.n_old; ++s) {
        S.sq_slot[s] = C.spq[S.sp_old][s];
        S.row_slot[s] = C.sprow[S.sp_old][s];
    }
    for (int s = 0; s < S.n_new; ++s) {
        S.sq_slot[C.ns + s] = C.spq[S.sp_new][s];
        S.row_slot[C.ns + s] = C.sprow[S.sp_new][s];
    }
    for (int e = 0; e < 2 * MAXS; ++e) S.sq32[e] = (float)S.sq_slot[e];
}

// ---- orientation-biased insertion and deletion (C.orient = k > 1; no
// counterpart in the reference engine). The standard orientational
// configurational-bias scheme for a rigid molecule: an insertion evaluates k
// orientations about the drawn centroid, picks one with probability w_j / W
// (w = exp(-U/T), W = sum w) and is accepted with the insertion ratio in
// which exp(-dU/T) is replaced by W / k; a deletion evaluates the molecule's
// own orientation and k - 1 random ones about its centroid and uses k / W in
// place of exp(+U/T). Insertion and deletion are then each other's reverse
// with the same proposal probabilities, so detailed balance holds. Energy
// passes: insertion trial j (k passes, then the picked one again unless it
// was the last); deletion: the molecule removed, then k - 1 rotations of it
// (U_j = U_0 + dU_rotation), then the removal again. The extra draws (k - 1
// quaternions, then the pick) follow the move's own draws.

// Thread 0, after plan_move: sets up the passes (S.cb = 0: the plain move).
__device__ void cbmc_begin(const GcmcConst& C, ChainState& c, StepShared& S) {
    S.cb = 0;
    S.cb_more = 0;
    S.cb_pass = 0;
    S.cb_ndraw = 0;
    if (C.orient <= 1 || !S.valid) return;
    if (S.move == 2 && C.sp_ns[S.sp_new] > 1) {
        // trials 1..k-1 take the next 3 (k - 1) calls; warp 0 forms them
        S.cb_call0 = c.call;
        S.cb_ndraw = C.orient - 1;
        c.call += 3 * (uint64_t)(C.orient - 1);
        S.cb = 1;
    } else if (S.move == 3 && C.sp_ns[S.sp_old] > 1) {
        for (int i = 0; i < 3; ++i) S.cb_ref[i] = 0.0;
        for (int s = 0; s < S.n_old; ++s)
            for (int i = 0; i < 3; ++i) S.cb_ref[i] += S.op[s][i];
        for (int i = 0; i < 3; ++i) S.cb_ref[i] /= (double)S.n_old;
        // one pass for every trial (FP32 form): the rotations drawn now, in the
        // order the pass-by-pass scheme draws them between its passes
        if (C.f32 && C.orient <= FUSE_MAX) {
            S.cb_call0 = c.call;
            S.cb_ndraw = C.orient - 1;
            c.call += 3 * (uint64_t)(C.orient - 1);
        }
        S.cb = 2;
    }
}

// log(sum_j exp(lw_j) / k) over the k trials
__device__ double cbmc_log_mean(const double* lw, int k) {
    double m = lw[0];
    for (int j = 1; j < k; ++j) m = fmax(m, lw[j]);
    double s = 0.0;
    for (int j = 0; j < k; ++j) s += exp(lw[j] - m);
    return m + log(s / (double)k);
}

// Thread 0, an insertion's k trial weights known: log(W / k), one draw picks
// trial j with probability w_j / W; its energy becomes the move's.
__device__ int cbmc_pick(ChainState& c, StepShared& S, int k, double T) {
    S.cb_logw = cbmc_log_mean(S.cb_lw, k);
    double m = S.cb_lw[0];
    for (int j = 1; j < k; ++j) m = fmax(m, S.cb_lw[j]);
    double tot = 0.0;
    for (int j = 0; j < k; ++j) tot += exp(S.cb_lw[j] - m);
    const double u = u01(c) * tot;
    int pick = k - 1;
    double cum = 0.0;
    for (int j = 0; j < k; ++j) {
        cum += exp(S.cb_lw[j] - m);
        if (u < cum) {
            pick = j;
            break;
        }
    }
    S.cb_du = -S.cb_lw[pick] * T;
    return pick;
}

// Thread 0, after an energy pass of an orientation-biased move: records the
// pass's energy and sets up the next pass (S.cb_more = 1) or ends (0).
__device__ void cbmc_after_pass(const GcmcConst& C, ChainState& c, StepShared& S, int NS) {
    S.cb_more = 0;
    if (!S.cb) return;
    const int k = C.orient;
    double u_old = 0.0, u_new = 0.0, e_old = 0.0, e_new = 0.0;
    for (int s = 0; s < S.n_old; ++s) {
        u_old += S.e_lj[s];
        e_old += S.e_el[s];
    }
    for (int s = 0; s < S.n_new; ++s) {
        u_new += S.e_lj[NS + s];
        e_new += S.e_el[NS + s];
    }
    const double rec = C.charged ? (S.rec_sum + S.dself) + S.dexcl : 0.0;
    const double T = C.temperature;
    const int p = S.cb_pass;
    if (S.cb == 1) {  // insertion
        if (p < k) S.cb_lw[p] = -(u_new + e_new + rec) / T;
        if (p + 1 < k) {
            place_new(C, S.sp_new, S.cb_ref, S.cb_q[p + 1], true, S);
            S.cb_pass = p + 1;
            S.cb_more = 1;
            return;
        }
        if (p == k - 1) {  // pick a trial with probability w_j / W
            const int pick = cbmc_pick(c, S, k, T);
            if (pick != k - 1) {  // evaluate the picked trial again (its sites and S(k) delta)
                place_new(C, S.sp_new, S.cb_ref, S.cb_q[pick], true, S);
                S.cb_pass = k;
                S.cb_more = 1;
            }
        }
        return;
    }
    // deletion
    if (p == 0) {
        S.cb_u0 = (u_old + e_old) - rec;  // the molecule's energy: dU of removal is -U_0
        S.cb_lw[0] = -S.cb_u0 / T;
    } else if (p < k) {
        S.cb_lw[p] = -(S.cb_u0 + ((u_new - u_old) + (e_new - e_old) + rec)) / T;
    }
    if (p + 1 < k) {  // the molecule in another orientation about its centroid
        double q[4];
        draw_quaternion(C, c, q, false);
        S.sp_new = S.sp_old;
        place_new(C, S.sp_old, S.cb_ref, q, true, S);
        slot_tables(C, S);
        S.cb_pass = p + 1;
        S.cb_more = 1;
        return;
    }
    if (p == k - 1) {  // the removal again, for its S(k) delta
        S.cb_logw = cbmc_log_mean(S.cb_lw, k);
        S.cb_du = -S.cb_u0;
        S.n_new = 0;
        slot_tables(C, S);
        S.cb_pass = k;
        S.cb_more = 1;
    }
}

// The grid's value at site slot e (old sites first, then new): its LJ
// species' table interpolated at the site (frameworkEnergyGrid_->interpolate,
// monte_carlo_engine.cc:353-356).
template <int NS>
__device__ __forceinline__ double site_grid_energy(const GcmcConst& C, const GcmcPtrs& P,
                                                   const StepShared& S, int e) {
    const int s = e < NS ? e : e - NS;
    const double* p = e < NS ? S.op[s] : S.np_[s];
    const double* tab = P.gtab[S.row_slot[e]];
    return C.grid_fast ? grid_interp_fast(C.L, C.gn[0], C.gn[1], C.gn[2], tab, p[0], p[1], p[2])
                       : grid_interp_ref(C.L, C.gn[0], C.gn[1], C.gn[2], tab, p[0], p[1], p[2]);
}

// Per-site phase tables in dynamic shared memory. FP64 form: e^{i n theta_a}
// per slot (old sites, then new), axis and n. FP32 form: the same in FP32,
// then (when it fits AB_TABLE_BUDGET) q e^{i (n0 theta_0 + n1 theta_1)} per
// slot and (n0, n1).
template <int NS>
__host__ __device__ size_t f32_ab_bytes(int kmax) {
    const size_t tw = 2 * (size_t)kmax + 1;
    return 2 * NS * tw * tw * sizeof(float2);
}
template <int NS>
__host__ __device__ size_t phase_bytes(int kmax, bool f32) {
    const size_t tw = 2 * (size_t)kmax + 1;
    if (!f32) return 2 * NS * 3 * tw * sizeof(double2);
    const size_t ab = f32_ab_bytes<NS>(kmax);
    return 2 * NS * 3 * tw * sizeof(float2) + (ab <= AB_TABLE_BUDGET ? ab : 0);
}

// FP32 form: slot e's site as double-float (hi, lo) and fixed-point copies.
template <int NS, bool FX>
__device__ __forceinline__ void prep_site_f32(const GcmcConst& C, const StepShared& S, int e,
                                              float4* sph, float4* spl, uint4* sfq) {
    const double* p = e < NS ? S.op[e] : S.np_[e - NS];
    const ff x = ff_from(p[0]), y = ff_from(p[1]), z = ff_from(p[2]);
    sph[e] = make_float4(x.hi, y.hi, z.hi, 0.f);
    spl[e] = make_float4(x.lo, y.lo, z.lo, 0.f);
    if constexpr (FX) sfq[e] = fixed_frac(C.L, p[0], p[1], p[2]);
}
template <int NS, bool FX>
__device__ __forceinline__ void prep_sites_f32(const GcmcConst& C, const StepShared& S, float4* sph,
                                               float4* spl, uint4* sfq) {
    for (int e = 0; e < 2 * NS; ++e) prep_site_f32<NS, FX>(C, S, e, sph, spl, sfq);
}

// FX (FP32 form, large cells): far pairs on the fixed-point displacement.
template <int NS, bool F32, bool FX>
__global__ void __launch_bounds__(GT)
gcmc_kernel(const GcmcConst C, const GcmcPtrs P, uint64_t steps) {
    __shared__ StepShared S;
    __shared__ double red[(GT / 32 + 1) * RSTRIDE];
    __shared__ double eq[2 * NS];
    __shared__ PairParams srow[F32 ? 1 : MAXROWS][64];
    __shared__ PairF32 srow32[F32 ? MAXROWS : 1][64];
    __shared__ PairCloseFF srowff[F32 ? MAXROWS : 1][64];
    __shared__ float4 sph[F32 ? 2 * NS : 1], spl[F32 ? 2 * NS : 1];  // trial sites, hi + lo
    __shared__ uint4 sfq[F32 ? 2 * NS : 1];                          // and in fixed point
    __shared__ uint32_t nearq[F32 ? GT / 32 : 1][NEAR_W];  // deferred near-Coulomb pairs (j << 4 | slot)
    // FP32 form, orientation trials in one pass: the trial sites (FP64, hi + lo, fixed point)
    __shared__ double tpos[F32 ? FUSE_MAX * NS : 1][3];
    __shared__ float4 tph[F32 ? FUSE_MAX * NS : 1], tpl[F32 ? FUSE_MAX * NS : 1];
    __shared__ uint4 tfq[F32 ? FUSE_MAX * NS : 1];
    __shared__ uint32_t nearn[GT / 32];
    extern __shared__ __align__(16) unsigned char dyn[];

    const int chain = blockIdx.x;
    ChainState c = P.st[chain];  // thread 0's copy is the authoritative one
    const size_t so = (size_t)chain * C.max_sites;
    double* gx = P.gx + so;
    double* gy = P.gy + so;
    double* gz = P.gz + so;
    double* gq = P.gq + so;
    uint32_t* gt = P.gt + so;
    float4* ghi = P.ghi + so;
    uint4* gq4 = P.gq4 + so;
    float4* glo = P.glo + so;
    uint32_t* mol = P.mol + (size_t)chain * C.max_mol * NS;
    uint32_t* msp = P.msp + (size_t)chain * C.max_mol;
    double* sre = P.sre + (size_t)chain * C.nk;
    double* sim = P.sim + (size_t)chain * C.nk;
    double* dre = P.dre + (size_t)chain * C.nk;
    double* dim = P.dim + (size_t)chain * C.nk;
    float2* sk_hi = F32 ? P.sk_hi + (size_t)chain * C.nk : nullptr;
    float2* sk_lo = F32 ? P.sk_lo + (size_t)chain * C.nk : nullptr;
    const int K = C.kmax;
    for (int i = threadIdx.x; i < C.n_rows * (int)C.n_species; i += GT) {
        const int r = i / C.n_species, t = i % C.n_species;
        const PairParams pp = P.table[(size_t)C.row_lj[r] * C.n_species + t];
        if constexpr (!F32) {
            srow[r][t] = pp;
        } else {
            const double s2 = pp.sigma * pp.sigma, s6 = s2 * s2 * s2;
            srow32[r][t] = PairF32{(float)(4.0 * pp.eps * s6 * s6), (float)(4.0 * pp.eps * s6),
                                   (float)pp.shift, (float)pp.dvdrc, (float)s2};
            const ff fs2 = ff_from(s2), fe4 = ff_from(4.0 * pp.eps), fsh = ff_from(pp.shift);
            srowff[r][t] = PairCloseFF{fs2.hi, fs2.lo, fe4.hi, fe4.lo, fsh.hi, fsh.lo,
                                       (float)pp.dvdrc, 0.f};
        }
    }
    const int tw = 2 * C.kmax + 1;
    double2* etab = reinterpret_cast<double2*>(dyn);               // FP64 form: [2NS][3][tw]
    float2* etab32 = reinterpret_cast<float2*>(dyn);               // FP32 form: [2NS][3][tw]
    float2* ab32 = etab32 + (size_t)2 * NS * 3 * tw;                // [2NS][tw][tw]
    float2* ftab32 = reinterpret_cast<float2*>(dyn + phase_bytes<NS>(C.kmax, true));  // [trial sites][3][tw]
    const bool ab_table = F32 && f32_ab_bytes<NS>(C.kmax) <= AB_TABLE_BUDGET;
    const ff alpha_ff = ff_from(C.alpha);
    __syncthreads();

    for (uint64_t step = 0; step < steps; ++step) {
        if (threadIdx.x == 0) {
            if (c.err == 0) {
                plan_move(C, P, c, gx, gy, gz, mol, msp, S);
                slot_tables(C, S);
                cbmc_begin(C, c, S);
            } else {
                S.valid = 0;
            }
        }
        __syncthreads();
        if (S.valid) {
            // the move's parallel set-up: trial orientations 1..cb_ndraw, one a
            // lane of warp 0 (the same draws and arithmetic as one after the
            // other on thread 0), and (FP32 form) the slots' FP32 copies, one a
            // thread of warp 1
            if (threadIdx.x < S.cb_ndraw) {
                const uint64_t c0 = S.cb_call0 + 3 * (uint64_t)threadIdx.x;
                const double v[3] = {philox_uniform(c.seed, c.stream, c0),
                                     philox_uniform(c.seed, c.stream, c0 + 1),
                                     philox_uniform(c.seed, c.stream, c0 + 2)};
                quaternion_from(v, S.cb_q[threadIdx.x + 1]);
            }
            if constexpr (F32)
                if (threadIdx.x >= 32 && threadIdx.x < 32 + 2 * NS)
                    prep_site_f32<NS, FX>(C, S, (int)threadIdx.x - 32, sph, spl, sfq);
            __syncthreads();
            int n_old = S.n_old, n_new = S.n_new;  // this energy pass's site counts
            const uint64_t n_all = C.n_fw + S.ng;
            // FP32 form: term t's S(k) delta, added sites first then removed
            // (ewald_incremental_state.cc:107-116), from this move's phase tables
            auto f32_delta = [&](uint32_t pk) -> float2 {
                const int n0 = pk & 0xff, n1 = (pk >> 8) & 0xff, n2 = (pk >> 16) & 0xff;
                float re = 0.f, im = 0.f;
                // q e^{i(n0 th0 + n1 th1)} of slot e: from the table, or formed here
                auto zq = [&](int e) -> float2 {
                    if (ab_table) return ab32[(e * tw + n0) * tw + n1];
                    const float2 A = etab32[(e * 3 + 0) * tw + n0], B = etab32[(e * 3 + 1) * tw + n1];
                    const float q = S.sq32[e];
                    return make_float2(q * (A.x * B.x - A.y * B.y), q * (A.x * B.y + A.y * B.x));
                };
                if (n_new)
#pragma unroll
                    for (int s = 0; s < NS; ++s) {
                        if (s >= n_new) break;  // a smaller species' unused slots hold stale phases
                        const float2 Z = zq(NS + s);
                        const float2 Cc = etab32[((NS + s) * 3 + 2) * tw + n2];
                        re = fmaf(Z.x, Cc.x, fmaf(-Z.y, Cc.y, re));
                        im = fmaf(Z.x, Cc.y, fmaf(Z.y, Cc.x, im));
                    }
                if (n_old)
#pragma unroll
                    for (int s = 0; s < NS; ++s) {
                        if (s >= n_old) break;
                        const float2 Z = zq(s);
                        const float2 Cc = etab32[(s * 3 + 2) * tw + n2];
                        re = fmaf(-Z.x, Cc.x, fmaf(Z.y, Cc.y, re));
                        im = fmaf(-Z.x, Cc.y, fmaf(-Z.y, Cc.x, im));
                    }
                return make_float2(re, im);
            };
            // with a grid the framework's LJ comes from the tables: its atoms
            // are visited only for the real-space Ewald terms
            const uint64_t j0 = (C.grid && !C.charged) ? C.n_fw : 0;
            // FP32 form: the slots' phase tables, e^{i n theta_a} in FP32 (the
            // angle reduced to [-pi, pi] in FP64 first), then (when it fits)
            // q e^{i (n0 theta_0 + n1 theta_1)}; every thread calls it
            auto tables_f32 = [&]() {
                for (int i = threadIdx.x; i < 2 * NS * 3 * tw; i += GT) {
                    const int e = i / (3 * tw), a = (i / tw) % 3, n = i % tw - K;
                    const bool is_old = e < NS;
                    if (is_old ? (e >= n_old) : (e - NS >= n_new)) continue;
                    const int s = is_old ? e : e - NS;
                    const double* p = is_old ? S.op[s] : S.np_[s];
                    const double th = C.b[3 * a] * p[0] + C.b[3 * a + 1] * p[1] + C.b[3 * a + 2] * p[2];
                    const double x = (double)n * th;
                    const double r = x - (2.0 * kPi) * rint(x * (0.5 / kPi));
                    float sn, cs;
                    sincosf((float)r, &sn, &cs);
                    etab32[i] = make_float2(cs, sn);
                }
                __syncthreads();
                for (int i = threadIdx.x; ab_table && i < 2 * NS * tw * tw; i += GT) {
                    const int e = i / (tw * tw), n0 = (i / tw) % tw, n1 = i % tw;
                    const bool is_old = e < NS;
                    if (is_old ? (e >= n_old) : (e - NS >= n_new)) continue;
                    const float2 A = etab32[(e * 3 + 0) * tw + n0], B = etab32[(e * 3 + 1) * tw + n1];
                    const float q = S.sq32[e];
                    ab32[i] = make_float2(q * (A.x * B.x - A.y * B.y), q * (A.x * B.y + A.y * B.x));
                }
                __syncthreads();
            };
            // FP32 form, orientation-biased move with k <= FUSE_MAX trials: every
            // trial in one energy pass. Trial t's site s is trial site t ns + s:
            // insertion, the species' template about its centroid cb_ref rotated
            // by cb_q[t]; deletion, trial 0 is the molecule itself (its energy
            // U_0 from its removal) and trial t > 0 the template rotated by
            // cb_q[t] about the molecule's centroid, inserted into the chain
            // without the molecule. Per trial: LJ and real-space sums over the
            // atoms (the molecule's own sites excluded in a deletion) and the
            // reciprocal change against S(k); thread 0 then forms the Rosenbluth
            // weights as the pass-by-pass scheme does, picks (insertion), and
            // leaves the move's final sites for the acceptance and the commit.
            const bool fused = F32 && S.cb != 0 && C.orient <= FUSE_MAX;
            if (fused) {
                const int k = C.orient;
                const bool ins = S.cb == 1;
                const int sp = ins ? S.sp_new : S.sp_old;
                const int ns = C.sp_ns[sp];
                const int nt = k * ns;
                for (int i = threadIdx.x; i < nt; i += GT) {
                    const int t = i / ns, s = i % ns;
                    double pos[3];
                    if (!ins && t == 0) {
                        for (int a = 0; a < 3; ++a) pos[a] = S.op[s][a];
                    } else {
                        const double loc[3] = {C.tc[sp][s][0], C.tc[sp][s][1], C.tc[sp][s][2]};
                        double rot[3];
                        rotate_site(loc, S.cb_q[t], rot);
                        for (int a = 0; a < 3; ++a) pos[a] = add_rn(S.cb_ref[a], rot[a]);
                    }
                    for (int a = 0; a < 3; ++a) tpos[i][a] = pos[a];
                    const ff x = ff_from(pos[0]), y = ff_from(pos[1]), z = ff_from(pos[2]);
                    tph[i] = make_float4(x.hi, y.hi, z.hi, 0.f);
                    tpl[i] = make_float4(x.lo, y.lo, z.lo, 0.f);
                    if constexpr (FX) tfq[i] = fixed_frac(C.L, pos[0], pos[1], pos[2]);
                }
                __syncthreads();
                float qs32[NS];
                double qs64[NS];
                int rows[NS];
#pragma unroll
                for (int s = 0; s < NS; ++s) {
                    qs64[s] = s < ns ? C.spq[sp][s] : 0.0;
                    qs32[s] = (float)qs64[s];
                    rows[s] = s < ns ? C.sprow[sp][s] : 0;
                }
                // per trial, in double-float: LJ (close pairs and far terms), the
                // far real-space terms times the site charges (a trial's sites'
                // terms cancel in part, which one FP32 sum would not resolve);
                // the near pairs' FP64 terms
                ff lj_t[FUSE_MAX], el_t[FUSE_MAX];
                double near_t[FUSE_MAX];
#pragma unroll
                for (int t = 0; t < FUSE_MAX; ++t) {
                    lj_t[t] = el_t[t] = ff{0.f, 0.f};
                    near_t[t] = 0.0;
                }
                const float rc2f = (float)C.rc2, rcf = (float)C.rc, rce2f = (float)C.rc_ew2,
                            alphaf = (float)C.alpha;
                const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
                // atom a's displacement from trial site i, double-float
                auto disp_ff = [&](const float4& ah, const float4& al, int i, ff& dx, ff& dy, ff& dz) {
                    const float4 ph = tph[i], pl = tpl[i];
                    dx = ff_add(ff{ah.x, al.x}, ff{-ph.x, -pl.x});
                    dy = ff_add(ff{ah.y, al.y}, ff{-ph.y, -pl.y});
                    dz = ff_add(ff{ah.z, al.z}, ff{-ph.z, -pl.z});
                    ff_min_image(C.lh, C.ll, C.linv, C.L.ortho, dx, dy, dz);
                };
                // the real-space term of near pair (atom a, trial site i) times
                // the site's charge, in double-float (FP64 beyond the series)
                auto near_term = [&](uint64_t a, int i) -> double {
                    float4 ah, al;
                    if (a < C.n_fw) {
                        ah = P.fwh[a];
                        al = P.fwl[a];
                    } else {
                        ah = ghi[a - C.n_fw];
                        al = glo[a - C.n_fw];
                    }
                    ff dx, dy, dz;
                    disp_ff(ah, al, i, dx, dy, dz);
                    double v;
                    if (near_coulomb_ff(dx, dy, dz, ff{ah.w, al.w}, alpha_ff, v)) return C.spq[sp][i % ns] * v;
                    const double ddx = (double)dx.hi + dx.lo, ddy = (double)dy.hi + dy.lo,
                                 ddz = (double)dz.hi + dz.lo;
                    const double rd = fmax(sqrt(ddx * ddx + ddy * ddy + ddz * ddz), 1e-6);
                    return C.spq[sp][i % ns] * (((double)ah.w + (double)al.w) * (erfc(C.alpha * rd) / rd));
                };
                uint32_t nq = 0;
                for (uint64_t jb = j0 + (uint64_t)(threadIdx.x & ~31); jb < n_all; jb += GT) {
                    const uint64_t j = jb + (uint64_t)lane;
                    uint64_t nm = 0;  // trial sites whose Coulomb pair with atom j is near
                    bool skip = j >= n_all;
                    if (!skip && !ins)
#pragma unroll
                        for (int x = 0; x < NS; ++x) skip |= (S.ex[x] == (uint32_t)j);
                    if (!skip) {
                        float4 ah, al;
                        uint4 aq = make_uint4(0u, 0u, 0u, 0u);
                        uint32_t ta;
                        if (j < C.n_fw) {
                            ah = P.fwh[j];
                            al = P.fwl[j];
                            if constexpr (FX) aq = P.fwq[j];
                            ta = P.fw_type[j];
                        } else {
                            const uint64_t g = j - C.n_fw;
                            ah = ghi[g];
                            al = glo[g];
                            if constexpr (FX) aq = gq4[g];
                            ta = gt[g];
                        }
#pragma unroll
                        for (int t = 0; t < FUSE_MAX; ++t) {
                            if (t >= k) break;
#pragma unroll
                            for (int s = 0; s < NS; ++s) {
                                if (s >= ns) break;
                                const int i = t * ns + s;
                                float cx = 0.f, cy = 0.f, cz = 0.f, r2 = 0.f;
                                bool near = true;
                                if constexpr (FX) {
                                    const uint4 pq = tfq[i];
                                    const float fx = (float)(int32_t)(aq.x - pq.x) * 2.3283064365386963e-10f;
                                    const float fy = (float)(int32_t)(aq.y - pq.y) * 2.3283064365386963e-10f;
                                    const float fz = (float)(int32_t)(aq.z - pq.z) * 2.3283064365386963e-10f;
                                    cx = fmaf(fx, C.lh[0], fmaf(fy, C.lh[3], fz * C.lh[6]));
                                    cy = fmaf(fx, C.lh[1], fmaf(fy, C.lh[4], fz * C.lh[7]));
                                    cz = fmaf(fx, C.lh[2], fmaf(fy, C.lh[5], fz * C.lh[8]));
                                    r2 = fmaf(cx, cx, fmaf(cy, cy, cz * cz));
                                    near = r2 < NEAR_R2 ||
                                           (C.trunc == ALEA_TRUNCATED && fabsf(r2 - rc2f) <= CUT_BAND * rc2f);
                                }
                                ff dx{cx, 0.f}, dy{cy, 0.f}, dz{cz, 0.f};
                                if (near) {
                                    disp_ff(ah, al, i, dx, dy, dz);
                                    r2 = fmaf(dx.hi, dx.hi, fmaf(dy.hi, dy.hi, dz.hi * dz.hi));
                                }
                                const bool lj_in = !(C.grid && j < C.n_fw) && r2 <= rc2f;
                                const bool el_in = C.charged && r2 <= rce2f;
                                if (lj_in) {
                                    const PairF32 q = srow32[rows[s]][ta];
                                    if (r2 < q.sig2) {
                                        const ff rr = ff_add(ff_add(ff_mul(dx, dx), ff_mul(dy, dy)), ff_mul(dz, dz));
                                        lj_t[t] = ff_add(lj_t[t], lj_close_ff(srowff[rows[s]][ta], rr, rcf, C.trunc));
                                    } else {
                                        const float ir2 = 1.0f / r2;
                                        const float ir6 = ir2 * ir2 * ir2;
                                        float v = ir6 * fmaf(q.a, ir6, -q.b) - q.shift;
                                        if (C.trunc == ALEA_LINEAR_FORCE_SHIFTED) v -= (sqrtf(r2) - rcf) * q.dvdrc;
                                        lj_t[t] = ff_add_f(lj_t[t], v);
                                    }
                                }
                                if (el_in) {
                                    if (r2 < NEAR_COULOMB_R2) {
                                        nm |= 1ull << i;
                                    } else {
                                        const float r = sqrtf(r2);
                                        el_t[t] = ff_add_f(el_t[t], qs32[s] * (ah.w * (erfcf(alphaf * r) / r)));
                                    }
                                }
                            }
                        }
                    }
                    // the chunk's near pairs into the warp's list (lane order,
                    // then trial-site order), or at once when it is full
                    const uint32_t cnt = (uint32_t)__popcll(nm);
                    uint32_t pre = cnt;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t y = __shfl_up_sync(0xffffffffu, pre, o);
                        if (lane >= o) pre += y;
                    }
                    const uint32_t tot = __shfl_sync(0xffffffffu, pre, 31);
                    if (nq + tot <= NEAR_W) {
                        uint32_t at = nq + pre - cnt;
                        for (uint64_t m = nm; m; m &= m - 1)
                            nearq[wid][at++] = ((uint32_t)j << 8) | (uint32_t)(__ffsll((long long)m) - 1);
                        nq += tot;
                    } else {
                        for (uint64_t m = nm; m; m &= m - 1) {
                            const int i = __ffsll((long long)m) - 1;
                            const double v = near_term(j, i);
#pragma unroll
                            for (int t = 0; t < FUSE_MAX; ++t)
                                if (i / ns == t) near_t[t] += v;
                        }
                    }
                }
                if (lane == 0) nearn[wid] = nq;
                __syncthreads();
                for (uint32_t e = threadIdx.x;; e += GT) {
                    uint32_t w = 0, base = 0;
                    while (w < GT / 32 && base + nearn[w] <= e) base += nearn[w++];
                    if (w == GT / 32) break;
                    const uint32_t code = nearq[w][e - base];
                    const int i = (int)(code & 255u);
                    const double v = near_term(code >> 8, i);
#pragma unroll
                    for (int t = 0; t < FUSE_MAX; ++t)
                        if (i / ns == t) near_t[t] += v;
                }
                if (C.grid) {  // thread i adds trial site i's interpolated table
                    if (threadIdx.x < nt) {
                        const int i = threadIdx.x;
                        const double* tab = P.gtab[C.sprow[sp][i % ns]];
                        const double g = C.grid_fast
                            ? grid_interp_fast(C.L, C.gn[0], C.gn[1], C.gn[2], tab, tpos[i][0], tpos[i][1], tpos[i][2])
                            : grid_interp_ref(C.L, C.gn[0], C.gn[1], C.gn[2], tab, tpos[i][0], tpos[i][1], tpos[i][2]);
#pragma unroll
                        for (int t = 0; t < FUSE_MAX; ++t)
                            if (i / ns == t) lj_t[t] = ff_add(lj_t[t], ff_from(g));
                    }
                }
                ff v[2 * FUSE_MAX];
#pragma unroll
                for (int t = 0; t < FUSE_MAX; ++t) {
                    v[2 * t] = lj_t[t];
                    v[2 * t + 1] = ff_add(ff_from(near_t[t]), el_t[t]);
                }
                static_assert(2 * FUSE_MAX < RSTRIDE, "fused sums fit a reduction row");
                block_sum_ff(v, 2 * FUSE_MAX, red);
                double pair_u[FUSE_MAX];  // per trial: LJ + real-space Coulomb
                if (threadIdx.x == 0)
#pragma unroll
                    for (int t = 0; t < FUSE_MAX; ++t)
                        pair_u[t] = red[(GT / 32) * RSTRIDE + 2 * t] +
                                    red[(GT / 32) * RSTRIDE + 2 * t + 1] * kCoulomb;
                __syncthreads();
                double rec_t[FUSE_MAX];  // per trial: the reciprocal change
#pragma unroll
                for (int t = 0; t < FUSE_MAX; ++t) rec_t[t] = 0.0;
                if (C.charged) {
                    // the trial sites' FP32 phases (angles reduced in FP64)
                    for (int i = threadIdx.x; i < nt * 3 * tw; i += GT) {
                        const int e = i / (3 * tw), a = (i / tw) % 3, n = i % tw - K;
                        const double th = C.b[3 * a] * tpos[e][0] + C.b[3 * a + 1] * tpos[e][1] +
                                          C.b[3 * a + 2] * tpos[e][2];
                        const double x = (double)n * th;
                        const double r = x - (2.0 * kPi) * rint(x * (0.5 / kPi));
                        float sn, cs;
                        sincosf((float)r, &sn, &cs);
                        ftab32[i] = make_float2(cs, sn);
                    }
                    __syncthreads();
                    // per term and trial: its sites' delta d_t; insertion
                    // w (2 S.d_t + |d_t|^2); deletion x = -d_0 for trial 0 and
                    // d_t - d_0 for the rotations, w (2 S.x + |x|^2)
                    float racc[FUSE_MAX];
#pragma unroll
                    for (int t = 0; t < FUSE_MAX; ++t) racc[t] = 0.f;
                    for (uint64_t tt = threadIdx.x; tt < C.nk; tt += GT) {
                        const uint32_t pk = P.npack[tt];
                        const int n0 = pk & 0xff, n1 = (pk >> 8) & 0xff, n2 = (pk >> 16) & 0xff;
                        const float2 o = sk_hi[tt];
                        const float wv = P.w32[tt];
                        float d0r = 0.f, d0i = 0.f;
#pragma unroll
                        for (int t = 0; t < FUSE_MAX; ++t) {
                            if (t >= k) break;
                            float re = 0.f, im = 0.f;
#pragma unroll
                            for (int s = 0; s < NS; ++s) {
                                if (s >= ns) break;
                                const int e = t * ns + s;
                                const float2 A = ftab32[(e * 3 + 0) * tw + n0], B = ftab32[(e * 3 + 1) * tw + n1],
                                             Cc = ftab32[(e * 3 + 2) * tw + n2];
                                const float zr = qs32[s] * (A.x * B.x - A.y * B.y),
                                            zi = qs32[s] * (A.x * B.y + A.y * B.x);
                                re = fmaf(zr, Cc.x, fmaf(-zi, Cc.y, re));
                                im = fmaf(zr, Cc.y, fmaf(zi, Cc.x, im));
                            }
                            float xr = re, xi = im;
                            if (!ins) {
                                if (t == 0) {
                                    d0r = re;
                                    d0i = im;
                                    xr = -re;
                                    xi = -im;
                                } else {
                                    xr = re - d0r;
                                    xi = im - d0i;
                                }
                            }
                            const float dot = fmaf(o.x, xr, o.y * xi);
                            racc[t] = fmaf(wv, fmaf(2.f, dot, fmaf(xr, xr, xi * xi)), racc[t]);
                        }
                    }
                    ff rv[FUSE_MAX];
#pragma unroll
                    for (int t = 0; t < FUSE_MAX; ++t) rv[t] = ff{racc[t], 0.f};
                    block_sum_ff(rv, FUSE_MAX, red);
#pragma unroll
                    for (int t = 0; t < FUSE_MAX; ++t) rec_t[t] = C.rec_pref * red[(GT / 32) * RSTRIDE + t];
                }
                const double T = C.temperature;
                if (threadIdx.x == 0) {
                    double q2 = 0.0;
                    for (int s = 0; s < ns; ++s) q2 += C.spq[sp][s] * C.spq[sp][s];
                    // an insertion's self and exclusion terms (a removal's are their negatives)
                    const double dself = C.charged ? C.self_pref * q2 : 0.0;
                    const double dexcl = C.charged ? -kCoulomb * C.excl_tmpl[sp] : 0.0;
                    if (ins) {
                        for (int t = 0; t < k; ++t) S.cb_lw[t] = -(pair_u[t] + ((rec_t[t] + dself) + dexcl)) / T;
                    } else {
                        S.cb_u0 = pair_u[0] - ((rec_t[0] - dself) - dexcl);
                        S.cb_lw[0] = -S.cb_u0 / T;
                        for (int t = 1; t < k; ++t)
                            S.cb_lw[t] = -(S.cb_u0 + ((pair_u[t] - pair_u[0]) + rec_t[t])) / T;
                    }
                }
                // the weights exp(lw_j - max lw), one a lane of warp 0; thread 0
                // then sums them in order (cbmc_log_mean and cbmc_pick's values)
                if (threadIdx.x < 32) {
                    __syncwarp();
                    double m = S.cb_lw[0];
                    for (int t = 1; t < k; ++t) m = fmax(m, S.cb_lw[t]);
                    if (threadIdx.x < k) S.cb_e[threadIdx.x] = exp(S.cb_lw[threadIdx.x] - m);
                    __syncwarp();
                    if (threadIdx.x == 0) {
                        double tot = 0.0;
                        for (int t = 0; t < k; ++t) tot += S.cb_e[t];
                        S.cb_logw = m + log(tot / (double)k);
                        if (ins) {
                            const double u = u01(c) * tot;
                            int pick = k - 1;
                            double cum = 0.0;
                            for (int t = 0; t < k; ++t) {
                                cum += S.cb_e[t];
                                if (u < cum) {
                                    pick = t;
                                    break;
                                }
                            }
                            S.cb_du = -S.cb_lw[pick] * T;
                            // the picked trial's sites (place_new's values)
                            for (int s = 0; s < ns; ++s)
                                for (int a = 0; a < 3; ++a) S.np_[s][a] = tpos[pick * ns + s][a];
                            S.n_new = ns;
                            S.sp_new = sp;
                        } else {
                            S.cb_du = -S.cb_u0;
                            S.n_new = 0;
                        }
                        slot_tables(C, S);
                    }
                }
                __syncthreads();
                n_old = S.n_old;
                n_new = S.n_new;
                // the final sites' phase tables, for the commit
                if (C.charged) tables_f32();
            } else
            for (;;) {  // energy passes: one, or several for an orientation-biased move
            n_old = S.n_old;
            n_new = S.n_new;
            // ---- LJ and real-space sums of old sites (e < NS) and new sites (e >= NS)
            double acc[4 * NS];
#pragma unroll
            for (int e = 0; e < 4 * NS; ++e) acc[e] = 0.0;
            if constexpr (F32) {
                // FP64 displacement and image, then FP32 terms; this thread's
                // few FP32 partials are added in FP64 by the block sum
                float accf[4 * NS];
                ff closef[2 * NS];  // pairs closer than sigma, double-float
                double near_el[2 * NS];  // Coulomb pairs within 4.5 A, FP64
#pragma unroll
                for (int e = 0; e < 4 * NS; ++e) accf[e] = 0.f;
#pragma unroll
                for (int e = 0; e < 2 * NS; ++e) {
                    closef[e] = ff{0.f, 0.f};
                    near_el[e] = 0.0;
                }
                const float rc2f = (float)C.rc2, rcf = (float)C.rc, rce2f = (float)C.rc_ew2,
                            alphaf = (float)C.alpha;
                const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
                // atom j's records and its real-space Coulomb term with site slot e
                // (a near pair, within 6 A) from the double-float displacement and
                // charge, in double-float (FP64 beyond the erfc series)
                auto near_coulomb = [&](uint64_t j, int e) -> double {
                    float4 ah, al;
                    if (j < C.n_fw) {
                        ah = P.fwh[j];
                        al = P.fwl[j];
                    } else {
                        ah = ghi[j - C.n_fw];
                        al = glo[j - C.n_fw];
                    }
                    const float4 ph = sph[e], pl = spl[e];
                    ff dx = ff_add(ff{ah.x, al.x}, ff{-ph.x, -pl.x});
                    ff dy = ff_add(ff{ah.y, al.y}, ff{-ph.y, -pl.y});
                    ff dz = ff_add(ff{ah.z, al.z}, ff{-ph.z, -pl.z});
                    ff_min_image(C.lh, C.ll, C.linv, C.L.ortho, dx, dy, dz);
                    double v;
                    if (near_coulomb_ff(dx, dy, dz, ff{ah.w, al.w}, alpha_ff, v)) return v;
                    const double ddx = (double)dx.hi + dx.lo, ddy = (double)dy.hi + dy.lo,
                                 ddz = (double)dz.hi + dz.lo;
                    const double rd = fmax(sqrt(ddx * ddx + ddy * ddy + ddz * ddz), 1e-6);
                    return ((double)ah.w + (double)al.w) * (erfc(C.alpha * rd) / rd);
                };
                // Warp-uniform chunks of 32 atoms (lane l: atom jb + l). The near
                // Coulomb pairs are not evaluated where they are found: FP64 issues
                // at a small fraction of the FP32 rate and a warp pays a whole FP64
                // instruction for one lane, so a chunk's near pairs are appended to
                // the warp's list in (lane, slot) order and evaluated after the loop
                // by all threads, one pair a thread (a warp whose list is full
                // evaluates them in place).
                uint32_t nq = 0;  // entries in this warp's list (the same on every lane)
                for (uint64_t jb = j0 + (uint64_t)(threadIdx.x & ~31); jb < n_all; jb += GT) {
                    const uint64_t j = jb + (uint64_t)lane;
                    uint32_t nm = 0;  // slots whose Coulomb pair with atom j is near
                    bool skip = j >= n_all;
                    if (!skip && n_old)
#pragma unroll
                        for (int x = 0; x < NS; ++x) skip |= (S.ex[x] == (uint32_t)j);
                    if (!skip) {
                    float4 ah, al;
                    uint4 aq = make_uint4(0u, 0u, 0u, 0u);
                    uint32_t ta;
                    if (j < C.n_fw) {
                        ah = P.fwh[j];
                        al = P.fwl[j];
                        if constexpr (FX) aq = P.fwq[j];
                        ta = P.fw_type[j];
                    } else {
                        const uint64_t g = j - C.n_fw;
                        ah = ghi[g];
                        al = glo[g];
                        if constexpr (FX) aq = gq4[g];
                        ta = gt[g];
                    }
                    const float qa = ah.w;
#pragma unroll
                    for (int e = 0; e < 2 * NS; ++e) {
                        const bool is_old = e < NS;
                        if (is_old ? (e >= n_old) : (e - NS >= n_new)) continue;
                        // large cells: the wrapped fractional displacement, exact in
                        // fixed point, to Cartesian in FP32 (~2e-7 relative); pairs
                        // within NEAR_R (and cutoff-ambiguous ones under plain
                        // truncation) in double-float, the rest on that displacement
                        float cx = 0.f, cy = 0.f, cz = 0.f, r2 = 0.f;
                        bool near = true;
                        if constexpr (FX) {
                            const uint4 pq = sfq[e];
                            const float fx = (float)(int32_t)(aq.x - pq.x) * 2.3283064365386963e-10f;
                            const float fy = (float)(int32_t)(aq.y - pq.y) * 2.3283064365386963e-10f;
                            const float fz = (float)(int32_t)(aq.z - pq.z) * 2.3283064365386963e-10f;
                            cx = fmaf(fx, C.lh[0], fmaf(fy, C.lh[3], fz * C.lh[6]));
                            cy = fmaf(fx, C.lh[1], fmaf(fy, C.lh[4], fz * C.lh[7]));
                            cz = fmaf(fx, C.lh[2], fmaf(fy, C.lh[5], fz * C.lh[8]));
                            r2 = fmaf(cx, cx, fmaf(cy, cy, cz * cz));
                            near = r2 < NEAR_R2 ||
                                   (C.trunc == ALEA_TRUNCATED && fabsf(r2 - rc2f) <= CUT_BAND * rc2f);
                        }
                        ff dx{cx, 0.f}, dy{cy, 0.f}, dz{cz, 0.f};
                        if (near) {
                            const float4 ph = sph[e], pl = spl[e];
                            dx = ff_add(ff{ah.x, al.x}, ff{-ph.x, -pl.x});
                            dy = ff_add(ff{ah.y, al.y}, ff{-ph.y, -pl.y});
                            dz = ff_add(ff{ah.z, al.z}, ff{-ph.z, -pl.z});
                            ff_min_image(C.lh, C.ll, C.linv, C.L.ortho, dx, dy, dz);
                            r2 = fmaf(dx.hi, dx.hi, fmaf(dy.hi, dy.hi, dz.hi * dz.hi));
                        }
                        const bool lj_in = !(C.grid && j < C.n_fw) && r2 <= rc2f;
                        const bool el_in = C.charged && r2 <= rce2f;
                        if (!lj_in && !el_in) continue;
                        if (lj_in) {
                            const PairF32 q = srow32[S.row_slot[e]][ta];
                            if (r2 < q.sig2) {  // r < sigma: only ever a near pair
                                const ff rr = ff_add(ff_add(ff_mul(dx, dx), ff_mul(dy, dy)), ff_mul(dz, dz));
                                closef[e] = ff_add(closef[e], lj_close_ff(srowff[S.row_slot[e]][ta], rr, rcf, C.trunc));
                            } else {
                                const float ir2 = 1.0f / r2;
                                const float ir6 = ir2 * ir2 * ir2;
                                float v = ir6 * fmaf(q.a, ir6, -q.b) - q.shift;
                                if (C.trunc == ALEA_LINEAR_FORCE_SHIFTED) v -= (sqrtf(r2) - rcf) * q.dvdrc;
                                accf[2 * e] += v;
                            }
                        }
                        if (el_in) {
                            if (r2 < NEAR_COULOMB_R2) {
                                nm |= 1u << e;  // (NEAR_COULOMB_R2 <= NEAR_R2: dx, dy, dz are double-float)
                            } else {
                                const float r = sqrtf(r2);
                                accf[2 * e + 1] += qa * (erfcf(alphaf * r) / r);
                            }
                        }
                    }
                    }
                    // append the chunk's near pairs: lane order, then slot order
                    const uint32_t cnt = (uint32_t)__popc(nm);
                    uint32_t pre = cnt;  // inclusive prefix over the lanes
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t y = __shfl_up_sync(0xffffffffu, pre, o);
                        if (lane >= o) pre += y;
                    }
                    const uint32_t tot = __shfl_sync(0xffffffffu, pre, 31);
                    if (nq + tot <= NEAR_W) {
                        uint32_t at = nq + pre - cnt;
                        for (uint32_t m = nm; m; m &= m - 1)
                            nearq[wid][at++] = ((uint32_t)j << 4) | (uint32_t)(__ffs(m) - 1);
                        nq += tot;
                    } else {
#pragma unroll
                        for (int e = 0; e < 2 * NS; ++e)
                            if ((nm >> e) & 1u) near_el[e] += near_coulomb(j, e);
                    }
                }
                if (lane == 0) nearn[wid] = nq;
                __syncthreads();
                // the warps' lists in warp order, entry i on thread i mod GT
                for (uint32_t i = threadIdx.x;; i += GT) {
                    uint32_t w = 0, base = 0;
                    while (w < GT / 32 && base + nearn[w] <= i) base += nearn[w++];
                    if (w == GT / 32) break;
                    const uint32_t code = nearq[w][i - base];
                    const int e = (int)(code & 15u);
                    const double val = near_coulomb(code >> 4, e);
#pragma unroll
                    for (int e2 = 0; e2 < 2 * NS; ++e2)
                        if (e == e2) near_el[e2] += val;
                }
                // this thread's sums as double-float, added over the block
                ff v[4 * NS];
#pragma unroll
                for (int e = 0; e < 2 * NS; ++e) {
                    v[2 * e] = ff_add_f(closef[e], accf[2 * e]);
                    v[2 * e + 1] = ff_add(ff_from(near_el[e]), ff{accf[2 * e + 1], 0.f});
                }
                if (C.grid) {  // thread e adds site slot e's interpolated table
#pragma unroll
                    for (int e = 0; e < 2 * NS; ++e)
                        if (threadIdx.x == e && (e < NS ? e < n_old : e - NS < n_new))
                            v[2 * e] = ff_add(v[2 * e], ff_from(site_grid_energy<NS>(C, P, S, e)));
                }
                block_sum_ff(v, 4 * NS, red);
#pragma unroll
                for (int e = 0; e < 4 * NS; ++e) acc[e] = red[(GT / 32) * RSTRIDE + e];
                __syncthreads();
            } else
            for (uint64_t j = j0 + threadIdx.x; j < n_all; j += GT) {
                bool skip = false;
                if (n_old)
#pragma unroll
                    for (int x = 0; x < NS; ++x) skip |= (S.ex[x] == (uint32_t)j);
                if (skip) continue;
                double4 a;
                uint32_t ta;
                if (j < C.n_fw) {
                    a = P.fw[j];
                    ta = P.fw_type[j];
                } else {
                    const uint64_t g = j - C.n_fw;
                    a = make_double4(gx[g], gy[g], gz[g], gq[g]);
                    ta = gt[g];
                }
#pragma unroll
                for (int e = 0; e < 2 * NS; ++e) {
                    const bool is_old = e < NS;
                    if (is_old ? (e >= n_old) : (e - NS >= n_new)) continue;
                    const int s = is_old ? e : e - NS;
                    const double* p = is_old ? S.op[s] : S.np_[s];
                    double dx, dy, dz;
                    min_image(C.L, a.x - p[0], a.y - p[1], a.z - p[2], dx, dy, dz);
                    const double r2 = dx * dx + dy * dy + dz * dz;
                    const bool lj_in = !(C.grid && j < C.n_fw) && r2 <= C.rc2 * (1.0 + 1e-12);
                    const bool el_in = C.charged && r2 <= C.rc_ew2 * (1.0 + 1e-12);
                    if (!lj_in && !el_in) continue;
                    const double r = sqrt(r2);
                    if (lj_in) acc[2 * e] += lj_pair_rt(C.trunc, r, C.rc, srow[S.row_slot[e]][ta]);
                    if (el_in && r <= C.rc_ew) acc[2 * e + 1] += a.w * (erfc(C.alpha * r) / r);
                }
            }
            if constexpr (!F32) {
                if (C.grid) {
#pragma unroll
                    for (int e = 0; e < 2 * NS; ++e)
                        if (threadIdx.x == e && (e < NS ? e < n_old : e - NS < n_new))
                            acc[2 * e] += site_grid_energy<NS>(C, P, S, e);
                }
                block_sum_n(acc, 4 * NS, red);
            }
            if (threadIdx.x == 0)
#pragma unroll
                for (int e = 0; e < 2 * NS; ++e) {
                    const int s = e < NS ? e : e - NS;
                    S.e_lj[e] = acc[2 * e];
                    S.e_el[e] = (S.sq_slot[e] * acc[2 * e + 1]) * kCoulomb;
                }

            // ---- reciprocal delta: removed = old sites, added = new sites
            if constexpr (F32) {
              if (C.charged) {
                tables_f32();
                // per term w (2 S.delta + |delta|^2) in FP32 from the hi part of
                // S; this thread's ~nk/256 terms summed in FP32, the block's
                // partials in FP64. The delta is not stored: a commit forms it again.
                // (four terms a turn: their global loads issued together; the
                // terms are still added in the order t, t + GT, t + 2 GT, ...)
                float racc = 0.f;
                for (uint64_t t0 = threadIdx.x; t0 < C.nk; t0 += TU * GT) {
                    uint32_t pk[TU];
                    float2 o[TU];
                    float wv[TU];
#pragma unroll
                    for (int u = 0; u < TU; ++u) {
                        const uint64_t t = t0 + (uint64_t)u * GT;
                        const bool in = t < C.nk;
                        pk[u] = in ? P.npack[t] : 0u;  // 0: a valid table entry, weight 0
                        o[u] = in ? sk_hi[t] : make_float2(0.f, 0.f);
                        wv[u] = in ? P.w32[t] : 0.f;
                    }
#pragma unroll
                    for (int u = 0; u < TU; ++u) {
                        const float2 d = f32_delta(pk[u]);
                        const float dot = fmaf(o[u].x, d.x, o[u].y * d.y);
                        racc = fmaf(wv[u], fmaf(2.f, dot, fmaf(d.x, d.x, d.y * d.y)), racc);
                    }
                }
                ff v[1] = {ff{racc, 0.f}};
                block_sum_ff(v, 1, red);
                if (threadIdx.x == 0) {
                    S.rec_sum = C.rec_pref * red[(GT / 32) * RSTRIDE];
                    double q2a = 0.0, q2r = 0.0;
                    for (int s = 0; s < n_new; ++s) q2a += S.sq_slot[NS + s] * S.sq_slot[NS + s];
                    for (int s = 0; s < n_old; ++s) q2r += S.sq_slot[s] * S.sq_slot[s];
                    S.dself = C.self_pref * (q2a - q2r);
                    // a rigid molecule's exclusion sum is the template's
                    S.dexcl = -kCoulomb * ((n_new ? C.excl_tmpl[S.sp_new] : 0.0) -
                                           (n_old ? C.excl_tmpl[S.sp_old] : 0.0));
                }
              }
            } else if (C.charged) {
                for (int i = threadIdx.x; i < 2 * NS * 3 * tw; i += GT) {
                    const int e = i / (3 * tw), a = (i / tw) % 3, n = i % tw - K;
                    const bool is_old = e < NS;
                    if (is_old ? (e >= n_old) : (e - NS >= n_new)) continue;
                    const int s = is_old ? e : e - NS;
                    const double* p = is_old ? S.op[s] : S.np_[s];
                    const double th = C.b[3 * a] * p[0] + C.b[3 * a + 1] * p[1] + C.b[3 * a + 2] * p[2];
                    double sn, cs;
                    sincos((double)n * th, &sn, &cs);
                    etab[(e * 3 + a) * tw + n + K] = make_double2(cs, sn);
                }
                if (threadIdx.x < 2 * NS) eq[threadIdx.x] = S.sq_slot[threadIdx.x];
                __syncthreads();
                double racc = 0.0;
                for (uint64_t t = threadIdx.x; t < C.nk; t += GT) {
                    const int n0 = P.nidx[3 * t] + K, n1 = P.nidx[3 * t + 1] + K, n2 = P.nidx[3 * t + 2] + K;
                    double re = 0.0, im = 0.0;
                    if (n_new)  // added first (ewald_incremental_state.cc:107-111)
#pragma unroll
                        for (int s = 0; s < NS; ++s) {
                            if (s >= n_new) break;  // a smaller species' unused slots hold stale phases
                            const double2 A = etab[((NS + s) * 3 + 0) * tw + n0], B = etab[((NS + s) * 3 + 1) * tw + n1],
                                          Cc = etab[((NS + s) * 3 + 2) * tw + n2];
                            const double abr = A.x * B.x - A.y * B.y, abi = A.x * B.y + A.y * B.x;
                            re += eq[NS + s] * (abr * Cc.x - abi * Cc.y);
                            im += eq[NS + s] * (abr * Cc.y + abi * Cc.x);
                        }
                    if (n_old)  // then removed (:112-116)
#pragma unroll
                        for (int s = 0; s < NS; ++s) {
                            if (s >= n_old) break;
                            const double2 A = etab[(s * 3 + 0) * tw + n0], B = etab[(s * 3 + 1) * tw + n1],
                                          Cc = etab[(s * 3 + 2) * tw + n2];
                            const double abr = A.x * B.x - A.y * B.y, abi = A.x * B.y + A.y * B.x;
                            re -= eq[s] * (abr * Cc.x - abi * Cc.y);
                            im -= eq[s] * (abr * Cc.y + abi * Cc.x);
                        }
                    const double o_re = sre[t], o_im = sim[t];
                    const double n_re = o_re + re, n_im = o_im + im;
                    racc += P.w[t] * ((n_re * n_re + n_im * n_im) - (o_re * o_re + o_im * o_im));
                    dre[t] = re;
                    dim[t] = im;
                }
                double v[1] = {racc};
                block_sum_n(v, 1, red);
                if (threadIdx.x == 0) {
                    S.rec_sum = C.rec_pref * v[0];
                    double q2a = 0.0, q2r = 0.0;
                    for (int s = 0; s < n_new; ++s) q2a += S.sq_slot[NS + s] * S.sq_slot[NS + s];
                    for (int s = 0; s < n_old; ++s) q2r += S.sq_slot[s] * S.sq_slot[s];
                    S.dself = C.self_pref * (q2a - q2r);
                    S.dexcl = -kCoulomb * (exclusion_sum(C.L, S.np_, &S.sq_slot[NS], n_new, C.alpha) -
                                           exclusion_sum(C.L, S.op, &S.sq_slot[0], n_old, C.alpha));
                }
            }

            if (!S.cb) break;
            if (threadIdx.x == 0) {
                cbmc_after_pass(C, c, S, NS);
                if constexpr (F32)
                    if (S.cb_more) prep_sites_f32<NS, FX>(C, S, sph, spl, sfq);
            }
            __syncthreads();
            if (!S.cb_more) break;
            }  // energy passes

            // ---- acceptance (gcmc_acceptance.hpp:28-101)
            if (threadIdx.x == 0) {
                n_old = S.n_old;
                n_new = S.n_new;
                double u_old = 0.0, u_new = 0.0, e_old = 0.0, e_new = 0.0;
                for (int s = 0; s < n_old; ++s) {
                    u_old += S.e_lj[s];
                    e_old += S.e_el[s];
                }
                for (int s = 0; s < n_new; ++s) {
                    u_new += S.e_lj[NS + s];
                    e_new += S.e_el[NS + s];
                }
                const double rec = C.charged ? (S.rec_sum + S.dself) + S.dexcl : 0.0;
                const double T = C.temperature;
                double du, ratio;
                // opt-in: U_tail(after) - U_tail(before) of a change in the molecule counts
                double dut = 0.0;
                if (C.tail && S.move >= 2) {
                    auto lin = [&](int s) {
                        double v = C.tail_fw[s];
                        for (int s2 = 0; s2 < C.n_gsp; ++s2) v += (double)c.n_of[s2] * C.tail_x[s][s2];
                        return v;
                    };
                    if (S.move == 2)
                        dut = lin(S.sp_new) + C.tail_self[S.sp_new];
                    else if (S.move == 3)
                        dut = C.tail_self[S.sp_old] - lin(S.sp_old);
                    else
                        dut = (lin(S.sp_new) - lin(S.sp_old)) +
                              ((C.tail_self[S.sp_new] + C.tail_self[S.sp_old]) - C.tail_x[S.sp_old][S.sp_new]);
                }
                if (S.cb == 1) {  // orientation-biased insertion: W / k for exp(-dU/T)
                    du = S.cb_du + dut;
                    ratio = (c.fugacity[S.sp_new] * C.volume / T) / (double)(c.n_of[S.sp_new] + 1) *
                            exp(S.cb_logw - dut / T);
                    if (C.prop_cells > 0) ratio *= exp(-S.lq);
                } else if (S.cb == 2) {  // orientation-biased deletion: k / W for exp(+U/T)
                    du = S.cb_du + dut;
                    ratio = (double)c.n_of[S.sp_old] / (c.fugacity[S.sp_old] * C.volume / T) *
                            exp(-S.cb_logw - dut / T);
                    if (C.prop_cells > 0) ratio *= exp(S.lq);
                } else if (S.move <= 1) {
                    du = (u_new - u_old) + (e_new - e_old) + rec;
                    ratio = exp(-du / T);
                } else if (S.move == 2) {
                    du = u_new + e_new + rec + dut;
                    ratio = (c.fugacity[S.sp_new] * C.volume / T) / (double)(c.n_of[S.sp_new] + 1) *
                            exp(-du / T);
                    // learned proposal: divided by its density (relative to uniform)
                    if (C.prop_cells > 0) ratio *= exp(-S.lq);
                } else if (S.move == 3) {
                    du = -(u_old + e_old) + rec + dut;
                    ratio = (double)c.n_of[S.sp_old] / (c.fugacity[S.sp_old] * C.volume / T) *
                            exp(-du / T);
                    // the reverse insertion's proposal density at this centroid
                    if (C.prop_cells > 0) ratio *= exp(S.lq);
                } else {  // swapRatio (gcmc_acceptance.hpp:89-95)
                    du = (u_new - u_old) + (e_new - e_old) + rec + dut;
                    ratio = (c.fugacity[S.sp_new] / c.fugacity[S.sp_old]) *
                            ((double)c.n_of[S.sp_old] / (double)(c.n_of[S.sp_new] + 1)) * exp(-du / T);
                }
                c.attempted[S.move]++;
                const double prob = ratio < 1.0 ? ratio : 1.0;
                S.accept = u01(c) < prob ? 1 : 0;
                if (S.accept && ((S.move == 2 && c.n_mol + 1 > C.max_mol) ||
                                 (S.move >= 2 && c.n_guest + S.n_new > C.max_sites))) {
                    c.err |= DEV_ERR_CAPACITY;  // the chain stops; the host reports it
                    S.accept = 0;
                }
                c.last_du = du;
            }
            __syncthreads();

            if (S.accept) {
                if (C.charged) {
                    if constexpr (F32) {  // S += delta in double-float on the FP32 pipe
                        for (uint64_t t = threadIdx.x; t < C.nk; t += GT) {
                            const float2 d = f32_delta(P.npack[t]);
                            const float2 h = sk_hi[t], l = sk_lo[t];
                            const ff re = ff_add_f(ff{h.x, l.x}, d.x), im = ff_add_f(ff{h.y, l.y}, d.y);
                            sk_hi[t] = make_float2(re.hi, im.hi);
                            sk_lo[t] = make_float2(re.lo, im.lo);
                        }
                    } else {
                        for (uint64_t t = threadIdx.x; t < C.nk; t += GT) {
                            sre[t] += dre[t];
                            sim[t] += dim[t];
                        }
                    }
                }
                if (threadIdx.x == 0) {
                    c.accepted[S.move]++;
                    if (C.charged) {
                        c.self_e += S.dself;
                        c.excl_e += S.dexcl;
                    }
                    // removeParticleIndices (monte_carlo_engine.cc:825-848):
                    // swap-with-last, fixing the molecule records that held the last site
                    auto remove_sites = [&](uint32_t* idx, int n) {
                        for (int k = 0; k < n; ++k) {
                            const uint32_t site = idx[k];
                            const uint32_t last = (uint32_t)(C.n_fw + c.n_guest - 1);
                            if (site != last) {
                                const uint32_t ds = site - (uint32_t)C.n_fw, ls = last - (uint32_t)C.n_fw;
                                gx[ds] = gx[ls];
                                gy[ds] = gy[ls];
                                gz[ds] = gz[ls];
                                gq[ds] = gq[ls];
                                gt[ds] = gt[ls];
                                ghi[ds] = ghi[ls];
                                glo[ds] = glo[ls];
                                gq4[ds] = gq4[ls];
                                for (uint64_t m = 0; m < c.n_mol; ++m) {
                                    const int nsm = C.sp_ns[msp[m]];
                                    for (int s2 = 0; s2 < nsm; ++s2)
                                        if (mol[(size_t)m * NS + s2] == last) mol[(size_t)m * NS + s2] = site;
                                }
                                for (int k2 = k + 1; k2 < n; ++k2)
                                    if (idx[k2] == last) idx[k2] = site;
                            }
                            c.n_guest -= 1;
                        }
                    };
                    // the new sites appended after the guests (insertion, swap)
                    auto append_new = [&](uint64_t mrec) {
                        for (int s = 0; s < S.n_new; ++s) {
                            const uint32_t slot = (uint32_t)c.n_guest + s;
                            gx[slot] = S.np_[s][0];
                            gy[slot] = S.np_[s][1];
                            gz[slot] = S.np_[s][2];
                            gq[slot] = S.sq_slot[NS + s];
                            gt[slot] = C.splj[S.sp_new][s];
                            put_hilo(C.L, ghi, glo, gq4, slot, S.np_[s], S.sq_slot[NS + s]);
                            mol[(size_t)mrec * NS + s] = (uint32_t)C.n_fw + slot;
                        }
                        msp[mrec] = (uint32_t)S.sp_new;
                        c.n_guest += S.n_new;
                    };
                    if (S.move <= 1) {
                        for (int s = 0; s < S.n_new; ++s) {
                            const uint32_t slot = S.ex[s] - (uint32_t)C.n_fw;
                            gx[slot] = S.np_[s][0];
                            gy[slot] = S.np_[s][1];
                            gz[slot] = S.np_[s][2];
                            put_hilo(C.L, ghi, glo, gq4, slot, S.np_[s], S.sq_slot[NS + s]);
                        }
                    } else if (S.move == 2) {
                        append_new(c.n_mol);
                        c.n_mol += 1;
                        c.n_of[S.sp_new] += 1;
                    } else if (S.move == 3) {  // removeMolecule (:814-823): erase, then remove
                        uint32_t idx[MAXS];
                        for (int s = 0; s < S.n_old; ++s) idx[s] = S.ex[s];
                        for (uint32_t m = S.mi; m + 1 < c.n_mol; ++m) {
                            for (int s = 0; s < NS; ++s) mol[(size_t)m * NS + s] = mol[(size_t)(m + 1) * NS + s];
                            msp[m] = msp[m + 1];
                        }
                        c.n_mol -= 1;
                        c.n_of[S.sp_old] -= 1;
                        remove_sites(idx, S.n_old);
                    } else {  // swap: the molecule becomes the new species, then the old sites go
                        uint32_t idx[MAXS];
                        for (int s = 0; s < S.n_old; ++s) idx[s] = S.ex[s];
                        append_new(S.mi);
                        c.n_of[S.sp_old] -= 1;
                        c.n_of[S.sp_new] += 1;
                        remove_sites(idx, S.n_old);
                    }
                    if (C.charged) {
                        c.moves_since_resync++;
                        if (c.moves_since_resync >= 100) {
                            S.do_resync = 1;
                            c.moves_since_resync = 0;
                            c.resyncs++;
                        }
                    }
                    S.ng_after = c.n_guest;
                }
                __syncthreads();
                if (S.do_resync) {
                    const uint64_t ng = S.ng_after;
                    if constexpr (F32) {
                        // the framework's S(k), then the guest sites in chunks of 2 NS
                        // through the phase tables (each site's angles reduced in FP64
                        // once per n), products in FP32, each chunk's sum added in
                        // double-float
                        for (uint64_t t = threadIdx.x; t < C.nk; t += GT) {
                            sk_hi[t] = P.sfw_hi[t];
                            sk_lo[t] = P.sfw_lo[t];
                        }
                        for (uint64_t g0 = 0; g0 < ng; g0 += 2 * NS) {
                            const int m = (int)min((uint64_t)(2 * NS), ng - g0);
                            __syncthreads();  // the previous chunk's tables are read
                            for (int i = threadIdx.x; i < m * 3 * tw; i += GT) {
                                const int e = i / (3 * tw), a = (i / tw) % 3, n = i % tw - K;
                                const uint64_t g = g0 + e;
                                const double th = C.b[3 * a] * gx[g] + C.b[3 * a + 1] * gy[g] + C.b[3 * a + 2] * gz[g];
                                const double x = (double)n * th;
                                const double r = x - (2.0 * kPi) * rint(x * (0.5 / kPi));
                                float sn, cs;
                                sincosf((float)r, &sn, &cs);
                                etab32[i] = make_float2(cs, sn);
                            }
                            __syncthreads();
                            for (uint64_t t = threadIdx.x; t < C.nk; t += GT) {
                                const uint32_t pk = P.npack[t];
                                const int n0 = pk & 0xff, n1 = (pk >> 8) & 0xff, n2 = (pk >> 16) & 0xff;
                                float re = 0.f, im = 0.f;
                                for (int e = 0; e < m; ++e) {
                                    const float q = ghi[g0 + e].w;
                                    const float2 A = etab32[(e * 3 + 0) * tw + n0], B = etab32[(e * 3 + 1) * tw + n1],
                                                 Cc = etab32[(e * 3 + 2) * tw + n2];
                                    const float abr = A.x * B.x - A.y * B.y, abi = A.x * B.y + A.y * B.x;
                                    re = fmaf(q, abr * Cc.x - abi * Cc.y, re);
                                    im = fmaf(q, abr * Cc.y + abi * Cc.x, im);
                                }
                                const float2 h = sk_hi[t], l = sk_lo[t];
                                const ff fr = ff_add_f(ff{h.x, l.x}, re), fi = ff_add_f(ff{h.y, l.y}, im);
                                sk_hi[t] = make_float2(fr.hi, fi.hi);
                                sk_lo[t] = make_float2(fr.lo, fi.lo);
                            }
                        }
                    } else {
                        for (uint64_t t = threadIdx.x; t < C.nk; t += GT) {
                            const double k0 = P.k[3 * t], k1 = P.k[3 * t + 1], k2 = P.k[3 * t + 2];
                            double re = P.sfw_re[t], im = P.sfw_im[t];
                            for (uint64_t g = 0; g < ng; ++g) {
                                double sn, cs;
                                sincos(k0 * gx[g] + k1 * gy[g] + k2 * gz[g], &sn, &cs);
                                re += gq[g] * cs;
                                im += gq[g] * sn;
                            }
                            sre[t] = re;
                            sim[t] = im;
                        }
                    }
                    if (threadIdx.x == 0) {
                        double q2 = C.fw_q2;
                        for (uint64_t g = 0; g < ng; ++g) q2 += gq[g] * gq[g];
                        c.self_e = C.self_pref * q2;
                        double ex = 0.0;
                        if constexpr (F32) {
                            for (uint32_t m = 0; m < c.n_mol; ++m) ex += C.excl_tmpl[msp[m]];
                        } else
                        for (uint32_t m = 0; m < c.n_mol; ++m) {
                            const int nsm = C.sp_ns[msp[m]];
                            double p[MAXS][3], q[MAXS];
                            for (int s = 0; s < nsm; ++s) {
                                const uint32_t slot = mol[(size_t)m * NS + s] - (uint32_t)C.n_fw;
                                p[s][0] = gx[slot];
                                p[s][1] = gy[slot];
                                p[s][2] = gz[slot];
                                q[s] = gq[slot];
                            }
                            ex += exclusion_sum(C.L, p, q, nsm, C.alpha);
                        }
                        c.excl_e = -kCoulomb * ex;
                    }
                }
            }
        }
        if (threadIdx.x == 0) {
            c.steps++;
            c.sum_n += (double)c.n_mol;
            c.sum_n2 += (double)c.n_mol * (double)c.n_mol;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        P.st[chain] = c;
        if (c.err) atomicOr(P.flags, c.err);
    }
}

template <int NS>
void launch_chains(unsigned n_chains, const GcmcConst& C, const GcmcPtrs& P, uint64_t steps,
                   cudaStream_t s) {
    size_t bytes = C.charged ? phase_bytes<NS>(C.kmax, C.f32 != 0) : 0;
    if (C.charged && C.f32 && C.orient > 1 && C.orient <= FUSE_MAX)  // the trial sites' tables
        bytes = phase_bytes<NS>(C.kmax, true) + (size_t)C.orient * NS * 3 * (2 * C.kmax + 1) * sizeof(float2);
    if (C.f32) {
        auto kern = C.fixed_far ? gcmc_kernel<NS, true, true> : gcmc_kernel<NS, true, false>;
        ALEA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
        kern<<<n_chains, GT, bytes, s>>>(C, P, steps);
    } else {
        ALEA_CUDA(cudaFuncSetAttribute(gcmc_kernel<NS, false, false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
        gcmc_kernel<NS, false, false><<<n_chains, GT, bytes, s>>>(C, P, steps);
    }
}

// The committed S(k) between the forms: FP64 to double-float (to_f32) or back.
__global__ void convert_sk_kernel(uint64_t n, int to_f32, double* re, double* im, float2* hi,
                                  float2* lo) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    if (to_f32) {
        const ff fr = ff_from(re[t]), fi = ff_from(im[t]);
        hi[t] = make_float2(fr.hi, fi.hi);
        lo[t] = make_float2(fr.lo, fi.lo);
    } else {
        re[t] = (double)hi[t].x + (double)lo[t].x;
        im[t] = (double)hi[t].y + (double)lo[t].y;
    }
}

// Every chain's committed S(k) starts as the framework's, in FP64 and as
// double-float; the weights' FP32 copy and the packed term indices too.
__global__ void gather_sfw_kernel(uint64_t nk, const double* re, const double* im, const double* w,
                                  const int* nidx, int kmax, double* out_re, double* out_im,
                                  float2* out_hi, float2* out_lo, float2* fw_hi, float2* fw_lo,
                                  float* w32, uint32_t* npack, unsigned n_chains) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nk) return;
    w32[t] = (float)w[t];
    npack[t] = (uint32_t)(nidx[3 * t] + kmax) | (uint32_t)(nidx[3 * t + 1] + kmax) << 8 |
               (uint32_t)(nidx[3 * t + 2] + kmax) << 16;
    const ff fr = ff_from(re[t]), fi = ff_from(im[t]);
    fw_hi[t] = make_float2(fr.hi, fi.hi);
    fw_lo[t] = make_float2(fr.lo, fi.lo);
    for (unsigned c = 0; c < n_chains; ++c) {
        out_re[(size_t)c * nk + t] = re[t];
        out_im[(size_t)c * nk + t] = im[t];
        out_hi[(size_t)c * nk + t] = make_float2(fr.hi, fi.hi);
        out_lo[(size_t)c * nk + t] = make_float2(fr.lo, fi.lo);
    }
}

}  // namespace

struct GcmcImpl {
    GcmcConst C{};
    unsigned n_chains = 0;
    DevBuf<double4> fw;
    DevBuf<uint32_t> fw_type;
    DevBuf<PairParams> table;
    DevBuf<double> k, w, sfw_re, sfw_im;
    DevBuf<int> nidx;
    DevBuf<ChainState> st;
    DevBuf<double> gx, gy, gz, gq, sre, sim, dre, dim;
    DevBuf<uint32_t> gt, mol;
    DevBuf<unsigned> flags;
    DevBuf<double> pcdf, plogp;  // the chains' copy of a tabulated proposal
    DevBuf<float4> fwh, fwl, ghi, glo;  // FP32 form: double-float positions
    DevBuf<uint4> fwq, gq4;             // FP32 form: fixed-point fractional positions
    DevBuf<uint32_t> msp;               // species of each molecule, per chain
    DevBuf<float> w32;                  // FP32 form: the weights
    DevBuf<float2> sk_hi, sk_lo;        // FP32 form: each chain's S(k) as double-float
    DevBuf<float2> sfw_hi, sfw_lo;      // FP32 form: the framework's S(k) as double-float
    DevBuf<uint32_t> npack;             // FP32 form: packed (n0, n1, n2) per term
    const double* gtab[MAXROWS] = {};  // the borrowed grid's tables, per pair-table row
    float last_ms = 0.f;
};

GcmcImpl* gcmc_create(const alea_lennard_jones& lj, const alea_ewald* ew, const alea_particles& fw,
                      const alea_lattice& lat, uint32_t n_gsp, const alea_molecule_species* guests,
                      double temperature, const double* fugacity_pa, const uint64_t* seeds,
                      const uint64_t* streams, uint32_t n_chains, double max_translation,
                      double max_rotation, int draw_order, uint32_t max_molecules) {
    require(n_chains >= 1, ALEA_ERR_INVALID_ARGUMENT, "GCMC: at least one chain");
    require(n_gsp >= 1 && n_gsp <= (uint32_t)MAXGS, ALEA_ERR_INVALID_ARGUMENT,
            "GCMC: 1..4 guest species");
    int ns_max = 0;
    for (uint32_t k = 0; k < n_gsp; ++k) {
        require(guests[k].n_sites >= 1 && guests[k].n_sites <= 5, ALEA_ERR_INVALID_ARGUMENT,
                "GCMC: 1..5 sites per molecule are compiled");
        ns_max = std::max(ns_max, (int)guests[k].n_sites);
    }
    require(temperature > 0.0, ALEA_ERR_INVALID_ARGUMENT,
            "MonteCarloEngine: temperatureKelvin must be positive");
    require(lj.cutoff > 0.0 && lj.n_species >= 1 && lj.n_species <= 64, ALEA_ERR_INVALID_ARGUMENT,
            "GCMC: LJ cutoff > 0 and 1..64 species");
    require(max_molecules >= 1, ALEA_ERR_INVALID_ARGUMENT, "GCMC: max_molecules >= 1");
    require(draw_order == ALEA_DRAWS_RIGHT_TO_LEFT || draw_order == ALEA_DRAWS_LEFT_TO_RIGHT,
            ALEA_ERR_INVALID_ARGUMENT, "GCMC: unknown draw order");
    require(fw.n == 0 || (fw.x && fw.y && fw.z), ALEA_ERR_INVALID_ARGUMENT,
            "GCMC: framework coordinates missing");
    for (uint64_t i = 0; i < (uint64_t)n_chains * n_gsp; ++i)
        require(fugacity_pa[i] * (1.0 / (1.380649e-23 * 1.0e30)) > 0.0, ALEA_ERR_INVALID_ARGUMENT,
                "MonteCarloEngine: every fugacityPascal must be positive");
    auto* g = new GcmcImpl();
    try {
        GcmcConst& C = g->C;
        C.L = make_lattice(lat.m);
        validate_cutoff(C.L, lj.cutoff, "MonteCarloEngine (LJ)");
        C.ns = ns_max;
        C.n_gsp = (int)n_gsp;
        C.n_rows = 0;
        for (uint32_t k = 0; k < n_gsp; ++k) {
            const alea_molecule_species& guest = guests[k];
            C.sp_ns[k] = (int)guest.n_sites;
            double qs = 0.0;
            for (uint32_t s = 0; s < guest.n_sites; ++s) {
                require(guest.lj_species[s] < lj.n_species, ALEA_ERR_OUT_OF_RANGE,
                        "GCMC: site LJ species out of range");
                C.spx[k][s] = guest.x[s];
                C.spy[k][s] = guest.y[s];
                C.spz[k][s] = guest.z[s];
                C.spq[k][s] = guest.charge ? guest.charge[s] : 0.0;
                C.splj[k][s] = guest.lj_species[s];
                int r = 0;
                while (r < C.n_rows && C.row_lj[r] != guest.lj_species[s]) ++r;
                if (r == C.n_rows) {
                    require(C.n_rows < MAXROWS, ALEA_ERR_INVALID_ARGUMENT,
                            "GCMC: at most 8 distinct LJ species among the guest sites");
                    C.row_lj[C.n_rows++] = guest.lj_species[s];
                }
                C.sprow[k][s] = r;
                C.tc[k][s][0] = guest.x[s];
                C.tc[k][s][1] = guest.y[s];
                C.tc[k][s][2] = guest.z[s];
                qs += C.spq[k][s];
            }
            // monte_carlo_engine.cc:273-293
            if (ew)
                require(std::fabs(qs) <= 1e-8, ALEA_ERR_INVALID_ARGUMENT,
                        "MonteCarloEngine: GCMC species " + std::to_string(k) +
                            " is not individually charge-neutral (total site charge = " +
                            std::to_string(qs) +
                            " e); every insertion/deletion/swap would drift the system away from "
                            "neutrality, which electrostatics requires");
            // pairExclusionSum of the template (ewald_incremental_state.cc:32-43): a rigid
            // molecule's, wherever it is (its pairs are far shorter than half a cell)
            double ex = 0.0;
            for (int i = 0; i < (int)guest.n_sites; ++i)
                for (int j = i + 1; j < (int)guest.n_sites; ++j) {
                    const double dx = guest.x[j] - guest.x[i], dy = guest.y[j] - guest.y[i],
                                 dz = guest.z[j] - guest.z[i];
                    const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
                    const double qq = C.spq[k][i] * C.spq[k][j];
                    if (ew) ex += qq * (r < 1e-8 ? 2.0 * ew->alpha / std::sqrt(kPi) : std::erf(ew->alpha * r) / r);
                }
            C.excl_tmpl[k] = ex;
            // the template about its centroid (the learned proposal's reference point)
            double m[3] = {0.0, 0.0, 0.0};
            for (int s = 0; s < C.sp_ns[k]; ++s)
                for (int i = 0; i < 3; ++i) m[i] += C.tc[k][s][i];
            for (int s = 0; s < C.sp_ns[k]; ++s)
                for (int i = 0; i < 3; ++i) C.tc[k][s][i] -= m[i] / C.sp_ns[k];
        }
        C.n_species = lj.n_species;
        C.rc = lj.cutoff;
        C.rc2 = lj.cutoff * lj.cutoff;
        C.trunc = lj.truncation;
        C.temperature = temperature;
        C.max_trans = max_translation;
        C.max_rot = max_rotation;
        C.draw_order = draw_order;
        C.n_fw = fw.n;
        C.max_mol = max_molecules;
        C.max_sites = max_molecules * (uint32_t)C.ns;
        C.volume = std::fabs(C.L.volume);
        std::vector<double4> packed(fw.n);
        std::vector<uint32_t> types(fw.n, 0);
        double fwq = 0.0, fwq2 = 0.0;
        for (uint64_t i = 0; i < fw.n; ++i) {
            const double q = fw.charge ? fw.charge[i] : 0.0;
            packed[i] = make_double4(fw.x[i], fw.y[i], fw.z[i], q);
            if (fw.species) {
                require(fw.species[i] < lj.n_species, ALEA_ERR_OUT_OF_RANGE,
                        "GCMC: framework species out of range");
                types[i] = fw.species[i];
            }
            fwq += q;
            fwq2 += q * q;
        }
        C.fw_q2 = fwq2;
        EwaldStateImpl* ews = nullptr;
        if (ew) {
            // monte_carlo_engine.cc:273-293
            require(std::fabs(fwq) <= 1e-8, ALEA_ERR_INVALID_ARGUMENT,
                    "MonteCarloEngine: framework is not charge-neutral (total charge = " +
                        std::to_string(fwq) + " e)");
            require(ew->kmax <= KMAXC, ALEA_ERR_INVALID_ARGUMENT, "GCMC: kMax <= 64 supported");
            validate_cutoff(C.L, ew->real_space_cutoff, "MonteCarloEngine (Ewald real space)");
        }
        require_device();
        g->n_chains = n_chains;
        g->fw.alloc(std::max<size_t>(fw.n, 1));
        g->fw_type.alloc(std::max<size_t>(fw.n, 1));
        g->fw.upload(packed.data(), fw.n);
        g->fw_type.upload(types.data(), fw.n);
        {
            std::vector<float4> h(fw.n), l(fw.n);
            for (uint64_t i = 0; i < fw.n; ++i) {
                const ff x = ff_from(packed[i].x), y = ff_from(packed[i].y), z = ff_from(packed[i].z),
                         q = ff_from(packed[i].w);
                h[i] = make_float4(x.hi, y.hi, z.hi, q.hi);
                l[i] = make_float4(x.lo, y.lo, z.lo, q.lo);
            }
            g->fwh.alloc(std::max<size_t>(fw.n, 1));
            g->fwl.alloc(std::max<size_t>(fw.n, 1));
            g->fwh.upload(h.data(), fw.n);
            g->fwl.upload(l.data(), fw.n);
            std::vector<uint4> fq(fw.n);
            for (uint64_t i = 0; i < fw.n; ++i)
                fq[i] = fixed_frac(C.L, packed[i].x, packed[i].y, packed[i].z);
            g->fwq.alloc(std::max<size_t>(fw.n, 1));
            g->fwq.upload(fq.data(), fw.n);
            C.fixed_far = std::fabs(C.L.volume) > FIXED_FAR_VOLUME;
            for (int i = 0; i < 9; ++i) {
                const ff m = ff_from(C.L.m[i]);
                C.lh[i] = m.hi;
                C.ll[i] = m.lo;
                C.linv[i] = (float)C.L.inv[i];
            }
        }
        std::vector<PairParams> table((size_t)lj.n_species * lj.n_species);
        mixed_table(lj, table.data());
        g->table.alloc(table.size());
        g->table.upload(table.data(), table.size());
        {  // the tail-correction constants (used when switched on)
            const uint32_t nsp = lj.n_species;
            const double rc = lj.cutoff, rc3 = rc * rc * rc;
            std::vector<double> f((size_t)nsp * nsp), fw_n(nsp, 0.0);
            for (uint32_t a = 0; a < nsp; ++a)
                for (uint32_t b = 0; b < nsp; ++b) {  // tailEnergyCorrection's integral
                    const PairParams& pp = table[(size_t)a * nsp + b];
                    const double sr3 = pp.sigma * pp.sigma * pp.sigma;
                    const double sr9 = sr3 * sr3 * sr3 / (rc3 * rc3 * rc3);
                    f[(size_t)a * nsp + b] = pp.eps * sr3 * ((4.0 / 9.0) * sr9 - (4.0 / 3.0) * (sr3 / rc3));
                }
            for (uint64_t i = 0; i < fw.n; ++i) fw_n[types[i]] += 1.0;
            std::vector<std::vector<double>> d(n_gsp, std::vector<double>(nsp, 0.0));
            for (uint32_t k = 0; k < n_gsp; ++k)
                for (int s = 0; s < C.sp_ns[k]; ++s) d[k][C.splj[k][s]] += 1.0;
            const double K = 2.0 * kPi / C.volume;
            auto form = [&](const std::vector<double>& u, const std::vector<double>& v) {
                double t = 0.0;
                for (uint32_t a = 0; a < nsp; ++a)
                    if (u[a] != 0.0)
                        for (uint32_t b = 0; b < nsp; ++b) t += u[a] * v[b] * f[(size_t)a * nsp + b];
                return t;
            };
            for (uint32_t k = 0; k < n_gsp; ++k) {
                C.tail_fw[k] = 2.0 * K * form(d[k], fw_n);
                C.tail_self[k] = K * form(d[k], d[k]);
                for (uint32_t k2 = 0; k2 < n_gsp; ++k2) C.tail_x[k][k2] = 2.0 * K * form(d[k], d[k2]);
            }
            C.tail = 0;
            C.orient = 1;
        }
        uint64_t nk = 0;
        if (ew) {
            ews = ewald_state_create(*ew, fw, lat);
            const EwaldDeviceView v = ewald_state_view(ews);
            nk = v.nk;
            C.charged = 1;
            C.alpha = ew->alpha;
            C.rc_ew = ew->real_space_cutoff;
            C.rc_ew2 = C.rc_ew * C.rc_ew;
            C.kmax = ew->kmax;
            C.nk = nk;
            for (int i = 0; i < 9; ++i) C.b[i] = v.b[i];
            C.self_pref = v.self_pref;
            C.rec_pref = v.rec_pref;
            g->k.alloc(3 * nk);
            g->w.alloc(nk);
            g->nidx.alloc(3 * nk);
            g->sfw_re.alloc(nk);
            g->sfw_im.alloc(nk);
            ALEA_CUDA(cudaMemcpy(g->k.p, v.k, 3 * nk * sizeof(double), cudaMemcpyDeviceToDevice));
            ALEA_CUDA(cudaMemcpy(g->w.p, v.w, nk * sizeof(double), cudaMemcpyDeviceToDevice));
            ALEA_CUDA(cudaMemcpy(g->nidx.p, v.nidx, 3 * nk * sizeof(int), cudaMemcpyDeviceToDevice));
            ALEA_CUDA(cudaMemcpy(g->sfw_re.p, v.sre, nk * sizeof(double), cudaMemcpyDeviceToDevice));
            ALEA_CUDA(cudaMemcpy(g->sfw_im.p, v.sim, nk * sizeof(double), cudaMemcpyDeviceToDevice));
        }
        const size_t nkc = std::max<uint64_t>(nk, 1);
        g->sre.alloc(nkc * n_chains);
        g->sim.alloc(nkc * n_chains);
        g->dre.alloc(nkc * n_chains);
        g->dim.alloc(nkc * n_chains);
        g->w32.alloc(nkc);
        g->npack.alloc(nkc);
        g->sk_hi.alloc(nkc * n_chains);
        g->sk_lo.alloc(nkc * n_chains);
        g->sfw_hi.alloc(nkc);
        g->sfw_lo.alloc(nkc);
        if (ews) {
            gather_sfw_kernel<<<(unsigned)((nk + 255) / 256), 256>>>(
                nk, g->sfw_re.p, g->sfw_im.p, g->w.p, g->nidx.p, C.kmax, g->sre.p, g->sim.p,
                g->sk_hi.p, g->sk_lo.p, g->sfw_hi.p, g->sfw_lo.p, g->w32.p, g->npack.p, n_chains);
            ALEA_CUDA(cudaGetLastError());
        }
        const size_t sites = (size_t)C.max_sites * n_chains;
        g->gx.alloc(sites);
        g->gy.alloc(sites);
        g->gz.alloc(sites);
        g->gq.alloc(sites);
        g->gt.alloc(sites);
        g->mol.alloc(sites);
        g->ghi.alloc(sites);
        g->glo.alloc(sites);
        g->gq4.alloc(sites);
        g->msp.alloc((size_t)max_molecules * n_chains);
        std::vector<ChainState> st(n_chains);
        const double self0 = ews ? ewald_state_view(ews).self_pref * fwq2 : 0.0;
        for (uint32_t c = 0; c < n_chains; ++c) {
            ChainState& s = st[c];
            s = ChainState{};
            s.seed = seeds[c];
            s.stream = streams[c];
            for (uint32_t k = 0; k < n_gsp; ++k)
                s.fugacity[k] = fugacity_pa[(size_t)c * n_gsp + k] * (1.0 / (1.380649e-23 * 1.0e30));
            s.self_e = self0;
        }
        if (ews) {
            // the committed self energy is the framework's (ewald_incremental_state.cc:77-81)
            const auto raw = ewald_state_raw(ews);
            for (auto& s : st) s.self_e = raw[2 * nk];
            ewald_state_destroy(ews);
        }
        g->st.alloc(n_chains);
        g->st.upload(st.data(), n_chains);
        g->flags.alloc(1);
        ALEA_CUDA(cudaMemset(g->flags.p, 0, sizeof(unsigned)));
        ALEA_CUDA(cudaDeviceSynchronize());
    } catch (...) {
        delete g;
        throw;
    }
    return g;
}

void gcmc_run(GcmcImpl* g, uint64_t steps, cudaStream_t s) {
    GcmcPtrs P{};
    P.fw = g->fw.p;
    P.fw_type = g->fw_type.p;
    P.table = g->table.p;
    P.k = g->k.p;
    P.w = g->w.p;
    P.nidx = g->nidx.p;
    P.sfw_re = g->sfw_re.p;
    P.sfw_im = g->sfw_im.p;
    P.st = g->st.p;
    P.gx = g->gx.p;
    P.gy = g->gy.p;
    P.gz = g->gz.p;
    P.gq = g->gq.p;
    P.gt = g->gt.p;
    P.mol = g->mol.p;
    P.sre = g->sre.p;
    P.sim = g->sim.p;
    P.dre = g->dre.p;
    P.dim = g->dim.p;
    P.flags = g->flags.p;
    P.pcdf = g->pcdf.p;
    P.plogp = g->plogp.p;
    P.fwh = g->fwh.p;
    P.fwl = g->fwl.p;
    P.ghi = g->ghi.p;
    P.gq4 = g->gq4.p;
    P.fwq = g->fwq.p;
    P.glo = g->glo.p;
    P.w32 = g->w32.p;
    for (int r = 0; r < MAXROWS; ++r) P.gtab[r] = g->gtab[r];
    P.msp = g->msp.p;
    P.sk_hi = g->sk_hi.p;
    P.sk_lo = g->sk_lo.p;
    P.sfw_hi = g->sfw_hi.p;
    P.sfw_lo = g->sfw_lo.p;
    P.npack = g->npack.p;
    cudaEvent_t e0, e1;
    ALEA_CUDA(cudaEventCreate(&e0));
    ALEA_CUDA(cudaEventCreate(&e1));
    ALEA_CUDA(cudaEventRecord(e0, s));
    switch (g->C.ns) {
        case 1: launch_chains<1>(g->n_chains, g->C, P, steps, s); break;
        case 2: launch_chains<2>(g->n_chains, g->C, P, steps, s); break;
        case 3: launch_chains<3>(g->n_chains, g->C, P, steps, s); break;
        case 4: launch_chains<4>(g->n_chains, g->C, P, steps, s); break;
        default: launch_chains<5>(g->n_chains, g->C, P, steps, s); break;
    }
    ALEA_CUDA(cudaGetLastError());
    ALEA_CUDA(cudaEventRecord(e1, s));
    ALEA_CUDA(cudaEventSynchronize(e1));
    ALEA_CUDA(cudaEventElapsedTime(&g->last_ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    check_device_flags(g->flags.p, s, "GCMC chains (capacity: raise max_molecules)");
}

void gcmc_states(const GcmcImpl* g, ChainState* out) {
    g->st.download(out, g->n_chains);
    ALEA_CUDA(cudaDeviceSynchronize());
}

uint64_t gcmc_particles(const GcmcImpl* g, uint32_t chain, double* xyz, uint64_t cap) {
    require(chain < g->n_chains, ALEA_ERR_OUT_OF_RANGE, "GCMC: chain index");
    ChainState s;
    ALEA_CUDA(cudaMemcpy(&s, g->st.p + chain, sizeof s, cudaMemcpyDeviceToHost));
    const uint64_t n = g->C.n_fw + s.n_guest;
    if (xyz && cap >= n) {
        std::vector<double4> f(g->C.n_fw);
        g->fw.download(f.data(), g->C.n_fw);
        std::vector<double> x(s.n_guest), y(s.n_guest), z(s.n_guest);
        const size_t so = (size_t)chain * g->C.max_sites;
        ALEA_CUDA(cudaMemcpy(x.data(), g->gx.p + so, s.n_guest * 8, cudaMemcpyDeviceToHost));
        ALEA_CUDA(cudaMemcpy(y.data(), g->gy.p + so, s.n_guest * 8, cudaMemcpyDeviceToHost));
        ALEA_CUDA(cudaMemcpy(z.data(), g->gz.p + so, s.n_guest * 8, cudaMemcpyDeviceToHost));
        ALEA_CUDA(cudaDeviceSynchronize());
        for (uint64_t i = 0; i < g->C.n_fw; ++i) {
            xyz[3 * i] = f[i].x;
            xyz[3 * i + 1] = f[i].y;
            xyz[3 * i + 2] = f[i].z;
        }
        for (uint64_t i = 0; i < s.n_guest; ++i) {
            xyz[3 * (g->C.n_fw + i)] = x[i];
            xyz[3 * (g->C.n_fw + i) + 1] = y[i];
            xyz[3 * (g->C.n_fw + i) + 2] = z[i];
        }
    }
    return n;
}

// One chain's guest sites (engine order): x, y, z, charge and LJ species.
uint64_t gcmc_guest_sites(const GcmcImpl* g, uint32_t chain, double* xyzq, uint32_t* lj_species,
                          uint64_t cap) {
    require(chain < g->n_chains, ALEA_ERR_OUT_OF_RANGE, "GCMC: chain index");
    ChainState s;
    ALEA_CUDA(cudaMemcpy(&s, g->st.p + chain, sizeof s, cudaMemcpyDeviceToHost));
    const uint64_t n = s.n_guest;
    if (xyzq && lj_species && cap >= n && n > 0) {
        const size_t so = (size_t)chain * g->C.max_sites;
        std::vector<double> x(n), y(n), z(n), q(n);
        ALEA_CUDA(cudaMemcpy(x.data(), g->gx.p + so, n * 8, cudaMemcpyDeviceToHost));
        ALEA_CUDA(cudaMemcpy(y.data(), g->gy.p + so, n * 8, cudaMemcpyDeviceToHost));
        ALEA_CUDA(cudaMemcpy(z.data(), g->gz.p + so, n * 8, cudaMemcpyDeviceToHost));
        ALEA_CUDA(cudaMemcpy(q.data(), g->gq.p + so, n * 8, cudaMemcpyDeviceToHost));
        ALEA_CUDA(cudaMemcpy(lj_species, g->gt.p + so, n * 4, cudaMemcpyDeviceToHost));
        for (uint64_t i = 0; i < n; ++i) {
            xyzq[4 * i] = x[i];
            xyzq[4 * i + 1] = y[i];
            xyzq[4 * i + 2] = z[i];
            xyzq[4 * i + 3] = q[i];
        }
    }
    return n;
}

// committedEnergy() of one chain's cache (ewald_incremental_state.cc:85-93)
double gcmc_ewald_energy(const GcmcImpl* g, uint32_t chain) {
    require(chain < g->n_chains, ALEA_ERR_OUT_OF_RANGE, "GCMC: chain index");
    if (!g->C.charged) return 0.0;
    const uint64_t nk = g->C.nk;
    std::vector<double> re(nk), im(nk), w(nk);
    if (g->C.f32) {  // the FP32 form keeps S(k) as double-float
        std::vector<float2> hi(nk), lo(nk);
        ALEA_CUDA(cudaMemcpy(hi.data(), g->sk_hi.p + (size_t)chain * nk, nk * sizeof(float2),
                             cudaMemcpyDeviceToHost));
        ALEA_CUDA(cudaMemcpy(lo.data(), g->sk_lo.p + (size_t)chain * nk, nk * sizeof(float2),
                             cudaMemcpyDeviceToHost));
        for (uint64_t t = 0; t < nk; ++t) {
            re[t] = (double)hi[t].x + (double)lo[t].x;
            im[t] = (double)hi[t].y + (double)lo[t].y;
        }
    } else {
        ALEA_CUDA(cudaMemcpy(re.data(), g->sre.p + (size_t)chain * nk, nk * 8, cudaMemcpyDeviceToHost));
        ALEA_CUDA(cudaMemcpy(im.data(), g->sim.p + (size_t)chain * nk, nk * 8, cudaMemcpyDeviceToHost));
    }
    ALEA_CUDA(cudaMemcpy(w.data(), g->w.p, nk * 8, cudaMemcpyDeviceToHost));
    ChainState s;
    ALEA_CUDA(cudaMemcpy(&s, g->st.p + chain, sizeof s, cudaMemcpyDeviceToHost));
    double sum = 0.0;
    for (uint64_t t = 0; t < nk; ++t) sum += w[t] * (re[t] * re[t] + im[t] * im[t]);
    return sum * kCoulomb * (2.0 * kPi / g->C.volume) + s.self_e + s.excl_e;
}

// Insertions and deletions from now on use the tabulated proposal (its
// tables are copied), or the reference's uniform insertion when t is null.
void gcmc_set_proposal(GcmcImpl* g, const ProposalTable* t) {
    if (!t) {
        g->C.prop_cells = 0;
        return;
    }
    const uint64_t n = (uint64_t)t->cells * t->cells * t->cells;
    g->pcdf.alloc(n);
    g->plogp.alloc(n);
    ALEA_CUDA(cudaMemcpy(g->pcdf.p, t->cdf, n * sizeof(double), cudaMemcpyDeviceToDevice));
    ALEA_CUDA(cudaMemcpy(g->plogp.p, t->logp, n * sizeof(double), cudaMemcpyDeviceToDevice));
    ALEA_CUDA(cudaDeviceSynchronize());
    g->C.prop_cells = t->cells;
}

// The engine's frameworkEnergyGrid (borrowed: it must outlive the chains'
// runs), or none. Its cell must be the chains' and it must hold a table for
// every site's LJ species.
void gcmc_set_grid(GcmcImpl* g, const GridImpl* grid) {
    if (!grid) {
        g->C.grid = 0;
        return;
    }
    const GridView v0 = grid_view(grid, g->C.row_lj[0]);
    for (int i = 0; i < 9; ++i)
        require(v0.L.m[i] == g->C.L.m[i], ALEA_ERR_INVALID_ARGUMENT,
                "GCMC: the energy grid is for another cell");
    for (int r = 0; r < g->C.n_rows; ++r) g->gtab[r] = grid_view(grid, g->C.row_lj[r]).table;
    for (int a = 0; a < 3; ++a) g->C.gn[a] = v0.n[a];
    g->C.grid_fast = v0.fast;
    g->C.grid = 1;
}

// Orientation trials of insertions and deletions of multi-site molecules in
// the next runs (1: the reference's single random orientation).
void gcmc_set_orientation_trials(GcmcImpl* g, int k) {
    require(k >= 1 && k <= MAXCB, ALEA_ERR_INVALID_ARGUMENT,
            "GCMC: orientation trials must be 1.." + std::to_string(MAXCB));
    g->C.orient = k;
}

// Opt-in: insertions, deletions and swaps of the next runs add the change of
// the LJ tail correction (off: the reference engine's energies).
void gcmc_set_tail_correction(GcmcImpl* g, int on) { g->C.tail = on ? 1 : 0; }

// ALEA_FP64 (the parity form) or ALEA_FP32 for the next runs.
void gcmc_set_precision(GcmcImpl* g, int precision) {
    require(precision == ALEA_FP64 || precision == ALEA_FP32, ALEA_ERR_INVALID_ARGUMENT,
            "GCMC: precision must be ALEA_FP64 or ALEA_FP32");
    const int f32 = precision == ALEA_FP32;
    // the FP32 form lists near pairs as (atom << 8 | trial site) in 32 bits
    require(!f32 || g->C.n_fw + g->C.max_sites < (1ull << 24), ALEA_ERR_INVALID_ARGUMENT,
            "GCMC (FP32 form): framework atoms + max_molecules x sites must be below 2^24");
    const uint64_t n = g->C.nk * g->n_chains;
    if (f32 != g->C.f32 && g->C.charged && n) {  // carry the committed S(k) across
        convert_sk_kernel<<<(unsigned)((n + 255) / 256), 256>>>(n, f32, g->sre.p, g->sim.p,
                                                                g->sk_hi.p, g->sk_lo.p);
        ALEA_CUDA(cudaGetLastError());
        ALEA_CUDA(cudaDeviceSynchronize());
    }
    g->C.f32 = f32;
}

unsigned gcmc_chains(const GcmcImpl* g) { return g->n_chains; }
float gcmc_last_ms(const GcmcImpl* g) { return g->last_ms; }
void gcmc_destroy(GcmcImpl* g) { delete g; }

}  // namespace alea
