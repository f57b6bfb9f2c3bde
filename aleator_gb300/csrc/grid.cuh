// Internal declarations shared between the kernels and the C-ABI layer.
#pragma once

#include <vector>

#include "common.cuh"
#include "ff.cuh"

namespace alea {

struct GridImpl;
GridImpl* grid_build(const alea_lennard_jones& lj, const alea_particles& fw,
                     const alea_lattice& lat, const uint32_t* guest, uint32_t n_guest,
                     double spacing, int precision);
GridImpl* grid_from_tables(const alea_lattice& lat, double spacing, const int32_t counts[3],
                           const std::vector<uint32_t>& species,
                           const std::vector<std::vector<double>>& tables);
void grid_rebuild(GridImpl* g, cudaStream_t s);
// grid_build whose tables are also copied into host[k] (one array per entry of
// guest, nodes long; pinned memory lets the copies overlap the build).
GridImpl* grid_build_to_host(const alea_lennard_jones& lj, const alea_particles& fw,
                             const alea_lattice& lat, const uint32_t* guest, uint32_t n_guest,
                             double spacing, int precision, double* const* host);
void grid_destroy(GridImpl* g);
const double* grid_table(const GridImpl* g, uint32_t species);
void grid_interpolate_device(const GridImpl* g, uint32_t species, const double* xyz, uint64_t n,
                             double* out, cudaStream_t s);
void grid_interpolate_host(const GridImpl* g, uint32_t species, const double* xyz, uint64_t n,
                           double* out);
void grid_download(const GridImpl* g, uint32_t species, double* out, uint64_t n);
void grid_counts(const GridImpl* g, int32_t* out);
double grid_spacing(const GridImpl* g);
const std::vector<uint32_t>& grid_species(const GridImpl* g);
void grid_stats(const GridImpl* g, alea_grid_stats* out);

// FrameworkEnergyGrid::interpolate (framework_energy_grid.cc:251-288) at one
// point, in the reference's operation order: the fractional transform by the
// cross products over the volume (IEEE divisions), wrap, floor, then x-, y-
// and z-lerps without fused multiply-adds, so the value equals the
// reference's bit for bit on the same table.
__device__ __forceinline__ double grid_interp_ref(const Lattice& L, int nx, int ny, int nz,
                                                  const double* __restrict__ table, double px,
                                                  double py, double pz) {
    double f[3];
    f[0] = __ddiv_rn(dot_rn(L.c12, px, py, pz), L.volume);
    f[1] = __ddiv_rn(dot_rn(L.c20, px, py, pz), L.volume);
    f[2] = __ddiv_rn(dot_rn(L.c01, px, py, pz), L.volume);
    const int cnt[3] = {nx, ny, nz};
    int i0[3], i1[3];
    double t[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        f[a] = sub_rn(f[a], floor(f[a]));
        const double g = mul_rn(f[a], (double)cnt[a]);
        const int base = (int)floor(g);
        t[a] = sub_rn(g, (double)base);
        const int w = ((base % cnt[a]) + cnt[a]) % cnt[a];
        i0[a] = w;
        i1[a] = (w + 1) % cnt[a];
    }
    auto V = [&](int ix, int iy, int iz) {
        return __ldg(&table[((size_t)iz * ny + iy) * nx + ix]);
    };
    const double u0 = sub_rn(1.0, t[0]);
    const double c00 = add_rn(mul_rn(V(i0[0], i0[1], i0[2]), u0), mul_rn(V(i1[0], i0[1], i0[2]), t[0]));
    const double c10 = add_rn(mul_rn(V(i0[0], i1[1], i0[2]), u0), mul_rn(V(i1[0], i1[1], i0[2]), t[0]));
    const double c01 = add_rn(mul_rn(V(i0[0], i0[1], i1[2]), u0), mul_rn(V(i1[0], i0[1], i1[2]), t[0]));
    const double c11 = add_rn(mul_rn(V(i0[0], i1[1], i1[2]), u0), mul_rn(V(i1[0], i1[1], i1[2]), t[0]));
    const double u1 = sub_rn(1.0, t[1]);
    const double c0 = add_rn(mul_rn(c00, u1), mul_rn(c10, t[1]));
    const double c1 = add_rn(mul_rn(c01, u1), mul_rn(c11, t[1]));
    return add_rn(mul_rn(c0, sub_rn(1.0, t[2])), mul_rn(c1, t[2]));
}

// The same interpolation for grids built in the FP32 form: multiplies by the
// inverse cell (no IEEE divisions) and fused lerps, about 40 FP64 operations
// instead of about 100, within ~1e-12 relative of the reference order.
__device__ __forceinline__ double grid_interp_fast(const Lattice& L, int nx, int ny, int nz,
                                                   const double* __restrict__ table, double px,
                                                   double py, double pz) {
    const int cnt[3] = {nx, ny, nz};
    int i0[3], i1[3];
    double t[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        double f = fma(px, L.inv[a], fma(py, L.inv[3 + a], pz * L.inv[6 + a]));
        f -= floor(f);
        const double g = f * (double)cnt[a];
        int base = (int)g;  // g >= 0
        t[a] = g - (double)base;
        if (base >= cnt[a]) base -= cnt[a];  // f rounded up to 1
        base = min(max(base, 0), cnt[a] - 1);  // NaN or infinite positions
        i0[a] = base;
        i1[a] = base + 1 == cnt[a] ? 0 : base + 1;
    }
    auto V = [&](int ix, int iy, int iz) {
        return __ldg(&table[((size_t)iz * ny + iy) * nx + ix]);
    };
    auto lerp = [](double a, double b, double w) { return fma(w, b - a, a); };
    const double c00 = lerp(V(i0[0], i0[1], i0[2]), V(i1[0], i0[1], i0[2]), t[0]);
    const double c10 = lerp(V(i0[0], i1[1], i0[2]), V(i1[0], i1[1], i0[2]), t[0]);
    const double c01 = lerp(V(i0[0], i0[1], i1[2]), V(i1[0], i0[1], i1[2]), t[0]);
    const double c11 = lerp(V(i0[0], i1[1], i1[2]), V(i1[0], i1[1], i1[2]), t[0]);
    return lerp(lerp(c00, c10, t[1]), lerp(c01, c11, t[1]), t[2]);
}

// hi + lo split of a double with integer operations only (no FP64
// instruction): hi keeps the top 24 significant bits, lo the next 29 rounded
// to 24, so hi + lo carries ~48 bits. False for subnormals and magnitudes
// outside [2^-60, 2^100], which the caller handles in FP64; zero splits exactly.
__device__ __forceinline__ bool ff_split_bits(double v, ff& out) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const int e = (int)((b >> 52) & 0x7ffu);
    const unsigned long long m = b & 0xfffffffffffffull;
    if (e == 0) {
        out = ff{__uint_as_float(sign), 0.f};
        return m == 0;
    }
    const int ue = e - 1023;
    if (ue < -60 || ue > 100) return false;
    const float hi = __uint_as_float(sign | ((unsigned)(ue + 127) << 23) | (unsigned)(m >> 29));
    const float scale = __uint_as_float((unsigned)(ue - 52 + 127) << 23);  // 2^(ue - 52)
    const float lo = __uint_as_float(
        __float_as_uint(__fmul_rn(__uint2float_rn((unsigned)(m & 0x1fffffffu)), scale)) | sign);
    out = ff_fast(hi, lo);
    return true;
}

// floor of a normalised double-float value with |hi| < 2^22 (so |lo| < 1/4)
__device__ __forceinline__ float ff_floor(ff v) {
    float f = floorf(v.hi);
    if (v.hi == f && v.lo < 0.f) f -= 1.f;
    return f;
}

// The inverse cell (f = c . inv) as double-float.
struct InvFF {
    float h[9], l[9];
};

// FP32-form grids: grid_interp_fast's fractional transform, wrap and
// trilinear weights in double-float on the FP32 pipe, in two steps so that a
// kernel can issue the eight corner loads between them. The position and the
// corners are split by integer operations, so FP64 runs only to form the
// result; a query whose operands fall outside the split's range (either step
// returns false) is answered by grid_interp_fast. Agrees with
// grid_interp_fast to ~48 bits of the position and of the corners.
//
// Step 1: the lower corner (i0), the upper one with wrap (i1) and the weights.
__device__ __forceinline__ bool grid_ff_locate(const InvFF& inv, const int* cnt, double px,
                                               double py, double pz, int* i0, int* i1, ff* t) {
    ff p[3];
    if (!ff_split_bits(px, p[0]) || !ff_split_bits(py, p[1]) || !ff_split_bits(pz, p[2]))
        return false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        ff f = ff_add(ff_add(ff_mul(p[0], ff{inv.h[a], inv.l[a]}), ff_mul(p[1], ff{inv.h[3 + a], inv.l[3 + a]})),
                      ff_mul(p[2], ff{inv.h[6 + a], inv.l[6 + a]}));
        // ff_floor needs |lo| < 1: beyond 2^22 cells the image is answered in FP64
        if (!(fabsf(f.hi) < 4194304.f)) return false;
        f = ff_add_f(f, -ff_floor(f));  // [0, 1)
        const ff g = ff_mul(f, ff{(float)cnt[a], 0.f});
        const float fb = ff_floor(g);
        t[a] = ff_add_f(g, -fb);
        int base = (int)fb;
        if (base >= cnt[a]) base -= cnt[a];
        base = min(max(base, 0), cnt[a] - 1);  // in range whatever the rounding
        i0[a] = base;
        i1[a] = base + 1 == cnt[a] ? 0 : base + 1;
    }
    return true;
}

// Step 2: the trilinear blend of the corners c[k] (k = x + 2y + 4z, 0 lower,
// 1 upper), the same lerp order as grid_interp_fast.
__device__ __forceinline__ bool grid_ff_blend(const double* c, const ff* t, double& out) {
    ff v[8];
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 8; ++k) ok &= ff_split_bits(c[k], v[k]);
    if (!ok) return false;
    auto lerp = [](ff a, ff b, ff w) { return ff_add(a, ff_mul(w, ff_add(b, ff{-a.hi, -a.lo}))); };
    const ff c00 = lerp(v[0], v[1], t[0]), c10 = lerp(v[2], v[3], t[0]);
    const ff c01 = lerp(v[4], v[5], t[0]), c11 = lerp(v[6], v[7], t[0]);
    const ff r = lerp(lerp(c00, c10, t[1]), lerp(c01, c11, t[1]), t[2]);
    out = (double)r.hi + (double)r.lo;
    return true;
}

// One species' table of a grid, for kernels that interpolate it.
struct GridView {
    Lattice L;
    int n[3];
    const double* table;
    int fast;  // built in the FP32 form: grid_interp_fast
};
GridView grid_view(const GridImpl* g, uint32_t species);

struct GridBatchImpl;
GridBatchImpl* grid_batch_create(uint32_t n, const alea_lennard_jones* lj, const alea_particles* fw,
                                 const alea_lattice* lat, const uint32_t* guests, uint32_t n_guest,
                                 double spacing);
void grid_batch_build(GridBatchImpl* b, cudaStream_t s);
void grid_batch_stats(const GridBatchImpl* b, alea_grid_batch_stats* out);
const GridImpl* grid_batch_item(const GridBatchImpl* b, uint32_t i);
void grid_batch_destroy(GridBatchImpl* b);

// Test support: the tile-wait poll limit of the next FP32-form build (< 0: none).
void grid_test_set_tile_wait_limit(int64_t limit);

// grid_cache.cpp: the reference's on-disk cache format (version 1).
void grid_cache_write(const char* path, const alea_lennard_jones& lj, const alea_particles& fw,
                      const alea_lattice& lat, const uint32_t* guest, uint32_t n_guest,
                      double spacing, const int32_t counts[3], const std::vector<uint32_t>& species,
                      const std::vector<std::vector<double>>& tables);
std::string grid_cache_file_name(const alea_lennard_jones& lj, const alea_particles& fw,
                                 const alea_lattice& lat, const uint32_t* guest, uint32_t n_guest,
                                 double spacing);
// cacheHit: false on a plain miss; throws Error(ALEA_ERR_RUNTIME) when a file at
// the key's path has another version or stored key. Host only.
bool grid_cache_hit(const char* dir, const alea_lennard_jones& lj, const alea_particles& fw,
                    const alea_lattice& lat, const uint32_t* guest, uint32_t n_guest,
                    double spacing);
// Returns false on a plain miss; throws Error(ALEA_ERR_RUNTIME) on a bad file.
bool grid_cache_read(const char* dir, const alea_lennard_jones& lj, const alea_particles& fw,
                     const alea_lattice& lat, const uint32_t* guest, uint32_t n_guest,
                     double spacing, int32_t counts[3], std::vector<uint32_t>& species,
                     std::vector<std::vector<double>>& tables);

// philox.cu
void philox_raw(const uint32_t* ctr, const uint32_t* key, uint32_t* out, uint64_t n);
void philox_fill_u64_device(uint64_t seed, uint64_t stream, uint64_t first, uint64_t n,
                            uint64_t* out, cudaStream_t s);
void philox_fill_uniform_device(uint64_t seed, uint64_t stream, uint64_t first, uint64_t n,
                                double* out, cudaStream_t s);

// lj.cu / ewald.cu
void lj_particle_energy(const alea_lennard_jones& lj, const alea_particles& p,
                        const alea_lattice& lat, const uint64_t* query, uint64_t nq,
                        const uint64_t* excluded, uint64_t nex, double* out);
void ewald_real_space_particle_energy(const alea_ewald& ew, const alea_particles& p,
                                      const alea_lattice& lat, const uint64_t* query, uint64_t nq,
                                      const uint64_t* excluded, uint64_t nex, double* out);
void ewald_breakdown(const alea_ewald& ew, const alea_particles& p, const alea_lattice& lat,
                     const uint64_t* excl, uint64_t n_excl, double* out);
uint64_t ewald_terms_host(const Lattice& L, double alpha, int kmax, double* k, double* w,
                          int32_t* nidx, uint64_t cap);

struct EwaldStateImpl;
EwaldStateImpl* ewald_state_create(const alea_ewald& ew, const alea_particles& p,
                                   const alea_lattice& lat);
void ewald_state_destroy(EwaldStateImpl* s);
double ewald_state_energy(const EwaldStateImpl* s);
double ewald_state_propose(const EwaldStateImpl* s, const double* removed, uint64_t nr,
                           const double* added, uint64_t na);
void ewald_state_commit(EwaldStateImpl* s, const double* removed, uint64_t nr, const double* added,
                        uint64_t na);
double ewald_state_recompute(const EwaldStateImpl* s, const alea_particles& p, uint64_t n_mol,
                             const uint64_t* offsets, const uint64_t* indices);
void ewald_state_resync(EwaldStateImpl* s, const alea_particles& p, uint64_t n_mol,
                        const uint64_t* offsets, const uint64_t* indices);
std::vector<double> ewald_state_raw(const EwaldStateImpl* s);
uint64_t ewald_state_nk(const EwaldStateImpl* s);
// Device views for kernels that read the committed cache (Widom).
struct EwaldDeviceView {
    uint64_t nk;
    const double* k;     // 3 per term
    const double* w;
    const double* sre;
    const double* sim;
    const int32_t* nidx; // (n0, n1, n2) per term
    double alpha;
    double volume;
    double self_pref;    // -kC * alpha / sqrt(pi)
    double rec_pref;     // kC * 2 pi / V
    int kmax;
    double b[9];         // reciprocal vectors (rows)
};
EwaldDeviceView ewald_state_view(const EwaldStateImpl* s);

// proposal.cu: the learned insertion proposal and its tabulated density
struct ProposalImpl;
struct ProposalTable {
    int cells;          // per axis; cell c = (iz cells + iy) cells + ix
    const double* cdf;  // cumulative cell probabilities (device), last = 1
    const double* logp; // log of the cell density relative to uniform (device)
};
ProposalImpl* proposal_create(const alea_proposal_config& c);
void proposal_destroy(ProposalImpl* P);
uint64_t proposal_param_count(const ProposalImpl* P);
const std::vector<int32_t>& proposal_wave_vectors(const ProposalImpl* P);
void proposal_get_params(const ProposalImpl* P, float* out);
void proposal_set_params(ProposalImpl* P, const float* in);
void proposal_forward_host(ProposalImpl* P, const float* s, uint64_t n, float* out);
double proposal_loss_grad_host(ProposalImpl* P, const float* samples, uint64_t n, double tau,
                               float* grad);
double proposal_train(ProposalImpl* P, const float* samples_dev, uint64_t pool,
                      const alea_proposal_train_config& c, cudaStream_t s);
void proposal_tabulate(ProposalImpl* P, uint32_t cells, double uniform_share);
ProposalTable proposal_table(const ProposalImpl* P);
double proposal_log_density_host(const ProposalImpl* P, const double* s);

// widom.cu
struct WidomImpl;
WidomImpl* widom_create(const alea_lennard_jones& lj, const alea_ewald* ew,
                        const alea_particles& fw, const alea_lattice& lat,
                        const alea_molecule_species& guest, double temperature, int precision);
void widom_run(WidomImpl* w, uint64_t seed, uint64_t stream, uint64_t first, uint64_t n,
               int draw_order, alea_widom_result* out, double* per_trial,
               const ProposalTable* proposal = nullptr, double* per_trial_frac = nullptr);
// Trials as training rows {s0, s1, s2, -dU/T, lq} (device): uniform when
// proposal is null (lq = 0), else drawn from the proposal (lq = log density).
void widom_samples(WidomImpl* w, uint64_t seed, uint64_t stream, uint64_t first, uint64_t n,
                   int draw_order, float* samples_dev, const ProposalTable* proposal);
void widom_destroy(WidomImpl* w);
void widom_set_tail_correction(WidomImpl* w, int on);
double widom_tail_change(const WidomImpl* w);
struct WidomBatchImpl;
WidomBatchImpl* widom_batch_create(uint32_t n, const alea_lennard_jones* lj, const alea_ewald* ew,
                                   const alea_particles* fw, const alea_lattice* lat,
                                   const alea_molecule_species* guest, double temperature,
                                   int precision);
void widom_batch_run(WidomBatchImpl* b, const uint64_t* seeds, const uint64_t* streams,
                     uint64_t first, uint64_t n, int draw_order, alea_widom_result* out,
                     cudaStream_t s);
void widom_batch_destroy(WidomBatchImpl* b);

// gcmc.cu
struct GcmcImpl;
struct ChainState;
GcmcImpl* gcmc_create(const alea_lennard_jones& lj, const alea_ewald* ew, const alea_particles& fw,
                      const alea_lattice& lat, uint32_t n_species, const alea_molecule_species* guests,
                      double temperature, const double* fugacity_pa, const uint64_t* seeds,
                      const uint64_t* streams, uint32_t n_chains, double max_translation,
                      double max_rotation, int draw_order, uint32_t max_molecules);
void gcmc_run(GcmcImpl* g, uint64_t steps, cudaStream_t s);
void gcmc_states(const GcmcImpl* g, ChainState* out);
uint64_t gcmc_particles(const GcmcImpl* g, uint32_t chain, double* xyz, uint64_t cap);
uint64_t gcmc_guest_sites(const GcmcImpl* g, uint32_t chain, double* xyzq, uint32_t* lj_species,
                          uint64_t cap);
double gcmc_ewald_energy(const GcmcImpl* g, uint32_t chain);
void gcmc_set_proposal(GcmcImpl* g, const ProposalTable* t);
void gcmc_set_precision(GcmcImpl* g, int precision);
void gcmc_set_grid(GcmcImpl* g, const GridImpl* grid);
void gcmc_set_tail_correction(GcmcImpl* g, int on);
void gcmc_set_orientation_trials(GcmcImpl* g, int k);
unsigned gcmc_chains(const GcmcImpl* g);
float gcmc_last_ms(const GcmcImpl* g);
void gcmc_destroy(GcmcImpl* g);

}  // namespace alea
