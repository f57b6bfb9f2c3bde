// Ewald summation on sm_103a: reciprocal-space term table, the incremental
// structure-factor cache (EwaldIncrementalState) in HBM, per-particle
// real-space energies and the full energy breakdown.
//
// References (forcefield/electrostatics/):
//   ewald.cc:29-45      reciprocal vectors b_i = 2 pi (a_j x a_k) / V
//   ewald.cc:137-161    spherical index set n != 0, |n|^2 < kMax^2 + 2 (n0, n1, n2 order)
//   ewald.cc:223-249    realSpaceParticleEnergy
//   ewald.cc:251-313    computeEnergyBreakdown
//   ewald_incremental_state.cc:55-257  the S(k) cache: ctor, committedEnergy,
//                       computeDelta/propose/commit, recompute, resync, raw state
//
// Layout in HBM: k (3 doubles per term), weight, (n0, n1, n2), and the
// committed sRe/sIm, one double each per term, in the reference's term order.
// Every per-term sum runs one thread per term; the scalar results are reduced
// per block in a fixed tree order and then across blocks in block order, so a
// call is deterministic.

#include <cmath>
#include <vector>

#include "common.cuh"
#include "grid.cuh"

namespace alea {

namespace {

constexpr int RT = 256;        // threads per block for the per-term kernels
constexpr int MAX_SITES = 64;  // sites per propose / commit call

struct Site {
    double x, y, z, q;
};

// Fixed-order block reduction of one double (RT threads).
__device__ double block_sum(double v, double* sh) {
    const int t = threadIdx.x;
    sh[t] = v;
    __syncthreads();
    for (int s = RT / 2; s > 0; s >>= 1) {
        if (t < s) sh[t] += sh[t + s];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

// ewald.cc:73-79 / ewald_incremental_state.cc:24-30
__device__ __forceinline__ double erf_over_r(double r, double alpha) {
    if (r < 1e-8) return 2.0 * alpha / sqrt(kPi);
    return erf(alpha * r) / r;
}

// ewald_incremental_state.cc:32-43 over one packed site list (device).
__device__ double pair_exclusion_sum(const Lattice& L, const Site* s, int n, double alpha) {
    double sum = 0.0;
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) {
            double dx, dy, dz;
            min_image(L, s[j].x - s[i].x, s[j].y - s[i].y, s[j].z - s[i].z, dx, dy, dz);
            const double r = sqrt(dx * dx + dy * dy + dz * dz);
            sum += s[i].q * s[j].q * erf_over_r(r, alpha);
        }
    return sum;
}

// computeDelta (ewald_incremental_state.cc:95-136), per term, plus the
// weighted |S|^2 change; apply = commit (S += delta) in the same pass.
__global__ void ews_delta_kernel(uint64_t nk, const double* __restrict__ k,
                                 const double* __restrict__ w, double* __restrict__ sre,
                                 double* __restrict__ sim, const Site* __restrict__ sites, int nr,
                                 int na, int apply, double* __restrict__ partial) {
    __shared__ Site s[MAX_SITES];
    __shared__ double sh[RT];
    const int n = nr + na;
    for (int i = threadIdx.x; i < n; i += RT) s[i] = sites[i];
    __syncthreads();
    double acc = 0.0;
    const uint64_t t = (uint64_t)blockIdx.x * RT + threadIdx.x;
    if (t < nk) {
        const double k0 = k[3 * t], k1 = k[3 * t + 1], k2 = k[3 * t + 2];
        double re = 0.0, im = 0.0;
        // added first, then removed (ewald_incremental_state.cc:107-116)
        for (int i = nr; i < n; ++i) {
            const double kr = k0 * s[i].x + k1 * s[i].y + k2 * s[i].z;
            double sn, cs;
            sincos(kr, &sn, &cs);
            re += s[i].q * cs;
            im += s[i].q * sn;
        }
        for (int i = 0; i < nr; ++i) {
            const double kr = k0 * s[i].x + k1 * s[i].y + k2 * s[i].z;
            double sn, cs;
            sincos(kr, &sn, &cs);
            re -= s[i].q * cs;
            im -= s[i].q * sn;
        }
        const double o_re = sre[t], o_im = sim[t];
        const double n_re = o_re + re, n_im = o_im + im;
        acc = w[t] * ((n_re * n_re + n_im * n_im) - (o_re * o_re + o_im * o_im));
        if (apply) {
            sre[t] = o_re + re;
            sim[t] = o_im + im;
        }
    }
    const double b = block_sum(acc, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = b;
}

// Sums per-block partials in block order and adds the self and exclusion
// parts of the delta. out = {reciprocal, self, exclusion, total}.
__global__ void ews_finish_kernel(const double* __restrict__ partial, int nblocks, Lattice L,
                                  double alpha, double rec_pref, const Site* __restrict__ sites,
                                  int nr, int na, double* __restrict__ out) {
    __shared__ double sh[RT];
    double acc = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += RT) acc += partial[i];
    const double sum = block_sum(acc, sh);
    if (threadIdx.x == 0) {
        __shared__ Site s[MAX_SITES];
        for (int i = 0; i < nr + na; ++i) s[i] = sites[i];
        double q2a = 0.0, q2r = 0.0;
        for (int i = nr; i < nr + na; ++i) q2a += s[i].q * s[i].q;
        for (int i = 0; i < nr; ++i) q2r += s[i].q * s[i].q;
        const double self_pref = -kCoulomb * (alpha / sqrt(kPi));
        const double self = self_pref * (q2a - q2r);
        const double ex = -kCoulomb * (pair_exclusion_sum(L, s + nr, na, alpha) -
                                       pair_exclusion_sum(L, s, nr, alpha));
        const double rec = rec_pref * sum;
        out[0] = rec;
        out[1] = self;
        out[2] = ex;
        out[3] = rec + self + ex;
    }
}

// S(k) = sum_i q_i (cos, sin)(k . r_i) for every term; particles staged in
// shared memory tiles (ewald_incremental_state.cc:64-76, 217-228).
__global__ void structure_factor_kernel(uint64_t nk, const double* __restrict__ k,
                                        const double4* __restrict__ p, uint64_t n,
                                        double* __restrict__ sre, double* __restrict__ sim) {
    __shared__ double4 tile[RT];
    const uint64_t t = (uint64_t)blockIdx.x * RT + threadIdx.x;
    double k0 = 0, k1 = 0, k2 = 0;
    if (t < nk) {
        k0 = k[3 * t];
        k1 = k[3 * t + 1];
        k2 = k[3 * t + 2];
    }
    double re = 0.0, im = 0.0;
    for (uint64_t base = 0; base < n; base += RT) {
        const uint64_t i = base + threadIdx.x;
        if (i < n) tile[threadIdx.x] = p[i];
        __syncthreads();
        const int cnt = (int)min((uint64_t)RT, n - base);
        if (t < nk) {
            for (int j = 0; j < cnt; ++j) {
                const double4 a = tile[j];
                const double kr = k0 * a.x + k1 * a.y + k2 * a.z;
                double sn, cs;
                sincos(kr, &sn, &cs);
                re += a.w * cs;
                im += a.w * sn;
            }
        }
        __syncthreads();
    }
    if (t < nk) {
        sre[t] = re;
        sim[t] = im;
    }
}

// sum_t w_t (sre_t^2 + sim_t^2) -> per-block partials
__global__ void weighted_mag_kernel(uint64_t nk, const double* __restrict__ w,
                                    const double* __restrict__ sre, const double* __restrict__ sim,
                                    double* __restrict__ partial) {
    __shared__ double sh[RT];
    const uint64_t t = (uint64_t)blockIdx.x * RT + threadIdx.x;
    double v = 0.0;
    if (t < nk) v = w[t] * (sre[t] * sre[t] + sim[t] * sim[t]);
    const double b = block_sum(v, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = b;
}

__global__ void sum_partials_kernel(const double* __restrict__ partial, int nblocks,
                                    double* __restrict__ out) {
    __shared__ double sh[RT];
    double acc = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += RT) acc += partial[i];
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) *out = s;
}

// sum of q^2 and the per-molecule exclusion sums (molecules as CSR)
__global__ void self_exclusion_kernel(const double4* __restrict__ p, uint64_t n,
                                      const uint64_t* __restrict__ offs,
                                      const uint64_t* __restrict__ idx, uint64_t n_mol, Lattice L,
                                      double alpha, double* __restrict__ out) {
    __shared__ double sh[RT];
    double q2 = 0.0;
    for (uint64_t i = threadIdx.x; i < n; i += RT) q2 += p[i].w * p[i].w;
    const double sq = block_sum(q2, sh);
    double ex = 0.0;
    for (uint64_t m = threadIdx.x; m < n_mol; m += RT) {
        const uint64_t b = offs[m], e = offs[m + 1];
        double s = 0.0;
        for (uint64_t i = b; i < e; ++i)
            for (uint64_t j = i + 1; j < e; ++j) {
                const double4 a = p[idx[i]], c = p[idx[j]];
                double dx, dy, dz;
                min_image(L, c.x - a.x, c.y - a.y, c.z - a.z, dx, dy, dz);
                s += a.w * c.w * erf_over_r(sqrt(dx * dx + dy * dy + dz * dz), alpha);
            }
        ex += s;
    }
    const double sex = block_sum(ex, sh);
    if (threadIdx.x == 0) {
        out[0] = sq;
        out[1] = sex;
    }
}

// realSpaceParticleEnergy (ewald.cc:223-249) for a batch of query indices.
__global__ void real_space_kernel(Lattice L, const double4* __restrict__ p, uint64_t n,
                                  const uint64_t* __restrict__ query, uint64_t nq,
                                  const uint64_t* __restrict__ excluded, int nex, double alpha,
                                  double rc, double* __restrict__ out) {
    const uint64_t qi = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= nq) return;
    const uint64_t i = query[qi];
    const double4 a = p[i];
    double e = 0.0;
    for (uint64_t j = 0; j < n; ++j) {
        if (j == i) continue;
        bool skip = false;
        for (int x = 0; x < nex; ++x) skip |= (excluded[x] == j);
        if (skip) continue;
        const double4 b = p[j];
        double dx, dy, dz;
        min_image(L, b.x - a.x, b.y - a.y, b.z - a.z, dx, dy, dz);
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        if (r > rc) continue;
        e += a.w * b.w * (erfc(alpha * r) / r);
    }
    out[qi] = e * kCoulomb;
}

// erfc(alpha r)/r for explicit pairs within rc (excluded pairs of the breakdown)
__global__ void pair_real_kernel(Lattice L, const double4* __restrict__ p,
                                 const uint64_t* __restrict__ pairs, uint64_t np, double alpha,
                                 double rc, double* __restrict__ real_out,
                                 double* __restrict__ excl_out) {
    const uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= np) return;
    const double4 a = p[pairs[2 * e]], b = p[pairs[2 * e + 1]];
    double dx, dy, dz;
    min_image(L, b.x - a.x, b.y - a.y, b.z - a.z, dx, dy, dz);
    const double r = sqrt(dx * dx + dy * dy + dz * dz);
    real_out[e] = r > rc ? 0.0 : a.w * b.w * (erfc(alpha * r) / r);
    excl_out[e] = a.w * b.w * erf_over_r(r, alpha);
}

std::vector<double4> pack(const alea_particles& p) {
    std::vector<double4> v(p.n);
    for (uint64_t i = 0; i < p.n; ++i)
        v[i] = make_double4(p.x[i], p.y[i], p.z[i], p.charge ? p.charge[i] : 0.0);
    return v;
}

void check_particles(const alea_particles& p, const char* what) {
    require(p.n == 0 || (p.x && p.y && p.z), ALEA_ERR_INVALID_ARGUMENT,
            std::string(what) + ": particle coordinates missing");
}

unsigned blocks_for(uint64_t n) { return (unsigned)std::max<uint64_t>(1, (n + RT - 1) / RT); }

}  // namespace

// buildReciprocalTerms (ewald.cc:137-161) in the reference's order, with the
// integer index triple of every term.
uint64_t ewald_terms_host(const Lattice& L, double alpha, int kmax, double* k, double* w,
                          int32_t* nidx, uint64_t cap) {
    const double* m = L.m;
    const double two_pi_over_v = 2.0 * kPi / L.volume;
    double b[3][3];
    for (int c = 0; c < 3; ++c) {
        b[0][c] = L.c12[c] * two_pi_over_v;
        b[1][c] = L.c20[c] * two_pi_over_v;
        b[2][c] = L.c01[c] * two_pi_over_v;
    }
    (void)m;
    const double four_a2 = 4.0 * alpha * alpha;
    const int bound = kmax * kmax + 2;
    uint64_t count = 0;
    for (int n0 = -kmax; n0 <= kmax; ++n0)
        for (int n1 = -kmax; n1 <= kmax; ++n1)
            for (int n2 = -kmax; n2 <= kmax; ++n2) {
                if (n0 == 0 && n1 == 0 && n2 == 0) continue;
                if (n0 * n0 + n1 * n1 + n2 * n2 >= bound) continue;
                if (count < cap) {
                    double kv[3];
                    for (int c = 0; c < 3; ++c)
                        kv[c] = (b[0][c] * (double)n0 + b[1][c] * (double)n1) + b[2][c] * (double)n2;
                    const double k2 = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
                    if (k) {
                        k[3 * count] = kv[0];
                        k[3 * count + 1] = kv[1];
                        k[3 * count + 2] = kv[2];
                    }
                    if (w) w[count] = std::exp(-k2 / four_a2) / k2;
                    if (nidx) {
                        nidx[3 * count] = n0;
                        nidx[3 * count + 1] = n1;
                        nidx[3 * count + 2] = n2;
                    }
                }
                ++count;
            }
    return count;
}

struct EwaldStateImpl {
    Lattice L{};
    double alpha = 0, rc = 0;
    int kmax = 0;
    uint64_t nk = 0;
    double volume = 0;
    DevBuf<double> k, w, sre, sim, partial, result;
    DevBuf<int32_t> nidx;
    DevBuf<Site> sites;
    double self_energy = 0, exclusion_energy = 0;
    double b[9];
};

static void ewald_validate(const alea_ewald& ew) {
    require(ew.alpha > 0.0, ALEA_ERR_INVALID_ARGUMENT, "Ewald: alpha must be positive");
    require(ew.real_space_cutoff > 0.0, ALEA_ERR_INVALID_ARGUMENT,
            "Ewald: realSpaceCutoff must be positive");
    require(ew.kmax >= 1, ALEA_ERR_INVALID_ARGUMENT, "Ewald: kMax must be at least 1");
}

// Structure factor of `p` into (sre, sim) of the state's terms.
static void structure_factor(const EwaldStateImpl& s, const alea_particles& p, double* sre,
                             double* sim) {
    const auto packed = pack(p);
    DevBuf<double4> dp(std::max<size_t>(packed.size(), 1));
    dp.upload(packed.data(), packed.size());
    if (s.nk)
        structure_factor_kernel<<<blocks_for(s.nk), RT>>>(s.nk, s.k.p, dp.p, p.n, sre, sim);
    ALEA_CUDA(cudaGetLastError());
    ALEA_CUDA(cudaDeviceSynchronize());
}

static double weighted_mag(const EwaldStateImpl& s, const double* sre, const double* sim) {
    if (s.nk == 0) return 0.0;
    const unsigned nb = blocks_for(s.nk);
    weighted_mag_kernel<<<nb, RT>>>(s.nk, s.w.p, sre, sim, s.partial.p);
    sum_partials_kernel<<<1, RT>>>(s.partial.p, (int)nb, s.result.p);
    ALEA_CUDA(cudaGetLastError());
    double out = 0;
    ALEA_CUDA(cudaMemcpy(&out, s.result.p, sizeof out, cudaMemcpyDeviceToHost));
    return out;
}

// (sum q^2, sum over molecules of pairExclusionSum)
static void self_and_exclusion(const EwaldStateImpl& s, const alea_particles& p, uint64_t n_mol,
                               const uint64_t* offsets, const uint64_t* indices, double* out2) {
    const auto packed = pack(p);
    DevBuf<double4> dp(std::max<size_t>(packed.size(), 1));
    dp.upload(packed.data(), packed.size());
    const uint64_t n_idx = n_mol ? offsets[n_mol] : 0;
    for (uint64_t i = 0; i < n_idx; ++i)
        require(indices[i] < p.n, ALEA_ERR_OUT_OF_RANGE, "EwaldIncrementalState: molecule index");
    DevBuf<uint64_t> doff(n_mol + 1), didx(std::max<uint64_t>(n_idx, 1));
    std::vector<uint64_t> offs(offsets ? offsets : nullptr, offsets ? offsets + n_mol + 1 : nullptr);
    if (offs.empty()) offs.push_back(0);
    doff.upload(offs.data(), offs.size());
    didx.upload(indices, n_idx);
    self_exclusion_kernel<<<1, RT>>>(dp.p, p.n, doff.p, didx.p, n_mol, s.L, s.alpha, s.result.p);
    ALEA_CUDA(cudaGetLastError());
    ALEA_CUDA(cudaMemcpy(out2, s.result.p, 2 * sizeof(double), cudaMemcpyDeviceToHost));
}

EwaldStateImpl* ewald_state_create(const alea_ewald& ew, const alea_particles& p,
                                   const alea_lattice& lat) {
    ewald_validate(ew);
    check_particles(p, "EwaldIncrementalState");
    make_lattice(lat.m);
    require_device();
    auto* s = new EwaldStateImpl();
    try {
        s->L = make_lattice(lat.m);
        s->alpha = ew.alpha;
        s->rc = ew.real_space_cutoff;
        s->kmax = ew.kmax;
        s->volume = std::fabs(s->L.volume);
        s->nk = ewald_terms_host(s->L, ew.alpha, ew.kmax, nullptr, nullptr, nullptr, 0);
        std::vector<double> k(3 * s->nk), w(s->nk);
        std::vector<int32_t> nidx(3 * s->nk);
        ewald_terms_host(s->L, ew.alpha, ew.kmax, k.data(), w.data(), nidx.data(), s->nk);
        const double tpv = 2.0 * kPi / s->L.volume;
        for (int c = 0; c < 3; ++c) {
            s->b[c] = s->L.c12[c] * tpv;
            s->b[3 + c] = s->L.c20[c] * tpv;
            s->b[6 + c] = s->L.c01[c] * tpv;
        }
        const size_t nk1 = std::max<uint64_t>(s->nk, 1);
        s->k.alloc(3 * nk1);
        s->w.alloc(nk1);
        s->nidx.alloc(3 * nk1);
        s->sre.alloc(nk1);
        s->sim.alloc(nk1);
        s->partial.alloc(blocks_for(s->nk));
        s->result.alloc(4);
        s->sites.alloc(MAX_SITES);
        s->k.upload(k.data(), k.size());
        s->w.upload(w.data(), w.size());
        s->nidx.upload(nidx.data(), nidx.size());
        structure_factor(*s, p, s->sre.p, s->sim.p);
        double se[2];
        self_and_exclusion(*s, p, 0, nullptr, nullptr, se);
        s->self_energy = -kCoulomb * (s->alpha / std::sqrt(kPi)) * se[0];
        s->exclusion_energy = 0.0;  // framework carries no exclusion (ewald_incremental_state.cc:82)
    } catch (...) {
        delete s;
        throw;
    }
    return s;
}

void ewald_state_destroy(EwaldStateImpl* s) { delete s; }

double ewald_state_energy(const EwaldStateImpl* s) {
    const double sum = weighted_mag(*s, s->sre.p, s->sim.p);
    const double reciprocal = sum * kCoulomb * (2.0 * kPi / s->volume);
    return reciprocal + s->self_energy + s->exclusion_energy;
}

static void delta(const EwaldStateImpl* s, const double* removed, uint64_t nr, const double* added,
                  uint64_t na, bool apply, double out[4]) {
    require(nr + na <= (uint64_t)MAX_SITES, ALEA_ERR_INVALID_ARGUMENT,
            "EwaldIncrementalState: at most 64 sites per trial");
    std::vector<Site> st(nr + na);
    for (uint64_t i = 0; i < nr; ++i)
        st[i] = Site{removed[4 * i], removed[4 * i + 1], removed[4 * i + 2], removed[4 * i + 3]};
    for (uint64_t i = 0; i < na; ++i)
        st[nr + i] = Site{added[4 * i], added[4 * i + 1], added[4 * i + 2], added[4 * i + 3]};
    auto* ms = const_cast<EwaldStateImpl*>(s);
    ms->sites.upload(st.data(), st.size());
    const unsigned nb = blocks_for(s->nk);
    if (s->nk)
        ews_delta_kernel<<<nb, RT>>>(s->nk, s->k.p, s->w.p, ms->sre.p, ms->sim.p, s->sites.p,
                                     (int)nr, (int)na, apply ? 1 : 0, ms->partial.p);
    else
        ALEA_CUDA(cudaMemset(ms->partial.p, 0, sizeof(double)));
    ews_finish_kernel<<<1, RT>>>(s->partial.p, s->nk ? (int)nb : 1, s->L, s->alpha,
                                 kCoulomb * (2.0 * kPi / s->volume), s->sites.p, (int)nr, (int)na,
                                 ms->result.p);
    ALEA_CUDA(cudaGetLastError());
    ALEA_CUDA(cudaMemcpy(out, s->result.p, 4 * sizeof(double), cudaMemcpyDeviceToHost));
}

double ewald_state_propose(const EwaldStateImpl* s, const double* removed, uint64_t nr,
                           const double* added, uint64_t na) {
    double out[4];
    delta(s, removed, nr, added, na, false, out);
    return out[3];
}

void ewald_state_commit(EwaldStateImpl* s, const double* removed, uint64_t nr, const double* added,
                        uint64_t na) {
    double out[4];
    delta(s, removed, nr, added, na, true, out);
    s->self_energy += out[1];
    s->exclusion_energy += out[2];
}

double ewald_state_recompute(const EwaldStateImpl* s, const alea_particles& p, uint64_t n_mol,
                             const uint64_t* offsets, const uint64_t* indices) {
    check_particles(p, "recomputeFromScratch");
    DevBuf<double> re(std::max<uint64_t>(s->nk, 1)), im(std::max<uint64_t>(s->nk, 1));
    structure_factor(*s, p, re.p, im.p);
    const double rsum = weighted_mag(*s, re.p, im.p);
    const double reciprocal = rsum * kCoulomb * (2.0 * kPi / s->volume);
    double se[2];
    self_and_exclusion(*s, p, n_mol, offsets, indices, se);
    const double self = -kCoulomb * (s->alpha / std::sqrt(kPi)) * se[0];
    const double exclusion = -kCoulomb * se[1];
    return reciprocal + self + exclusion;
}

void ewald_state_resync(EwaldStateImpl* s, const alea_particles& p, uint64_t n_mol,
                        const uint64_t* offsets, const uint64_t* indices) {
    check_particles(p, "resync");
    structure_factor(*s, p, s->sre.p, s->sim.p);
    double se[2];
    self_and_exclusion(*s, p, n_mol, offsets, indices, se);
    s->self_energy = -kCoulomb * (s->alpha / std::sqrt(kPi)) * se[0];
    s->exclusion_energy = -kCoulomb * se[1];
}

std::vector<double> ewald_state_raw(const EwaldStateImpl* s) {
    std::vector<double> raw(2 * s->nk + 2);
    s->sre.download(raw.data(), s->nk);
    s->sim.download(raw.data() + s->nk, s->nk);
    ALEA_CUDA(cudaDeviceSynchronize());
    raw[2 * s->nk] = s->self_energy;
    raw[2 * s->nk + 1] = s->exclusion_energy;
    return raw;
}

uint64_t ewald_state_nk(const EwaldStateImpl* s) { return s->nk; }

EwaldDeviceView ewald_state_view(const EwaldStateImpl* s) {
    EwaldDeviceView v{};
    v.nk = s->nk;
    v.k = s->k.p;
    v.w = s->w.p;
    v.sre = s->sre.p;
    v.sim = s->sim.p;
    v.nidx = s->nidx.p;
    v.alpha = s->alpha;
    v.volume = s->volume;
    v.self_pref = -kCoulomb * (s->alpha / std::sqrt(kPi));
    v.rec_pref = kCoulomb * (2.0 * kPi / s->volume);
    v.kmax = s->kmax;
    for (int i = 0; i < 9; ++i) v.b[i] = s->b[i];
    return v;
}

void ewald_real_space_particle_energy(const alea_ewald& ew, const alea_particles& p,
                                      const alea_lattice& lat, const uint64_t* query, uint64_t nq,
                                      const uint64_t* excluded, uint64_t nex, double* out) {
    require(ew.real_space_cutoff > 0.0, ALEA_ERR_INVALID_ARGUMENT,
            "Ewald: realSpaceCutoff must be positive");
    check_particles(p, "realSpaceParticleEnergy");
    const Lattice L = make_lattice(lat.m);
    validate_cutoff(L, ew.real_space_cutoff, "Ewald::realSpaceParticleEnergy");
    for (uint64_t i = 0; i < nq; ++i)
        require(query[i] < p.n, ALEA_ERR_OUT_OF_RANGE, "realSpaceParticleEnergy: index out of range");
    require(nex <= 1024, ALEA_ERR_INVALID_ARGUMENT, "realSpaceParticleEnergy: at most 1024 excluded");
    if (nq == 0) return;
    require_device();
    const auto packed = pack(p);
    DevBuf<double4> dp(std::max<size_t>(packed.size(), 1));
    dp.upload(packed.data(), packed.size());
    DevBuf<uint64_t> dq(nq), dx(std::max<uint64_t>(nex, 1));
    DevBuf<double> dout(nq);
    dq.upload(query, nq);
    dx.upload(excluded, nex);
    real_space_kernel<<<(unsigned)((nq + 127) / 128), 128>>>(L, dp.p, p.n, dq.p, nq, dx.p, (int)nex,
                                                             ew.alpha, ew.real_space_cutoff, dout.p);
    ALEA_CUDA(cudaGetLastError());
    dout.download(out, nq);
    ALEA_CUDA(cudaDeviceSynchronize());
}

// computeEnergyBreakdown (ewald.cc:251-313): real space as half the sum of the
// per-particle sums minus the excluded pairs; reciprocal from S(k); self;
// exclusion over the listed pairs; surface 0 (tinfoil).
void ewald_breakdown(const alea_ewald& ew, const alea_particles& p, const alea_lattice& lat,
                     const uint64_t* excl, uint64_t n_excl, double* out) {
    ewald_validate(ew);
    check_particles(p, "Ewald::computeEnergyBreakdown");
    double qsum = 0.0;
    for (uint64_t i = 0; i < p.n; ++i) qsum += p.charge ? p.charge[i] : 0.0;
    if (std::fabs(qsum) > 1e-8)  // ewald.cc:181-195
        throw Error(ALEA_ERR_INVALID_ARGUMENT,
                    "Ewald: system is not charge-neutral (total charge = " + std::to_string(qsum) +
                        " e); the reciprocal-space k=0 term is only well-defined for a neutral system");
    for (uint64_t e = 0; e < 2 * n_excl; ++e)
        require(excl[e] < p.n, ALEA_ERR_OUT_OF_RANGE, "Ewald: exclusion index out of range");
    validate_cutoff(make_lattice(lat.m), ew.real_space_cutoff, "Ewald::computeEnergyBreakdown");
    require_device();
    EwaldStateImpl* s = ewald_state_create(ew, p, lat);
    try {
        std::vector<uint64_t> all(p.n);
        for (uint64_t i = 0; i < p.n; ++i) all[i] = i;
        std::vector<double> per(p.n);
        ewald_real_space_particle_energy(ew, p, lat, all.data(), p.n, nullptr, 0, per.data());
        // Real space: per-particle sums are computed on the device; the N
        // results are combined here in index order.
        double real = 0.0;
        for (double v : per) real += v;
        real *= 0.5;
        double excl_real = 0.0, excl_erf = 0.0;
        if (n_excl) {
            const auto packed = pack(p);
            DevBuf<double4> dp(packed.size());
            dp.upload(packed.data(), packed.size());
            DevBuf<uint64_t> dpairs(2 * n_excl);
            dpairs.upload(excl, 2 * n_excl);
            DevBuf<double> dr(n_excl), de(n_excl);
            pair_real_kernel<<<(unsigned)((n_excl + 127) / 128), 128>>>(
                s->L, dp.p, dpairs.p, n_excl, ew.alpha, ew.real_space_cutoff, dr.p, de.p);
            ALEA_CUDA(cudaGetLastError());
            std::vector<double> hr(n_excl), he(n_excl);
            dr.download(hr.data(), n_excl);
            de.download(he.data(), n_excl);
            ALEA_CUDA(cudaDeviceSynchronize());
            for (uint64_t e = 0; e < n_excl; ++e) {
                excl_real += hr[e];
                excl_erf += he[e];
            }
        }
        out[0] = real - excl_real * kCoulomb;
        const double sum = weighted_mag(*s, s->sre.p, s->sim.p);
        out[1] = sum * kCoulomb * (2.0 * kPi / s->volume);
        out[2] = s->self_energy;
        out[3] = -excl_erf * kCoulomb;
        out[4] = 0.0;
    } catch (...) {
        ewald_state_destroy(s);
        throw;
    }
    ewald_state_destroy(s);
}

}  // namespace alea
