// Allocation-free form of the Ewald structure-factor propose delta.
//
// Some callers cannot let a library allocate device memory: an engine that
// carves every device buffer out of its own pre-reserved pool (so a hidden
// cudaMalloc would break its memory budget), or one that cannot afford the
// device-wide synchronisation cudaMalloc/cudaFree can imply while other
// streams are busy. alea_ewald_propose_no_alloc serves them: the caller owns
// every input and output buffer, the trial sites travel as kernel parameters,
// and the per-block partial sums live in a file-scope __device__ array of a
// fixed size (below), held by every GPU that loads this library until the
// process exits. Nothing here calls cudaMalloc, cudaFree or any allocating
// library routine.
//
// Set-up: the first call on each device (with that device current) looks up
// the array's device address with cudaGetSymbolAddress and caches it; that
// first call should therefore come before any stream capture. All calls share
// the one array and it keeps the last call's contents; every slot a call reads
// is written earlier in the same call, so nothing needs clearing between calls.
// Calls that overlap on the GPU (different streams, or different host threads)
// race on the array: serialise them.

#include <cmath>
#include <mutex>

#include "common.cuh"

namespace alea {
namespace {

constexpr int NA_THREADS = 256;
constexpr uint64_t NA_MAX_TERMS = 262144;                 // reciprocal terms per call
constexpr int NA_MAX_BLOCKS = (int)(NA_MAX_TERMS / NA_THREADS);
constexpr int NA_MAX_SITES = 64;                          // removed + added sites

struct NaSites {
    double x[NA_MAX_SITES], y[NA_MAX_SITES], z[NA_MAX_SITES], q[NA_MAX_SITES];
    int nr, na;
};

// The scratch: per-block partial sums of the weighted |S|^2 change.
static __device__ __align__(256) double g_noalloc_partial[NA_MAX_BLOCKS];

__device__ double na_block_sum(double v, double* sh) {
    const int t = threadIdx.x;
    sh[t] = v;
    __syncthreads();
    for (int s = NA_THREADS / 2; s > 0; s >>= 1) {
        if (t < s) sh[t] += sh[t + s];
        __syncthreads();
    }
    return sh[0];
}

// computeDelta's per-term loop (ewald_incremental_state.cc:95-125): added
// sites first, then removed, never touching the committed cache.
__global__ void na_delta_kernel(uint64_t nk, const double* __restrict__ k,
                                const double* __restrict__ w, const double* __restrict__ sre,
                                const double* __restrict__ sim, const NaSites s,
                                double* __restrict__ partial) {
    __shared__ double sh[NA_THREADS];
    const uint64_t t = (uint64_t)blockIdx.x * NA_THREADS + threadIdx.x;
    double acc = 0.0;
    if (t < nk) {
        const double k0 = k[3 * t], k1 = k[3 * t + 1], k2 = k[3 * t + 2];
        double re = 0.0, im = 0.0;
        const int n = s.nr + s.na;
        for (int i = s.nr; i < n; ++i) {
            double sn, cs;
            sincos(k0 * s.x[i] + k1 * s.y[i] + k2 * s.z[i], &sn, &cs);
            re += s.q[i] * cs;
            im += s.q[i] * sn;
        }
        for (int i = 0; i < s.nr; ++i) {
            double sn, cs;
            sincos(k0 * s.x[i] + k1 * s.y[i] + k2 * s.z[i], &sn, &cs);
            re -= s.q[i] * cs;
            im -= s.q[i] * sn;
        }
        const double o_re = sre[t], o_im = sim[t];
        const double n_re = o_re + re, n_im = o_im + im;
        acc = w[t] * ((n_re * n_re + n_im * n_im) - (o_re * o_re + o_im * o_im));
    }
    const double b = na_block_sum(acc, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = b;
}

__device__ double na_erf_over_r(double r, double alpha) {
    if (r < 1e-8) return 2.0 * alpha / sqrt(kPi);
    return erf(alpha * r) / r;
}

// Partials in block order, then the self and exclusion parts
// (ewald_incremental_state.cc:125-135). out = {reciprocal, self, exclusion, total}.
__global__ void na_finish_kernel(const double* __restrict__ partial, int nblocks, Lattice L,
                                 double alpha, double rec_pref, const NaSites s,
                                 double* __restrict__ out) {
    __shared__ double sh[NA_THREADS];
    double acc = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += NA_THREADS) acc += partial[i];
    const double sum = na_block_sum(acc, sh);
    if (threadIdx.x != 0) return;
    double q2a = 0.0, q2r = 0.0, exa = 0.0, exr = 0.0;
    for (int pass = 0; pass < 2; ++pass) {
        const int b = pass == 0 ? s.nr : 0, e = pass == 0 ? s.nr + s.na : s.nr;
        double q2 = 0.0, ex = 0.0;
        for (int i = b; i < e; ++i) {
            q2 += s.q[i] * s.q[i];
            for (int j = i + 1; j < e; ++j) {
                double dx, dy, dz;
                min_image(L, s.x[j] - s.x[i], s.y[j] - s.y[i], s.z[j] - s.z[i], dx, dy, dz);
                ex += s.q[i] * s.q[j] * na_erf_over_r(sqrt(dx * dx + dy * dy + dz * dz), alpha);
            }
        }
        if (pass == 0) {
            q2a = q2;
            exa = ex;
        } else {
            q2r = q2;
            exr = ex;
        }
    }
    const double self = -kCoulomb * (alpha / sqrt(kPi)) * (q2a - q2r);
    const double excl = -kCoulomb * (exa - exr);
    const double rec = rec_pref * sum;
    out[0] = rec;
    out[1] = self;
    out[2] = excl;
    out[3] = rec + self + excl;
}

std::mutex g_addr_mutex;
double* g_addr[128] = {};  // cached device address of g_noalloc_partial, per device

double* scratch_address() {
    int dev = 0;
    ALEA_CUDA(cudaGetDevice(&dev));
    require(dev >= 0 && dev < 128, ALEA_ERR_RUNTIME, "alea_ewald_propose_no_alloc: device index");
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    if (!g_addr[dev]) {
        void* ptr = nullptr;
        ALEA_CUDA(cudaGetSymbolAddress(&ptr, g_noalloc_partial));
        g_addr[dev] = static_cast<double*>(ptr);
    }
    return g_addr[dev];
}

}  // namespace
}  // namespace alea

extern "C" alea_status alea_ewald_propose_no_alloc(const double* k, const double* weight,
                                                   const double* sre, const double* sim,
                                                   uint64_t n_terms, double alpha,
                                                   const alea_lattice* lattice,
                                                   const double* removed, uint64_t n_removed,
                                                   const double* added, uint64_t n_added,
                                                   double* out, void* cuda_stream) {
    using namespace alea;
    try {
        require(lattice != nullptr && out != nullptr, ALEA_ERR_INVALID_ARGUMENT,
                "alea_ewald_propose_no_alloc: lattice and out are required");
        require(n_terms <= NA_MAX_TERMS, ALEA_ERR_INVALID_ARGUMENT,
                "alea_ewald_propose_no_alloc: at most 262144 reciprocal terms (the size of its "
                "fixed scratch array)");
        // each count on its own first: their sum could wrap around
        require(n_removed <= (uint64_t)NA_MAX_SITES &&
                    n_added <= (uint64_t)NA_MAX_SITES - n_removed,
                ALEA_ERR_INVALID_ARGUMENT,
                "alea_ewald_propose_no_alloc: at most 64 removed + added sites");
        require(n_terms == 0 || (k && weight && sre && sim), ALEA_ERR_INVALID_ARGUMENT,
                "alea_ewald_propose_no_alloc: k, weight, sre and sim are required");
        require(alpha > 0.0, ALEA_ERR_INVALID_ARGUMENT, "Ewald: alpha must be positive");
        require((n_removed == 0 || removed) && (n_added == 0 || added), ALEA_ERR_INVALID_ARGUMENT,
                "alea_ewald_propose_no_alloc: site arrays are required");
        const Lattice L = make_lattice(lattice->m);
        NaSites s{};
        s.nr = (int)n_removed;
        s.na = (int)n_added;
        for (uint64_t i = 0; i < n_removed; ++i) {
            s.x[i] = removed[4 * i];
            s.y[i] = removed[4 * i + 1];
            s.z[i] = removed[4 * i + 2];
            s.q[i] = removed[4 * i + 3];
        }
        for (uint64_t i = 0; i < n_added; ++i) {
            s.x[n_removed + i] = added[4 * i];
            s.y[n_removed + i] = added[4 * i + 1];
            s.z[n_removed + i] = added[4 * i + 2];
            s.q[n_removed + i] = added[4 * i + 3];
        }
        require_device();
        double* partial = scratch_address();
        const cudaStream_t st = (cudaStream_t)cuda_stream;
        const int nb = n_terms ? (int)((n_terms + NA_THREADS - 1) / NA_THREADS) : 0;
        if (nb) na_delta_kernel<<<nb, NA_THREADS, 0, st>>>(n_terms, k, weight, sre, sim, s, partial);
        ALEA_CUDA(cudaGetLastError());
        const double rec_pref = kCoulomb * (2.0 * kPi / std::fabs(L.volume));
        na_finish_kernel<<<1, NA_THREADS, 0, st>>>(partial, nb, L, alpha, rec_pref, s, out);
        ALEA_CUDA(cudaGetLastError());
        record_last_error("");
        return ALEA_OK;
    } catch (const Error& e) {
        record_last_error(e.what());
        return e.status;
    } catch (...) {
        record_last_error("unknown error");
        return ALEA_ERR_RUNTIME;
    }
}
