// Shared device/host definitions for the aleator_gb300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/aleator_gb300.h"

namespace alea {

// ---------------------------------------------------------------- errors
// Host-side exception carrying an alea_status; caught at the C-ABI boundary.
struct Error : std::runtime_error {
    alea_status status;
    Error(alea_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess)
        throw Error(ALEA_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define ALEA_CUDA(call) ::alea::cuda_check((call), #call)

inline void require(bool ok, alea_status s, const std::string& msg) {
    if (!ok) throw Error(s, msg);
}

// Device-side error flag bits, written by kernels instead of trapping.
enum : unsigned {
    DEV_ERR_BOUNDS = 1u,   // an index check failed; the access was skipped
    DEV_ERR_WAIT = 2u,     // a bounded wait gave up
    DEV_ERR_CAPACITY = 4u, // a per-block staging list overflowed
};

__device__ __forceinline__ void flag_error(unsigned* flags, unsigned bit) {
    if (flags) atomicOr(flags, bit);
}

// ---------------------------------------------------------------- constants
constexpr double kPi = 3.14159265358979323846;
constexpr double kCoulomb = 167100.9468982874;  // ewald.hpp:62
constexpr double kEnergyCap = 1.0e5;            // framework_energy_grid.hpp:110

// ---------------------------------------------------------------- Philox4x32-10
// counter_based_rng.cc:13-54: 10 rounds, Weyl key bumps before rounds 1..9.
struct U32x4 {
    uint32_t v[4];
};

__host__ __device__ __forceinline__ void philox_mulhilo(uint32_t a, uint32_t b, uint32_t& hi,
                                                        uint32_t& lo) {
#ifdef __CUDA_ARCH__
    hi = __umulhi(a, b);
    lo = a * b;
#else
    const uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
#endif
}

__host__ __device__ __forceinline__ U32x4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                                        uint32_t c3, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint32_t hi0, lo0, hi1, lo1;
        philox_mulhilo(0xD2511F53u, c0, hi0, lo0);
        philox_mulhilo(0xCD9E8D57u, c2, hi1, lo1);
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    U32x4 o;
    o.v[0] = c0;
    o.v[1] = c1;
    o.v[2] = c2;
    o.v[3] = c3;
    return o;
}

// Philox4x32Rng::nextU64 at a given call index (counter_based_rng.cc:56-71).
__host__ __device__ __forceinline__ uint64_t philox_u64(uint64_t seed, uint64_t stream,
                                                        uint64_t call) {
    const U32x4 o = philox4x32_10((uint32_t)call, (uint32_t)(call >> 32), (uint32_t)stream,
                                  (uint32_t)(stream >> 32), (uint32_t)seed, (uint32_t)(seed >> 32));
    return ((uint64_t)o.v[0] << 32) | (uint64_t)o.v[1];
}

// Philox4x32Rng::nextUniform (counter_based_rng.cc:73-79): exact in FP64.
__host__ __device__ __forceinline__ double philox_uniform(uint64_t seed, uint64_t stream,
                                                          uint64_t call) {
    return (double)(philox_u64(seed, stream, call) >> 11) * (1.0 / 9007199254740992.0);
}

// ---------------------------------------------------------------- lattice
// Row-vector convention of core::Lattice: cart = f0 a0 + f1 a1 + f2 a2.
struct Lattice {
    double m[9];    // rows a_i
    double c12[3];  // a1 x a2  (cartesianToFractional, lattice.cc:166-175)
    double c20[3];  // a2 x a0
    double c01[3];  // a0 x a1
    double volume;  // signed a0 . (a1 x a2)
    double inv[9];  // column i = (a_j x a_k) / volume, so f = c . inv
    double perp[3]; // perpendicular widths (lattice.cc:257-284)
    int ortho;      // lattice.cc:115-132 tolerance 1e-9
};

Lattice make_lattice(const double* m);  // host
void validate_cutoff(const Lattice& L, double cutoff, const char* what);  // host

// Non-contracted FP64 helpers: keep the reference's rounding sequence where
// bit-level agreement is the goal (no fused multiply-add).
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dot_rn(const double* a, double x, double y, double z) {
    return add_rn(add_rn(mul_rn(a[0], x), mul_rn(a[1], y)), mul_rn(a[2], z));
}

// Minimum-image displacement for pairs that can lie within a cutoff
// rc <= L_perp/2: rounding each fractional coordinate of the displacement
// yields the unique image within rc whenever one exists (its fractional
// components are bounded by rc / L_perp <= 1/2), which is all an energy sum
// with pairEnergy(r > rc) = 0 needs (lattice.cc:185-255 finds the same image).
__device__ __forceinline__ void min_image(const Lattice& L, double dx, double dy, double dz,
                                          double& ox, double& oy, double& oz) {
    if (L.ortho) {
        ox = dx - L.m[0] * rint(dx / L.m[0]);
        oy = dy - L.m[4] * rint(dy / L.m[4]);
        oz = dz - L.m[8] * rint(dz / L.m[8]);
        return;
    }
    double f0 = dx * L.inv[0] + dy * L.inv[3] + dz * L.inv[6];
    double f1 = dx * L.inv[1] + dy * L.inv[4] + dz * L.inv[7];
    double f2 = dx * L.inv[2] + dy * L.inv[5] + dz * L.inv[8];
    f0 -= rint(f0);
    f1 -= rint(f1);
    f2 -= rint(f2);
    ox = f0 * L.m[0] + f1 * L.m[3] + f2 * L.m[6];
    oy = f0 * L.m[1] + f1 * L.m[4] + f2 * L.m[7];
    oz = f0 * L.m[2] + f1 * L.m[5] + f2 * L.m[8];
}

// ---------------------------------------------------------------- Lennard-Jones
// Mixed pair parameters for (guest species, framework species), precomputed on
// the host exactly as LennardJones::mixedParameters (lennard_jones.cc:49-68)
// and pairEnergy's shift terms (lennard_jones.cc:70-86).
struct PairParams {
    double eps;
    double sigma;
    double shift;   // rawPotential(rc) for Shifted / LFS, else 0
    double dvdrc;   // rawDerivative(rc) for LFS, else 0
};

// lennard_jones.cc:15-20 in FP64, reference operation order.
__host__ __device__ __forceinline__ double lj_raw(double r, double eps, double sigma) {
    const double sr = sigma / r;
    const double sr6 = sr * sr * sr * sr * sr * sr;
    const double sr12 = sr6 * sr6;
    return 4.0 * eps * (sr12 - sr6);
}

__host__ __device__ __forceinline__ double lj_raw_derivative(double r, double eps, double sigma) {
    const double sr = sigma / r;
    const double sr6 = sr * sr * sr * sr * sr * sr;
    const double sr12 = sr6 * sr6;
    return (24.0 * eps / r) * (sr6 - 2.0 * sr12);
}

// pairEnergy (lennard_jones.cc:70-86) with precomputed shift terms.
template <int TRUNC>
__host__ __device__ __forceinline__ double lj_pair(double r, double rc, const PairParams& p) {
    if (r > rc) return 0.0;
    const double v = lj_raw(r, p.eps, p.sigma);
    if (TRUNC == ALEA_TRUNCATED) return v;
    if (TRUNC == ALEA_SHIFTED) return v - p.shift;
    return v - p.shift - (r - rc) * p.dvdrc;
}

__device__ __forceinline__ double lj_pair_rt(int trunc, double r, double rc, const PairParams& p) {
    if (trunc == ALEA_TRUNCATED) return lj_pair<ALEA_TRUNCATED>(r, rc, p);
    if (trunc == ALEA_SHIFTED) return lj_pair<ALEA_SHIFTED>(r, rc, p);
    return lj_pair<ALEA_LINEAR_FORCE_SHIFTED>(r, rc, p);
}

// Host: mixed parameter table [n_species x n_species].
void mixed_table(const alea_lennard_jones& lj, PairParams* out);

// ---------------------------------------------------------------- device buffers
// Device memory for DevBuf: blocks of 64 MB and more are kept on release (up to
// 16 GB idle, over all devices) and handed out again for a request of the same
// size on the same device, so that objects rebuilt step after step (a grid's
// tables) skip cudaMalloc/cudaFree. Keeping a block synchronizes the block's
// own device first, as cudaFree would; an allocation that fails for memory
// releases the device's kept blocks and tries once more; dev_release_cached
// frees every idle block (alea_release_cached).
void* dev_alloc(size_t bytes);
void dev_free(void* p, size_t bytes);
size_t dev_cached_bytes();
size_t dev_release_cached();

// The idle-block bookkeeping of the allocator: blocks keyed by (device, size),
// at most `cap` bytes in total. No CUDA calls, so the keying is testable on any
// host (alea_test_block_cache).
class KeptBlocks {
public:
    struct Block {
        int device;
        size_t bytes;
        void* p;
    };
    void* take(int device, size_t bytes);                    // null when none kept
    bool put(int device, size_t bytes, void* p, size_t cap);  // false: over the cap
    std::vector<Block> drain(int device);                     // device < 0: all devices
    size_t bytes() const { return bytes_; }

private:
    std::multimap<std::pair<int, size_t>, void*> blocks_;
    size_t bytes_ = 0;
};

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    explicit DevBuf(size_t count) { alloc(count); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) {
        o.p = nullptr;
        o.n = 0;
    }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p;
            n = o.n;
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t count) {
        release();
        if (count) p = static_cast<T*>(dev_alloc(count * sizeof(T)));
        n = count;
    }
    void release() {
        if (p) dev_free(p, n * sizeof(T));
        p = nullptr;
        n = 0;
    }
    void upload(const T* host, size_t count, cudaStream_t s = 0) {
        if (count) ALEA_CUDA(cudaMemcpyAsync(p, host, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void download(T* host, size_t count, cudaStream_t s = 0) const {
        if (count) ALEA_CUDA(cudaMemcpyAsync(host, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
};

// Checks and clears a device error-flag word after a kernel sequence.
void check_device_flags(unsigned* d_flags, cudaStream_t s, const char* what);

// Records the calling thread's last error message (capi.cu) for entry points
// that do not go through the C-ABI wrapper.
void record_last_error(const char* message);

// Ensures a CUDA device exists (throws ALEA_ERR_NO_DEVICE otherwise).
void require_device();

// Host-side mirror of the particle SoA with defaults filled in.
struct HostParticles {
    uint64_t n = 0;
    const double *x = nullptr, *y = nullptr, *z = nullptr;
    std::string err;
};

}  // namespace alea
