// Host helpers shared by the kernels: lattice geometry, cutoff validation,
// mixed LJ parameter tables, device error flags.
#include <cmath>
#include <cstdio>
#include <map>
#include <vector>
#include <mutex>
#include <string>

#include "common.cuh"

namespace alea {

// lattice.hpp:35-41, lattice.cc:115-132, 166-175, 257-284
Lattice make_lattice(const double* m) {
    Lattice L{};
    for (int i = 0; i < 9; ++i) L.m[i] = m[i];
    auto cross = [](const double* a, const double* b, double* o) {
        o[0] = a[1] * b[2] - a[2] * b[1];
        o[1] = a[2] * b[0] - a[0] * b[2];
        o[2] = a[0] * b[1] - a[1] * b[0];
    };
    cross(m + 3, m + 6, L.c12);
    cross(m + 6, m, L.c20);
    cross(m, m + 3, L.c01);
    const double cx = m[4] * m[8] - m[5] * m[7];
    const double cy = m[5] * m[6] - m[3] * m[8];
    const double cz = m[3] * m[7] - m[4] * m[6];
    L.volume = m[0] * cx + m[1] * cy + m[2] * cz;
    require(std::fabs(L.volume) >= 1e-10, ALEA_ERR_INVALID_ARGUMENT,
            "Lattice: degenerate lattice (volume ~ 0)");
    for (int c = 0; c < 3; ++c) {
        L.inv[3 * c + 0] = L.c12[c] / L.volume;
        L.inv[3 * c + 1] = L.c20[c] / L.volume;
        L.inv[3 * c + 2] = L.c01[c] / L.volume;
    }
    const double* faces[3] = {L.c12, L.c20, L.c01};
    for (int a = 0; a < 3; ++a) {
        const double* f = faces[a];
        L.perp[a] = std::fabs(L.volume) / std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    }
    L.ortho = 1;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            if (i == j) continue;
            double scale = std::fabs(m[4 * i]);
            if (std::fabs(m[4 * j]) > scale) scale = std::fabs(m[4 * j]);
            if (1.0 > scale) scale = 1.0;
            if (std::fabs(m[3 * i + j]) > 1e-9 * scale) L.ortho = 0;
        }
    return L;
}

// Lattice::validateCutoff (lattice.cc:286-300), same message shape.
void validate_cutoff(const Lattice& L, double cutoff, const char* what) {
    static const char* names[3] = {"a0", "a1", "a2"};
    for (int a = 0; a < 3; ++a) {
        if (cutoff > 0.5 * L.perp[a]) {
            char buf[512];
            std::snprintf(buf, sizeof buf,
                          "%s: cutoff (%g Å) exceeds half the perpendicular width along lattice "
                          "direction %s (L_perp = %g Å, L_perp/2 = %g Å); minimum image would "
                          "double-count neighbors through two periodic images -- reduce the "
                          "cutoff or enlarge the cell along %s.",
                          what, cutoff, names[a], L.perp[a], 0.5 * L.perp[a], names[a]);
            throw Error(ALEA_ERR_INVALID_ARGUMENT, buf);
        }
    }
}

// LennardJones::mixedParameters (lennard_jones.cc:49-68) and the pairEnergy
// shift terms (lennard_jones.cc:70-86) for every ordered species pair.
void mixed_table(const alea_lennard_jones& lj, PairParams* out) {
    const uint32_t n = lj.n_species;
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t j = 0; j < n; ++j) {
            PairParams p{};
            if (i == j) {
                p.eps = lj.epsilon[i];
                p.sigma = lj.sigma[i];
            } else {
                p.eps = std::sqrt(lj.epsilon[i] * lj.epsilon[j]);
                p.sigma = lj.mixing == ALEA_LORENTZ_BERTHELOT ? 0.5 * (lj.sigma[i] + lj.sigma[j])
                                                              : std::sqrt(lj.sigma[i] * lj.sigma[j]);
            }
            if (lj.truncation != ALEA_TRUNCATED) p.shift = lj_raw(lj.cutoff, p.eps, p.sigma);
            if (lj.truncation == ALEA_LINEAR_FORCE_SHIFTED)
                p.dvdrc = lj_raw_derivative(lj.cutoff, p.eps, p.sigma);
            out[(size_t)i * n + j] = p;
        }
}

void check_device_flags(unsigned* d_flags, cudaStream_t s, const char* what) {
    unsigned f = 0;
    ALEA_CUDA(cudaMemcpyAsync(&f, d_flags, sizeof f, cudaMemcpyDeviceToHost, s));
    ALEA_CUDA(cudaStreamSynchronize(s));
    if (f) {
        ALEA_CUDA(cudaMemsetAsync(d_flags, 0, sizeof f, s));
        throw Error(ALEA_ERR_DEVICE_CHECK,
                    std::string(what) + ": device check failed (flags=" + std::to_string(f) +
                        (f & DEV_ERR_BOUNDS ? " bounds" : "") + (f & DEV_ERR_WAIT ? " wait" : "") +
                        (f & DEV_ERR_CAPACITY ? " capacity" : "") + ")");
    }
}

void require_device() {
    int n = 0;
    const cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        throw Error(ALEA_ERR_NO_DEVICE, std::string("no CUDA device available: ") +
                                            (e != cudaSuccess ? cudaGetErrorString(e) : "count 0"));
}

// ---------------------------------------------------------------- device memory
namespace {
constexpr size_t kKeepMin = 64ull << 20;   // blocks this large are kept on release
constexpr size_t kKeepMax = 16ull << 30;   // at most this much kept idle
std::mutex g_mem_mu;
KeptBlocks g_kept;                          // idle blocks by (device, size)

void free_on_device(int dev, void* p) {
    int cur = -1;
    cudaGetDevice(&cur);
    if (cur != dev) cudaSetDevice(dev);
    cudaFree(p);
    if (cur != dev && cur >= 0) cudaSetDevice(cur);
}

void free_all(std::vector<KeptBlocks::Block>&& blocks) {
    for (auto& b : blocks) free_on_device(b.device, b.p);
}
}  // namespace

// ---- KeptBlocks: the idle-block bookkeeping, no CUDA calls (tested on CPU)
void* KeptBlocks::take(int device, size_t bytes) {
    const auto it = blocks_.find({device, bytes});
    if (it == blocks_.end()) return nullptr;
    void* p = it->second;
    blocks_.erase(it);
    bytes_ -= bytes;
    return p;
}

bool KeptBlocks::put(int device, size_t bytes, void* p, size_t cap) {
    if (bytes_ + bytes > cap) return false;
    blocks_.emplace(std::make_pair(device, bytes), p);
    bytes_ += bytes;
    return true;
}

std::vector<KeptBlocks::Block> KeptBlocks::drain(int device) {
    std::vector<Block> out;
    for (auto it = blocks_.begin(); it != blocks_.end();) {
        if (device < 0 || it->first.first == device) {
            out.push_back({it->first.first, it->first.second, it->second});
            bytes_ -= it->first.second;
            it = blocks_.erase(it);
        } else {
            ++it;
        }
    }
    return out;
}

void* dev_alloc(size_t bytes) {
    int dev = 0;
    ALEA_CUDA(cudaGetDevice(&dev));
    if (bytes >= kKeepMin) {
        std::lock_guard<std::mutex> lock(g_mem_mu);
        if (void* p = g_kept.take(dev, bytes)) return p;
    }
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaErrorMemoryAllocation) {
        (void)cudaGetLastError();
        std::vector<KeptBlocks::Block> idle;
        {
            std::lock_guard<std::mutex> lock(g_mem_mu);
            idle = g_kept.drain(dev);
        }
        if (!idle.empty()) {
            free_all(std::move(idle));
            e = cudaMalloc(&p, bytes);
        }
    }
    ALEA_CUDA(e);
    return p;
}

// A kept block must not be handed out while kernels may still use it, so it
// is kept only after its own device has finished its work (the ordering
// cudaFree gives). The synchronisation runs outside the lock; a device that
// cannot be synchronised (a stream of it being captured, say) gets the block
// freed instead.
void dev_free(void* p, size_t bytes) {
    if (!p) return;
    int dev = -1;
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, p) == cudaSuccess && attr.type == cudaMemoryTypeDevice)
        dev = attr.device;
    else
        (void)cudaGetLastError();
    if (bytes >= kKeepMin && dev >= 0) {
        int cur = -1;
        cudaGetDevice(&cur);
        if (cur != dev) cudaSetDevice(dev);
        const bool idle = cudaDeviceSynchronize() == cudaSuccess;
        if (!idle) (void)cudaGetLastError();
        if (cur != dev && cur >= 0) cudaSetDevice(cur);
        if (idle) {
            std::lock_guard<std::mutex> lock(g_mem_mu);
            if (g_kept.put(dev, bytes, p, kKeepMax)) return;
        }
    }
    if (dev >= 0)
        free_on_device(dev, p);
    else
        cudaFree(p);
}

size_t dev_cached_bytes() {
    std::lock_guard<std::mutex> lock(g_mem_mu);
    return g_kept.bytes();
}

size_t dev_release_cached() {
    std::vector<KeptBlocks::Block> idle;
    {
        std::lock_guard<std::mutex> lock(g_mem_mu);
        idle = g_kept.drain(-1);
    }
    size_t n = 0;
    for (auto& b : idle) n += b.bytes;
    free_all(std::move(idle));
    return n;
}

}  // namespace alea
