// Framework energy grid on sm_103a: build (FP64 parity form and FP32 form
// with FP64 accumulation) and trilinear interpolation.
//
// Reference: FrameworkEnergyGrid (engines/monte_carlo/framework_energy_grid.cc:193-288).
// For every node (ix/nx, iy/ny, iz/nz) the reference sums pairEnergy over all
// framework atoms under the minimum-image convention and stores min(E, 1e5 K).
// Pairs beyond the cutoff contribute exactly 0, so with rc <= L_perp/2 the sum
// equals the sum over the (unique) periodic image of each atom within rc.
//
// Layout in HBM:
//   images   : periodic images of the framework atoms whose fractional
//              coordinates lie within rc/L_perp of the node range, as 32-byte
//              records {double x, y, z; uint32 type; uint32 pad}, sorted by a
//              fractional bin (bz, by, bx) and indexed by a CSR bin_start[].
//   tables   : one double table per guest species, flat (iz*ny+iy)*nx+ix.
// Kernel: one CTA per brick of 16x8x8 nodes (256 threads, 4 nodes each). The
// CTA culls candidate bins against its brick with a lower bound on the
// parallelepiped distance, merges each bin row into one contiguous atom
// range, and streams the ranges through shared memory in 256-record tiles.
// The FP64 form stages a tile with cp.async.bulk (TMA) copies, one per row
// range, completed on an mbarrier and double-buffered. The FP32 form gathers
// a tile with per-thread cp.async copies (record t*256 + tid by thread tid,
// issued one tile ahead): its bins are 4 A wide and a brick's ~100 row ranges
// hold ~7 records each, too short for bulk copies (issued one after another,
// they cost more than the sweep of the tile they fetch).
// The FP32 form then groups each tile by framework type, skips per warp the
// atoms beyond reach of the warp's 8x4x4 sub-box, and evaluates the rest as
// r^-6 (A r^-6 - B) with the shift terms applied per same-type run.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <numeric>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "ff.cuh"
#include "grid.cuh"

namespace alea {

namespace {

constexpr int BX = 16, BY = 8, BZ = 8;   // brick of nodes
constexpr int THREADS = 256;
constexpr int NPT = 4;                    // nodes per thread (along z)
constexpr int TILE = 256;                 // image records per shared-memory stage
constexpr int MAX_ROWS = 512;             // bin rows a brick may touch
constexpr int MAX_NG = 4;                 // guest species per launch
constexpr unsigned WAIT_LIMIT = 1u << 20; // bounded mbarrier polls (~0.1 s worst case)

struct __align__(16) ImageRec {
    double x, y, z;
    uint32_t type;
    uint32_t pad;
};
static_assert(sizeof(ImageRec) == 32, "image record must stay 32 bytes");

// The FP32 form's copy of an image: the position as double-float
// (x = xh + xl, ...), also 32 bytes so that both forms share the staging code.
struct __align__(16) ImageRecF {
    float xh, yh, zh;
    uint32_t type;
    float xl, yl, zl;
    float pad;
};
static_assert(sizeof(ImageRecF) == 32, "image record must stay 32 bytes");

struct GridGeom {
    Lattice L;
    int n[3];
    double lo[3], hi[3];     // fractional extent of the binned image range
    int nb[3];               // bins per axis
    double binw[3];          // fractional bin width
    float Gf[9];             // metric tensor a_i . a_j in FP32 (bin culling)
    float Ginvf[3];          // 1 / G_ii
    float lof[3], binwf[3], inv_binwf[3];  // lo, binw and 1 / binw in FP32
    float inv_nf[3];         // 1 / n per axis
    float hf[3];             // rc / L_perp per axis: the cutoff in fractional units
    float keep2f;            // rc^2 plus the bin-culling margin
    float hf_near[3];        // smax / L_perp: reach of the close-pair correction
    float keep2_near;        // smax^2 plus the bin-culling margin
    float rcf, rc2f, irc2f;  // rc, rc^2 and 1 / rc^2 in FP32
    float smaxf;             // largest mixed sigma of the grid's guests (close-pair reach)
    float sh[9], sl[9];      // row a: lattice vector a / n[a] as double-float (hi, lo)
    double rc, rc2;
    int bricks[3];
    int n_types;             // framework LJ species in the table
    int brick0;              // first brick of a launch (a slab of a pipelined build)
};

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}
// Non-blocking probe of one mbarrier phase (test_wait never suspends, so a
// loop of them is bounded by its iteration count).
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bulk global->shared copy (TMA, non-tensor): 16-byte aligned ends, size % 16 == 0.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Waits for one phase of an mbarrier with an iteration limit; on timeout the
// error flag is raised and false returned (the caller stops using the tile).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, unsigned* flags,
                                                  unsigned limit = WAIT_LIMIT) {
    for (unsigned it = 0; it < limit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if (it > 64) __nanosleep(64);
    }
    flag_error(flags, DEV_ERR_WAIT);
    return false;
}

// Lower bound on min |D . M|^2 over the fractional box D = [dlo, dhi]:
// a few coordinate-descent sweeps of the convex quadratic D^T G D, then the
// first-order bound f(x) + min_{y in box} grad(x).(y - x), which never exceeds
// the true minimum whatever point x of the box the sweeps end on (so Ginv,
// the reciprocal diagonal of G, need not be exact). Exact for orthorhombic cells. FP32 (FP64 issues at a small
// fraction of the FP32 rate on this part); the caller compares against rc^2
// with a relative margin far above FP32 rounding, so culling stays conservative.
__device__ __forceinline__ float box_min_dist2_lb(const float* G, const float* Ginv,
                                                  const float* dlo, const float* dhi) {
    float x[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) x[i] = fminf(fmaxf(0.0f, dlo[i]), dhi[i]);
#pragma unroll
    for (int sweep = 0; sweep < 4; ++sweep) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            float s = 0.0f;
#pragma unroll
            for (int j = 0; j < 3; ++j)
                if (j != i) s += G[3 * i + j] * x[j];
            x[i] = fminf(fmaxf(-s * Ginv[i], dlo[i]), dhi[i]);
        }
    }
    float g[3];
    float f = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        g[i] = 2.0f * (G[3 * i] * x[0] + G[3 * i + 1] * x[1] + G[3 * i + 2] * x[2]);
        f += 0.5f * g[i] * x[i];
    }
    float lb = f;
#pragma unroll
    for (int i = 0; i < 3; ++i) lb += fminf(g[i] * (dlo[i] - x[i]), g[i] * (dhi[i] - x[i]));
    return lb;
}

struct alignas(16) ParamFF {
    float sig2_hi, sig2_lo, eps4_hi, eps4_lo, shift_hi, shift_lo, dvdrc, pad;
};

// The FP32 main loop's pair term: 4 eps ((sigma/r)^12 - (sigma/r)^6) =
// r^-6 (A r^-6 - B) with A = 4 eps sigma^12 and B = 4 eps sigma^6: two FMAs
// per guest species once r^-6 is known.
struct alignas(16) ParamAB {
    float a, b, shift, dvdrc;
};

// Approximate reciprocal (MUFU, relative error within 1 ulp; ftz).
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}


// Node ownership inside a 16x8x8 brick: warp w covers the 8x4x4 sub-box
// ((w&1)*8, ((w>>1)&1)*4, (w>>2)*4); lane l the column (l%8, l/8) of it and
// NPT consecutive nodes along z. A compact sub-box keeps the warp's bounding
// sphere small for the per-warp atom cull.
__device__ __forceinline__ void thread_nodes(int tid, int& tx, int& ty, int& tz0) {
    const int w = tid >> 5, l = tid & 31;
    tx = (w & 1) * 8 + (l & 7);
    ty = ((w >> 1) & 1) * 4 + (l >> 3);
    tz0 = (w >> 2) * 4;
}

// Shared memory carved by hand (dynamic, above the 48 KB static limit); the
// host mirrors each kernel's layout to size the launch.
__host__ __device__ constexpr size_t carve(size_t bytes) { return (bytes + 127) & ~(size_t)127; }
struct SmemCarve {
    unsigned char* p;
    template <typename T>
    __device__ T* take(size_t n) {
        T* q = reinterpret_cast<T*>(p);
        p += carve(n * sizeof(T));
        return q;
    }
};

// ---------------------------------------------------------------- brick plan
// The bin rows a brick can reach: one thread per (by, bz) row finds the first
// and last bins within reach of the brick's nodes (FP32 lower bound on the
// parallelepiped distance against keep2 = reach^2 plus a margin; reach_frac =
// reach / L_perp per axis bounds the bin range), then an exclusive scan turns the
// row lengths into offsets of one concatenated candidate list. Row slots
// follow the row enumeration, so the candidate order (and the floating-point
// summation order) is the same on every run. Returns the number of rows, or
// -1 with the error flag raised when the brick touches more than MAX_ROWS
// rows (the same on every thread). Every thread of the block calls it.
__device__ int plan_rows(const GridGeom& geo, const float* reach_frac, float keep2,
                         const uint32_t* __restrict__ bin_start, int x0, int y0, int z0,
                         uint32_t* row_begin, uint32_t* row_off, uint32_t* warp_tot,
                         unsigned* flags) {
    const int tid = threadIdx.x;
    const int lo_i[3] = {x0, y0, z0};
    const int hi_i[3] = {min(x0 + BX, geo.n[0]) - 1, min(y0 + BY, geo.n[1]) - 1,
                         min(z0 + BZ, geo.n[2]) - 1};
    float flof[3], fhif[3];
    int blo[3], bhi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        flof[a] = lo_i[a] * geo.inv_nf[a];
        fhif[a] = hi_i[a] * geo.inv_nf[a];
        // one bin of margin on each side covers the FP32 rounding here
        blo[a] = max(0, (int)floorf((flof[a] - reach_frac[a] - geo.lof[a]) * geo.inv_binwf[a]) - 1);
        bhi[a] = min(geo.nb[a] - 1,
                     (int)floorf((fhif[a] + reach_frac[a] - geo.lof[a]) * geo.inv_binwf[a]) + 1);
    }
    const int rows_y = bhi[1] - blo[1] + 1, rows_z = bhi[2] - blo[2] + 1;
    const int nr = rows_y * rows_z;
    if (nr > MAX_ROWS) {
        if (tid == 0) flag_error(flags, DEV_ERR_CAPACITY);
        return -1;
    }
    for (int r = tid; r < nr; r += THREADS) {
        const int ry = blo[1] + r % rows_y, rz = blo[2] + r / rows_y;
        int first = -1, last = -1;
        float dlo[3], dhi[3];
        const int byz[2] = {ry, rz};
#pragma unroll
        for (int a = 1; a < 3; ++a) {
            const float b0 = geo.lof[a] + byz[a - 1] * geo.binwf[a];
            dlo[a] = b0 - fhif[a];
            dhi[a] = b0 + geo.binwf[a] - flof[a];
        }
        for (int rx = blo[0]; rx <= bhi[0]; ++rx) {
            const float b0 = geo.lof[0] + rx * geo.binwf[0];
            dlo[0] = b0 - fhif[0];
            dhi[0] = b0 + geo.binwf[0] - flof[0];
            if (box_min_dist2_lb(geo.Gf, geo.Ginvf, dlo, dhi) <= keep2) {
                if (first < 0) first = rx;
                last = rx;
            }
        }
        uint32_t s = 0, e = 0;
        if (first >= 0) {
            const size_t row = ((size_t)rz * geo.nb[1] + ry) * geo.nb[0];
            s = bin_start[row + first];
            e = bin_start[row + last + 1];
        }
        row_begin[r] = s;
        row_off[r + 1] = e - s;
    }
    __syncthreads();
    // exclusive scan of the row counts: each thread sums a run of rows, a
    // warp scan over those sums, then a scan of the warp totals
    {
        constexpr int PER = (MAX_ROWS + THREADS - 1) / THREADS;
        const int r0 = tid * PER;
        uint32_t run = 0;
        for (int i = 0; i < PER; ++i)
            if (r0 + i < nr) run += row_off[r0 + i + 1];
        uint32_t incl = run;
        const int lane = tid & 31, wid = tid >> 5;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 31) warp_tot[wid] = incl;
        __syncthreads();
        uint32_t base = 0;
        for (int w = 0; w < wid; ++w) base += warp_tot[w];
        uint32_t acc = base + incl - run;
        for (int i = 0; i < PER; ++i)
            if (r0 + i < nr) {
                const uint32_t c = row_off[r0 + i + 1];
                row_off[r0 + i + 1] = acc + c;
                acc += c;
            }
        if (tid == 0) row_off[0] = 0;
    }
    __syncthreads();
    return nr;
}

// Stages tile t of the brick's concatenated candidate list (32-byte records)
// into dst: one bulk copy per overlapping row range, completing on bar.
__device__ void issue_tile(uint32_t t, uint32_t n_cand, int nr, const uint32_t* row_begin,
                           const uint32_t* row_off, const unsigned char* images,
                           unsigned char* dst, uint64_t* bar) {
    constexpr uint32_t REC = 32;
    const uint32_t a = t * TILE;
    const uint32_t b = min(a + (uint32_t)TILE, n_cand);
    mbar_expect_tx(bar, (b - a) * REC);
    int lo = 0, hi = nr - 1;  // last row with row_off[r] <= a
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (row_off[mid] <= a) lo = mid; else hi = mid - 1;
    }
    for (int r = lo; r < nr && row_off[r] < b; ++r) {
        const uint32_t s = max(row_off[r], a), e = min(row_off[r + 1], b);
        if (e > s)
            bulk_g2s(dst + (size_t)(s - a) * REC,
                     images + (size_t)(row_begin[r] + (s - row_off[r])) * REC, (e - s) * REC, bar);
    }
}

// Per-thread asynchronous global->shared copies (16 bytes, L2 only), waited
// for by the issuing thread.
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// FP32 form: candidate t * TILE + tid of the brick's concatenated list into
// this thread's 32-byte slot of dst (the thread that later converts it).
__device__ __forceinline__ void gather_tile(uint32_t t, uint32_t n_cand, int nr, const uint32_t* row_begin,
                                            const uint32_t* row_off, const unsigned char* images,
                                            unsigned char* dst) {
    constexpr uint32_t REC = 32;
    const uint32_t c = t * TILE + threadIdx.x;
    if (c < n_cand) {
        int lo = 0, hi = nr - 1;  // last row with row_off[r] <= c: the row holding c
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (row_off[mid] <= c) lo = mid; else hi = mid - 1;
        }
        const unsigned char* src = images + (size_t)(row_begin[lo] + (c - row_off[lo])) * REC;
        cp_async16(dst + threadIdx.x * REC, src);
        cp_async16(dst + threadIdx.x * REC + 16, src + 16);
    }
    cp_async_commit();
}

// After a timed-out wait: tiles failed_tile and failed_tile + 1 are the only
// ones issued and not consumed; wait for each (again bounded) before exit.
__device__ void drain_tiles(uint32_t failed_tile, uint32_t n_tiles, uint64_t* bars) {
    if (threadIdx.x == 0)
        for (uint32_t t = failed_tile; t < failed_tile + 2 && t < n_tiles; ++t)
            for (unsigned it = 0; it < WAIT_LIMIT && !mbar_try_wait(&bars[t & 1], (t >> 1) & 1); ++it)
                __nanosleep(64);
    __syncthreads();
}

// ---------------------------------------------------------------- large cutoffs
// A cutoff above half a perpendicular width (rc > L_perp/2): the reference's
// constructor does not check this (framework_energy_grid.cc:193-249) and sums,
// per node and atom, pairEnergy of the single minimum-image displacement
// (Lattice::minimumImageDisplacement, lattice.cc:185-255: per axis for an
// orthorhombic cell, else the best of the 125 lattice translations around the
// nearest one in the greedily reduced basis, lattice.cc:70-101). Beyond L_perp/2
// an atom can have several images within rc but only that one counts, so the
// image-list kernels (which add every image within rc) would differ; this
// FP64 kernel restates the reference's loop instead: a thread per node, the
// atoms in index order through shared-memory tiles.
struct MiGeom {
    double m[9];     // lattice rows
    int ortho;
    double r[9];     // the reduced basis, rows
    double t0[3], t1[3], t2[3];  // r1 x r2, r2 x r0, r0 x r1
    double rvol;     // r0 . (r1 x r2)
    int n[3];
    double rc;
    int trunc;
    uint32_t n_species;
};

// lattice.cc:70-101 (greedyReduce): size reduction of each vector against the
// others, then the three sorted by squared length, until nothing changes.
static void reduced_basis(const double* m, double* out) {
    double v[3][3];
    for (int i = 0; i < 3; ++i)
        for (int c = 0; c < 3; ++c) v[i][c] = m[3 * i + c];
    auto n2 = [](const double* a) { return a[0] * a[0] + a[1] * a[1] + a[2] * a[2]; };
    for (int iter = 0; iter < 50; ++iter) {
        bool changed = false;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                if (i == j) continue;
                const double nj2 = n2(v[j]);
                if (nj2 < 1e-10) continue;
                const double t = std::round((v[i][0] * v[j][0] + v[i][1] * v[j][1] + v[i][2] * v[j][2]) / nj2);
                if (t != 0.0) {
                    for (int c = 0; c < 3; ++c) v[i][c] = v[i][c] - v[j][c] * t;
                    changed = true;
                }
            }
        for (int i = 1; i < 3; ++i) {  // three elements: an insertion sort on the squared length
            double tmp[3] = {v[i][0], v[i][1], v[i][2]};
            const double key = n2(tmp);
            int j = i - 1;
            while (j >= 0 && key < n2(v[j])) {
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

__device__ __forceinline__ void mi_reference(const MiGeom& G, const double* d, double* out) {
    if (G.ortho) {
        for (int a = 0; a < 3; ++a) {
            const double len = G.m[4 * a];
            out[a] = d[a] - len * round(d[a] / len);
        }
        return;
    }
    const double f0 = (d[0] * G.t0[0] + d[1] * G.t0[1] + d[2] * G.t0[2]) / G.rvol;
    const double f1 = (d[0] * G.t1[0] + d[1] * G.t1[1] + d[2] * G.t1[2]) / G.rvol;
    const double f2 = (d[0] * G.t2[0] + d[1] * G.t2[1] + d[2] * G.t2[2]) / G.rvol;
    const double n0 = round(f0), n1 = round(f1), n2 = round(f2);
    out[0] = d[0];
    out[1] = d[1];
    out[2] = d[2];
    double best2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    for (int a = -2; a <= 2; ++a)
        for (int b = -2; b <= 2; ++b)
            for (int c = -2; c <= 2; ++c) {
                const double c0 = n0 + a, c1 = n1 + b, c2 = n2 + c;
                double cand[3];
                for (int k = 0; k < 3; ++k) cand[k] = d[k] - ((G.r[k] * c0 + G.r[3 + k] * c1) + G.r[6 + k] * c2);
                const double cn2 = cand[0] * cand[0] + cand[1] * cand[1] + cand[2] * cand[2];
                if (cn2 < best2) {
                    best2 = cn2;
                    out[0] = cand[0];
                    out[1] = cand[1];
                    out[2] = cand[2];
                }
            }
}

constexpr int MI_THREADS = 128;

__global__ void __launch_bounds__(MI_THREADS)
grid_build_mi_kernel(MiGeom G, const ImageRec* __restrict__ atoms, uint64_t n_atoms,
                     const PairParams* __restrict__ params, const uint32_t* __restrict__ guests,
                     int ng, double* __restrict__ tables) {
    __shared__ ImageRec tile[MI_THREADS];
    const uint64_t nodes = (uint64_t)G.n[0] * G.n[1] * G.n[2];
    const uint64_t idx = (uint64_t)blockIdx.x * MI_THREADS + threadIdx.x;
    const bool on = idx < nodes;
    const int ix = (int)(idx % G.n[0]), iy = (int)((idx / G.n[0]) % G.n[1]), iz = (int)(idx / ((uint64_t)G.n[0] * G.n[1]));
    const double f[3] = {(double)ix / G.n[0], (double)iy / G.n[1], (double)iz / G.n[2]};
    double cart[3];
    for (int c = 0; c < 3; ++c) cart[c] = (f[0] * G.m[c] + f[1] * G.m[3 + c]) + f[2] * G.m[6 + c];
    for (int g = 0; g < ng; ++g) {
        const PairParams* row = params + (size_t)guests[g] * G.n_species;
        double e = 0.0;
        for (uint64_t base = 0; base < n_atoms; base += MI_THREADS) {
            __syncthreads();
            if (base + threadIdx.x < n_atoms) tile[threadIdx.x] = atoms[base + threadIdx.x];
            __syncthreads();
            const int cnt = (int)min((uint64_t)MI_THREADS, n_atoms - base);
            if (!on) continue;
            for (int j = 0; j < cnt; ++j) {
                const ImageRec a = tile[j];
                const double d[3] = {a.x - cart[0], a.y - cart[1], a.z - cart[2]};
                double o[3];
                mi_reference(G, d, o);
                const double r = sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
                e += lj_pair_rt(G.trunc, r, G.rc, row[a.type]);
            }
        }
        if (on) tables[(size_t)g * nodes + idx] = (kEnergyCap < e) ? kEnergyCap : e;  // capped()
    }
}

// ---------------------------------------------------------------- FP64 build kernel
// The parity form: the reference's node positions and pairEnergy in FP64 on
// global Cartesian coordinates, candidates in a fixed order.
template <int NG, int TRUNC>
__global__ void __launch_bounds__(THREADS, 2)
grid_build_f64_kernel(GridGeom geo, const ImageRec* __restrict__ images,
                      const uint32_t* __restrict__ bin_start, const PairParams* __restrict__ params,
                      const uint32_t* __restrict__ guests, double* __restrict__ tables,
                      unsigned long long* __restrict__ executed, unsigned* flags,
                      unsigned tile_wait) {
    extern __shared__ __align__(128) unsigned char smem[];
    SmemCarve sc{smem};
    ImageRec* raw = sc.take<ImageRec>(2 * TILE);
    uint64_t* bars = sc.take<uint64_t>(2);
    uint32_t* row_begin = sc.take<uint32_t>(MAX_ROWS);
    uint32_t* row_off = sc.take<uint32_t>(MAX_ROWS + 1);
    uint32_t* warp_tot = sc.take<uint32_t>(THREADS / 32);
    PairParams* pd = sc.take<PairParams>(64 * NG);

    const int tid = threadIdx.x;
    const int nx = geo.n[0], ny = geo.n[1], nz = geo.n[2];
    const int brick = geo.brick0 + (int)blockIdx.x;
    const int bxn = geo.bricks[0], byn = geo.bricks[1];
    const int bx = brick % bxn, by = (brick / bxn) % byn, bz = brick / (bxn * byn);
    const int x0 = bx * BX, y0 = by * BY, z0 = bz * BZ;

    for (int i = tid; i < geo.n_types * NG; i += THREADS) {
        const int t = i / NG, g = i % NG;
        pd[i] = params[(size_t)guests[g] * geo.n_types + t];
    }
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_barrier_init();
    }
    __syncthreads();
    const int nr = plan_rows(geo, geo.hf, geo.keep2f, bin_start, x0, y0, z0, row_begin, row_off,
                             warp_tot, flags);
    if (nr < 0) return;
    const uint32_t n_cand = row_off[nr];

    int tx, ty, tz0;
    thread_nodes(tid, tx, ty, tz0);
    const int ixn = x0 + tx, iyn = y0 + ty;
    const double* M = geo.L.m;
    double nxr[NPT], nyr[NPT], nzr[NPT];
#pragma unroll
    for (int k = 0; k < NPT; ++k) {
        // framework_energy_grid.cc:227-231 node position
        const int izn = z0 + tz0 + k;
        const double f0 = (double)ixn / nx, f1 = (double)iyn / ny, f2 = (double)izn / nz;
        double c[3];
#pragma unroll
        for (int cc = 0; cc < 3; ++cc)
            c[cc] = add_rn(add_rn(mul_rn(f0, M[cc]), mul_rn(f1, M[3 + cc])), mul_rn(f2, M[6 + cc]));
        nxr[k] = c[0];
        nyr[k] = c[1];
        nzr[k] = c[2];
    }
    double acc[NG][NPT];
#pragma unroll
    for (int g = 0; g < NG; ++g)
#pragma unroll
        for (int k = 0; k < NPT; ++k) acc[g][k] = 0.0;

    const unsigned char* img = reinterpret_cast<const unsigned char*>(images);
    unsigned char* rawb = reinterpret_cast<unsigned char*>(raw);
    const uint32_t n_tiles = (n_cand + TILE - 1) / TILE;
    if (tid == 0) {
        if (n_tiles > 0) issue_tile(0, n_cand, nr, row_begin, row_off, img, rawb, &bars[0]);
        if (n_tiles > 1)
            issue_tile(1, n_cand, nr, row_begin, row_off, img, rawb + TILE * sizeof(ImageRec), &bars[1]);
    }
    for (uint32_t t = 0; t < n_tiles; ++t) {
        const int buf = t & 1;
        const uint32_t cnt = min((uint32_t)TILE, n_cand - t * TILE);
        // block-wide vote so that every thread takes the same path on a timeout
        const bool got = mbar_wait_bounded(&bars[buf], (t >> 1) & 1, flags, tile_wait);
        if (!__syncthreads_and(got)) {
            drain_tiles(t, n_tiles, bars);
            return;
        }
        for (uint32_t j = 0; j < cnt; ++j) {
            const ImageRec a = raw[buf * TILE + j];
            const PairParams* pp = &pd[a.type * NG];
#pragma unroll
            for (int k = 0; k < NPT; ++k) {
                const double dx = a.x - nxr[k];
                const double dy = a.y - nyr[k];
                const double dz = a.z - nzr[k];
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (r2 > geo.rc2 * (1.0 + 1e-12)) continue;
                const double r = sqrt(r2);
#pragma unroll
                for (int g = 0; g < NG; ++g) acc[g][k] += lj_pair<TRUNC>(r, geo.rc, pp[g]);
            }
        }
        __syncthreads();
        if (tid == 0 && t + 2 < n_tiles) {
            fence_proxy_async();
            issue_tile(t + 2, n_cand, nr, row_begin, row_off, img, rawb + buf * TILE * sizeof(ImageRec),
                       &bars[buf]);
        }
    }

    // store min(E, cap) (framework_energy_grid.cc:22, 243)
    const size_t plane = (size_t)nx * ny;
    const size_t per_table = plane * nz;
#pragma unroll
    for (int k = 0; k < NPT; ++k) {
        const int izn = z0 + tz0 + k;
        if (ixn < nx && iyn < ny && izn < nz) {
            const size_t idx = (size_t)izn * plane + (size_t)iyn * nx + ixn;
#pragma unroll
            for (int g = 0; g < NG; ++g) {
                const double e = acc[g][k];
                tables[(size_t)g * per_table + idx] = (kEnergyCap < e) ? kEnergyCap : e;
            }
        }
    }
    if (tid == 0) {
        const unsigned long long active = (unsigned long long)(min(x0 + BX, nx) - x0) *
                                          (min(y0 + BY, ny) - y0) * (min(z0 + BZ, nz) - z0);
        atomicAdd(executed, active * n_cand);
    }
}

template <int NG>
constexpr size_t f64_smem_bytes() {
    return carve(2 * TILE * sizeof(ImageRec)) + carve(2 * sizeof(uint64_t)) +
           carve(MAX_ROWS * sizeof(uint32_t)) + carve((MAX_ROWS + 1) * sizeof(uint32_t)) +
           carve((THREADS / 32) * sizeof(uint32_t)) + carve(64 * NG * sizeof(PairParams));
}

// ---------------------------------------------------------------- packed FP32
// Two FP32 lanes in one 64-bit register (PTX .f32x2, sm_100 family): one
// instruction adds, multiplies or fuses two lanes, each rounded exactly as the
// scalar instruction would round it. The FP32 kernel keeps the nodes k and
// k + 1 of a thread in the two lanes.
typedef unsigned long long f2;
__device__ __forceinline__ f2 f2_pack(float lo, float hi) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2 v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) {
    f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// ---------------------------------------------------------------- FP32 build: shared pieces
// The FP32 form runs in two kernels, the sweep and the close-pair correction,
// which must classify every (atom, node) pair identically. Both therefore
// build positions and r^2 with the same explicitly rounded operations below
// (no contraction can differ between them).

// Per (framework type t, guest g) parameters in shared memory, and per type
// the FP32 window's inner edge sigma_t^2 (the largest sigma^2 over the
// guests) with the value the sweep adds for a pair clamped to it.
template <int NG, int TRUNC>
struct F32Params {
    ulonglong2 ab[64 * NG];  // {A, A}, {-B, -B}
    float shift[64 * NG];
    float dvdrc[64 * NG];
    float vclose[64 * NG];
    float close2[64];
};

template <int NG, int TRUNC>
__device__ void load_f32_params(F32Params<NG, TRUNC>& P, const ParamAB* __restrict__ pab_g,
                                const ParamFF* __restrict__ pff_g, int nt, float rcf) {
    const int tid = threadIdx.x;
    for (int i = tid; i < nt * NG; i += THREADS) {
        const int t = i / NG, g = i % NG;
        const ParamAB p = pab_g[(size_t)g * nt + t];
        P.ab[i] = make_ulonglong2(f2_pack(p.a, p.a), f2_pack(-p.b, -p.b));
        P.shift[i] = TRUNC == ALEA_TRUNCATED ? 0.f : p.shift;
        P.dvdrc[i] = p.dvdrc;
    }
    __syncthreads();
    // the sweep's operations, in its order, at r^2 = sigma_t^2
    for (int t = tid; t < nt; t += THREADS) {
        float m = 0.f;
        for (int g = 0; g < NG; ++g) m = fmaxf(m, pff_g[(size_t)g * nt + t].sig2_hi);
        P.close2[t] = m;
        const float ir2 = rcp_approx(m);
        const float ir6 = __fmul_rn(ir2, __fmul_rn(ir2, ir2));
        for (int g = 0; g < NG; ++g) {
            float a, nb, dummy;
            f2_unpack(P.ab[t * NG + g].x, a, dummy);
            f2_unpack(P.ab[t * NG + g].y, nb, dummy);
            float v = __fmul_rn(ir6, __fmaf_rn(a, ir6, nb));
            if (TRUNC == ALEA_LINEAR_FORCE_SHIFTED)
                v = __fmaf_rn(-P.dvdrc[t * NG + g], __fsub_rn(__fmul_rn(m, rsqrtf(m)), rcf), v);
            P.vclose[t * NG + g] = v;
        }
    }
    __syncthreads();
}

// The brick centre (x0 + 7.5, y0 + 3.5, z0 + 3.5 in node units) in
// double-float: sum over axes of (centre index) x (lattice vector / n).
__device__ __forceinline__ void brick_origin(const GridGeom& geo, int x0, int y0, int z0, ff* org) {
    const float cen[3] = {x0 + 0.5f * (BX - 1), y0 + 0.5f * (BY - 1), z0 + 0.5f * (BZ - 1)};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        ff v = ff_scale(cen[0], ff{geo.sh[c], geo.sl[c]});
        v = ff_add(v, ff_scale(cen[1], ff{geo.sh[3 + c], geo.sl[3 + c]}));
        org[c] = ff_add(v, ff_scale(cen[2], ff{geo.sh[6 + c], geo.sl[6 + c]}));
    }
}

// A node relative to the brick centre, from its offsets (small half-integers,
// exact in FP32), as double-float components.
__device__ __forceinline__ void node_local(const GridGeom& geo, float dxi, float dyi, float dzi,
                                           ff* v) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        ff w = ff_scale(dxi, ff{geo.sh[c], geo.sl[c]});
        w = ff_add(w, ff_scale(dyi, ff{geo.sh[3 + c], geo.sl[3 + c]}));
        v[c] = ff_add(w, ff_scale(dzi, ff{geo.sh[6 + c], geo.sl[6 + c]}));
    }
}

// An image relative to the brick centre, as double-float components.
__device__ __forceinline__ void atom_local(const ImageRecF& r, const ff* org, ff* v) {
    v[0] = ff_add(ff{r.xh, r.xl}, ff{-org[0].hi, -org[0].lo});
    v[1] = ff_add(ff{r.yh, r.yl}, ff{-org[1].hi, -org[1].lo});
    v[2] = ff_add(ff{r.zh, r.zl}, ff{-org[2].hi, -org[2].lo});
}

// FP32 r^2 from the hi parts, rounded exactly as the packed sweep rounds it.
__device__ __forceinline__ float r2_f32(float ax, float ay, float az, float nx, float ny, float nz) {
    const float dx = __fsub_rn(ax, nx), dy = __fsub_rn(ay, ny), dz = __fsub_rn(az, nz);
    return __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
}

// Double-float energy of one close pair for one guest, shift (and the linear
// force shift) included, minus what the sweep adds for it (vclose) and plus
// the -V(rc) the sweep charges every pair: the correction that turns the
// sweep's value for this pair into the exact one.
// 4 eps ((sigma^2/r^2)^6 - (sigma^2/r^2)^3) in double-float, from r^2.
__device__ __forceinline__ ff pair_ff(const ParamFF& q, ff rr) {
    const ff s2 = ff_mul(ff{q.sig2_hi, q.sig2_lo}, ff_rcp(rr));
    const ff s6 = ff_mul(ff_mul(s2, s2), s2);
    return ff_mul(ff{q.eps4_hi, q.eps4_lo}, ff_mul(s6, ff_add(s6, ff{-1.f, 0.f})));
}

template <int NG, int TRUNC>
__device__ __forceinline__ ff close_pair(const F32Params<NG, TRUNC>& P, const ParamFF* pff, int type, int g, ff ddx,
                                         ff ddy, ff ddz, float rcf) {
    ff rr = ff_add(ff_add(ff_mul(ddx, ddx), ff_mul(ddy, ddy)), ff_mul(ddz, ddz));
    if (rr.hi < 1e-4f) rr = ff{1e-4f, 0.f};
    const ParamFF q = pff[type * NG + g];
    ff e = ff_add(pair_ff(q, rr), ff{-q.shift_hi, -q.shift_lo});
    if (TRUNC == ALEA_LINEAR_FORCE_SHIFTED) {
        const float rs = sqrtf(rr.hi);
        e = ff_add(e, ff{-(rs - rcf) * q.dvdrc, 0.f});
    }
    e = ff_add_f(e, -P.vclose[type * NG + g]);
    return ff_add_f(e, P.shift[type * NG + g]);
}

// Nodes whose FP32 close-pair estimate |ce| stays within this multiple of
// max(floor, |E|) keep the FP32 sum; the others get the double-float
// correction. The estimate's FP32 error stays within about 1.5e-6 |ce|, so
// within 3e-6 x max(floor, |E|) here. (On dense frameworks about 1-2% of the
// nodes exceed the ratio: nodes near 0 K with a few strongly repulsive pairs.)
constexpr float CLOSE_FP32_RATIO = 2.0f;
constexpr float CLOSE_FP32_FLOOR = 300.0f;  // K

// Plain truncation: V jumps by V(rc) at the cutoff, so a pair whose FP32 r^2
// lies within this fraction of rc^2 may be on the wrong side of it (the FP32
// r^2 of brick-centred positions is off by ~1e-4 A^2 at most, 6e-7 of rc^2
// for rc = 12.8 A); the node goes to the correction, which redoes those
// pairs' decisions in double-float.
constexpr float CUT_AMBIGUITY = 4e-6f;
constexpr uint32_t FIX_AT_CUTOFF = 0x80;  // flag-mask bit: pairs at rc to redo

// ---------------------------------------------------------------- FP32 sweep kernel
// Pair terms in FP32 on brick-centred coordinates, double-float where a
// rounding error would reach the result (image and node positions, the
// per-node accumulators). FP64 issues at a small fraction of the FP32 rate on
// this part, so the only FP64 operations left are the final stores.
//
// Per tile of 256 candidates each thread converts one record to brick-centred
// FP32 (hi + lo parts); then every warp walks the tile, skipping atoms beyond
// rc + (its sub-box radius) of its sub-box centre (a warp-uniform branch).
// For each remaining atom and node:
//   * r^2 is clamped to [sigma_t^2, rc^2] (sigma_t: the atom type's largest
//     sigma over the guests) and r^-6 (A r^-6 - B) evaluated in FP32 at the
//     clamped value, two nodes per instruction;
//   * every evaluated pair is charged -V(rc) (the shift; summed per atom, not
//     per pair), so a pair beyond rc contributes V(rc) - V(rc) = 0 to FP32
//     rounding and a pair within the window V(r) - V(rc);
//   * for a pair closer than sigma_t (only atoms within sigma_t + radius of
//     the warp centre can have one: a warp-uniform branch) the exact value
//     minus the clamped one is estimated in FP32 into a separate per-node sum.
// Per node and guest the result is then: the sweep's sum when there is no
// close pair; the cap when sum + estimate exceeds it by 1%; sum + estimate
// when the estimate is small against max(300 K, |E|); otherwise the sweep's
// sum is stored and the node's close pairs redone in double-float at the end
// of the brick (fix_flagged).
// With plain truncation a pair beyond rc gets r^-2 = 0 instead (no shift).
// Linear force shifting adds -(r - rc) V'(rc) per pair at the clamped r.
// Pointers of one grid for the FP32 kernels.
struct F32GridArgs {
    const ImageRecF* images;
    const uint32_t* bin_start;
    const ParamAB* pab;  // [guest of this launch][type]
    const ParamFF* pff;  // [guest of this launch][type]
    double* tables;
    // the bricks' row plans made by grid_plan_kernel (stride words a brick:
    // nr, row_begin[nr], row_off[nr + 1]), or null: each brick plans itself
    const uint32_t* plans;
    uint32_t plan_stride;
};

// The row plan of every brick of a launch (plan_rows), ahead of the sweep: a
// light kernel (small registers and shared memory, so many CTAs a SM hide
// the bin loads and the per-row bin tests), where in the sweep each brick's
// planning held its CTA's warps from the pair loop. nr = ~0u: the brick
// touches more rows than a plan holds (the error flag is raised).
__global__ void __launch_bounds__(THREADS)
grid_plan_kernel(GridGeom geo, const uint32_t* __restrict__ bin_start, uint32_t* __restrict__ plans,
                 uint32_t stride, unsigned* flags) {
    __shared__ uint32_t row_begin[MAX_ROWS], row_off[MAX_ROWS + 1], warp_tot[THREADS / 32];
    const int brick = geo.brick0 + (int)blockIdx.x;
    const int bxn = geo.bricks[0], byn = geo.bricks[1];
    const int bx = brick % bxn, by = (brick / bxn) % byn, bz = brick / (bxn * byn);
    uint32_t* out = plans + (size_t)brick * stride;
    const int nr = plan_rows(geo, geo.hf, geo.keep2f, bin_start, bx * BX, by * BY, bz * BZ, row_begin,
                             row_off, warp_tot, flags);
    if (nr < 0 || 2 * (uint32_t)nr + 2 > stride) {
        if (threadIdx.x == 0) {
            if (nr >= 0) flag_error(flags, DEV_ERR_CAPACITY);
            out[0] = ~0u;
        }
        return;
    }
    if (threadIdx.x == 0) out[0] = (uint32_t)nr;
    for (int i = threadIdx.x; i < nr; i += THREADS) out[1 + i] = row_begin[i];
    for (int i = threadIdx.x; i <= nr; i += THREADS) out[1 + nr + i] = row_off[i];
}

// ---------------------------------------------------------------- FP32 close-pair correction
// For the nodes the sweep flagged: the pairs closer than sigma_t, exactly as
// the sweep classified them, evaluated in double-float; their correction is
// added to the stored sweep sum and the cap applied. It runs at the end of
// the flagged node's brick, in the sweep's CTA and shared memory (its stalls
// are covered by the other CTAs on the SM, which are sweeping). The images
// that can be that close to one of the brick's nodes are gathered and
// converted into shared memory (in windows, in a fixed order); each flagged
// node has a thread that walks them and evaluates its close pairs.
constexpr int NEAR_CHUNK = 512;

template <int NG>
__host__ __device__ constexpr size_t fix_buf_bytes() {
    return 2 * carve(NEAR_CHUNK * sizeof(float4)) + carve(THREADS * NPT * sizeof(uint16_t)) +
           carve(THREADS * NPT * sizeof(uint8_t));
}

// gm[k]: this thread's node k, bit g set when guest g is flagged. fbuf and
// pff are shared memory free at this point; row_begin, row_off and warp_tot
// are the sweep's (free after its tile loop). Every thread of the CTA calls it.
template <int NG, int TRUNC>
__device__ __forceinline__ void fix_flagged(const GridGeom& geo, const F32GridArgs& A,
                                            const F32Params<NG, TRUNC>& P, const ff (&org)[3],
                                            int x0, int y0, int z0, const uint32_t (&gm)[NPT],
                                            unsigned char* fbuf, ParamFF* pff, uint32_t* row_begin,
                                            uint32_t* row_off, uint32_t* warp_tot, unsigned* flags) {
    SmemCarve sc{fbuf};
    float4* ahi = sc.take<float4>(NEAR_CHUNK);  // x, y, z hi, type
    float4* alo = sc.take<float4>(NEAR_CHUNK);  // x, y, z lo
    uint16_t* fnode = sc.take<uint16_t>(THREADS * NPT);  // (thread << 2) | k
    uint8_t* fmask = sc.take<uint8_t>(THREADS * NPT);    // flagged guests
    static_assert(NPT == 4 && NG <= 7, "node and guest bits (bit 7: FIX_AT_CUTOFF)");
    const ImageRecF* __restrict__ images = A.images;
    double* __restrict__ tables = A.tables;
    const int tid = threadIdx.x;
    const int nx = geo.n[0], ny = geo.n[1], nz = geo.n[2];
    const size_t plane = (size_t)nx * ny;
    const size_t per_table = plane * nz;

    uint32_t cnt_nodes = 0;
#pragma unroll
    for (int k = 0; k < NPT; ++k) cnt_nodes += gm[k] != 0;
    if (!__syncthreads_or(cnt_nodes != 0)) return;  // (every thread: a uniform vote)

    // compact the flagged nodes: exclusive scan of the per-thread counts
    uint32_t n_fn;
    {
        const int lane = tid & 31, wid = tid >> 5;
        uint32_t incl = cnt_nodes;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 31) warp_tot[wid] = incl;
        __syncthreads();
        uint32_t base = 0;
        n_fn = 0;
        for (int w = 0; w < THREADS / 32; ++w) {
            if (w < wid) base += warp_tot[w];
            n_fn += warp_tot[w];
        }
        uint32_t off = base + incl - cnt_nodes;
#pragma unroll
        for (int k = 0; k < NPT; ++k)
            if (gm[k]) {
                fnode[off] = (uint16_t)((tid << 2) | k);
                fmask[off] = (uint8_t)gm[k];
                ++off;
            }
    }
    for (int i = tid; i < geo.n_types * NG; i += THREADS)
        pff[i] = A.pff[(size_t)(i % NG) * geo.n_types + i / NG];
    float rb2 = 0.f;  // the brick's bounding radius about its centre, squared
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const float d0 = (c & 1 ? 0.5f : -0.5f) * (BX - 1), d1 = (c & 2 ? 0.5f : -0.5f) * (BY - 1),
                    d2 = (c & 4 ? 0.5f : -0.5f) * (BZ - 1);
        float q2 = 0.f;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float w = d0 * geo.sh[a] + d1 * geo.sh[3 + a] + d2 * geo.sh[6 + a];
            q2 = fmaf(w, w, q2);
        }
        rb2 = fmaxf(rb2, q2);
    }
    const float rb = sqrtf(rb2) + 1e-3f;  // 1e-3 A of margin for the FP32 tests below
    const float4* __restrict__ img4 = reinterpret_cast<const float4*>(images);  // 2 per record
    const int lane = tid & 31, wid = tid >> 5;

    // Gathers the images of rows [0, nr) that pass keep(|p|^2, type) (p: the
    // image from the brick centre, from the hi parts, off by ~1e-5 A at
    // most) into ahi / alo and calls use(count) per window of NEAR_CHUNK.
    // Warp w scans rows w, w + 8, ...: a count pass, then a pass that writes
    // each warp's images after the earlier warps' (a fixed order).
    auto gather = [&](int nr, auto keep, auto use) {
        auto passes = [&](uint32_t rec) -> bool {
            const float4 h = img4[2 * (size_t)rec];  // xh, yh, zh, type
            const float px = h.x - org[0].hi, py = h.y - org[1].hi, pz = h.z - org[2].hi;
            return keep(fmaf(px, px, fmaf(py, py, pz * pz)), __float_as_int(h.w));
        };
        uint32_t mine = 0;
        for (int r = wid; r < nr; r += THREADS / 32) {
            const uint32_t beg = row_begin[r], len = row_off[r + 1] - row_off[r];
            for (uint32_t i0 = 0; i0 < len; i0 += 32) {
                const bool k = i0 + lane < len && passes(beg + i0 + lane);
                mine += __popc(__ballot_sync(0xffffffffu, k));
            }
        }
        __syncthreads();  // earlier reads of warp_tot
        if (lane == 0) warp_tot[wid] = mine;
        __syncthreads();
        uint32_t base = 0, n_cand = 0;
        for (int w = 0; w < THREADS / 32; ++w) {
            if (w < wid) base += warp_tot[w];
            n_cand += warp_tot[w];
        }
        for (uint32_t c0 = 0; c0 < n_cand; c0 += NEAR_CHUNK) {
            const uint32_t cnt = min((uint32_t)NEAR_CHUNK, n_cand - c0);
            if (base < c0 + cnt && base + mine > c0) {  // this warp has images in the window
                uint32_t o = base;
                for (int r = wid; r < nr && o < c0 + cnt; r += THREADS / 32) {
                    const uint32_t beg = row_begin[r], len = row_off[r + 1] - row_off[r];
                    for (uint32_t i0 = 0; i0 < len; i0 += 32) {
                        const bool k = i0 + lane < len && passes(beg + i0 + lane);
                        const uint32_t b = __ballot_sync(0xffffffffu, k);
                        const uint32_t at = o + __popc(b & ((1u << lane) - 1u));
                        if (k && at >= c0 && at < c0 + cnt) {
                            const ImageRecF rr = images[beg + i0 + lane];
                            ff v[3];
                            atom_local(rr, org, v);
                            ahi[at - c0] = make_float4(v[0].hi, v[1].hi, v[2].hi, __int_as_float((int)rr.type));
                            alo[at - c0] = make_float4(v[0].lo, v[1].lo, v[2].lo, 0.f);
                        }
                        o += __popc(b);
                    }
                }
            }
            __syncthreads();
            use(cnt);
            __syncthreads();
        }
    };
    // a thread per flagged node (whose mask has any of the bits `need`):
    // body(node position, image, its lo part, guest mask, acc) per image of
    // the window, then the sums added to the node's table entries
    auto per_node = [&](uint32_t cnt, uint32_t need, auto body) {
        for (uint32_t f = tid; f < n_fn; f += THREADS) {
            const uint32_t gmask = fmask[f];
            if (!(gmask & need)) continue;
            const uint32_t node = fnode[f];
            int jx, jy, jz0;
            thread_nodes((int)(node >> 2), jx, jy, jz0);
            const int jz = jz0 + (int)(node & 3);
            ff v[3];
            node_local(geo, jx - 0.5f * (BX - 1), jy - 0.5f * (BY - 1), jz - 0.5f * (BZ - 1), v);
            ff acc[NG];
#pragma unroll
            for (int g = 0; g < NG; ++g) acc[g] = ff{0.f, 0.f};
            for (uint32_t i = 0; i < cnt; ++i) body(v, ahi[i], i, gmask, acc);
            const size_t idx = (size_t)(z0 + jz) * plane + (size_t)(y0 + jy) * nx + (x0 + jx);
#pragma unroll
            for (int g = 0; g < NG; ++g)
                if (gmask & (1u << g))
                    tables[(size_t)g * per_table + idx] += (double)acc[g].hi + (double)acc[g].lo;
        }
    };
    auto delta = [&](const float4& a, uint32_t i, const ff (&v)[3], ff& ddx, ff& ddy, ff& ddz) {
        const float4 l = alo[i];
        ddx = ff_add(ff{a.x, l.x}, ff{-v[0].hi, -v[0].lo});
        ddy = ff_add(ff{a.y, l.y}, ff{-v[1].hi, -v[1].lo});
        ddz = ff_add(ff{a.z, l.z}, ff{-v[2].hi, -v[2].lo});
    };

    // 1. the close pairs: images within rb + sigma_t of the brick centre
    // (plan_rows writes warp_tot only after a barrier of its own)
    int nr = plan_rows(geo, geo.hf_near, geo.keep2_near, A.bin_start, x0, y0, z0, row_begin,
                       row_off, warp_tot, flags);
    if (nr < 0) return;
    gather(
        nr,
        [&](float p2, int type) {
            const float reach = rb + sqrtf(P.close2[type]);
            return p2 < reach * reach;
        },
        [&](uint32_t cnt) {
            per_node(cnt, (1u << NG) - 1u, [&](const ff (&v)[3], const float4& a, uint32_t i, uint32_t gmask, ff (&acc)[NG]) {
                const int type = __float_as_int(a.w);
                if (!(r2_f32(a.x, a.y, a.z, v[0].hi, v[1].hi, v[2].hi) < P.close2[type])) return;
                ff ddx, ddy, ddz;
                delta(a, i, v, ddx, ddy, ddz);
#pragma unroll
                for (int g = 0; g < NG; ++g)
                    if (gmask & (1u << g))
                        acc[g] = ff_add(acc[g], close_pair(P, pff, type, g, ddx, ddy, ddz, geo.rcf));
            });
        });

    // 2. (plain truncation) the pairs at rc of the nodes that have one:
    // images within rb of the cutoff sphere about the brick centre; a pair
    // whose FP32 r^2 was near rc^2 gets its decision redone on the
    // double-float r^2, and where the sweep's differs its V is added or
    // taken back
    if (TRUNC == ALEA_TRUNCATED) {
        uint32_t at_cut = 0;
        for (uint32_t f = tid; f < n_fn; f += THREADS) at_cut |= fmask[f] & FIX_AT_CUTOFF;
        if (__syncthreads_or(at_cut != 0)) {
            nr = plan_rows(geo, geo.hf, geo.keep2f, A.bin_start, x0, y0, z0, row_begin, row_off,
                           warp_tot, flags);
            if (nr < 0) return;
            const float inner = fmaxf(geo.rcf - rb, 0.f), outer = geo.rcf + rb;
            const float amb2 = CUT_AMBIGUITY * geo.rc2f;
            gather(
                nr, [&](float p2, int) { return p2 > inner * inner && p2 < outer * outer; },
                [&](uint32_t cnt) {
                    per_node(cnt, FIX_AT_CUTOFF, [&](const ff (&v)[3], const float4& a, uint32_t i, uint32_t gmask, ff (&acc)[NG]) {
                        const float r2 = r2_f32(a.x, a.y, a.z, v[0].hi, v[1].hi, v[2].hi);
                        if (!(fabsf(r2 - geo.rc2f) <= amb2)) return;
                        ff ddx, ddy, ddz;
                        delta(a, i, v, ddx, ddy, ddz);
                        const ff rr = ff_add(ff_add(ff_mul(ddx, ddx), ff_mul(ddy, ddy)), ff_mul(ddz, ddz));
                        const bool in_exact = (double)rr.hi + (double)rr.lo <= geo.rc2;
                        const bool in_sweep = !(r2 > geo.rc2f);
                        if (in_exact == in_sweep) return;
                        const int type = __float_as_int(a.w);
#pragma unroll
                        for (int g = 0; g < NG; ++g)
                            if (gmask & (1u << g)) {
                                const ff e = pair_ff(pff[type * NG + g], rr);
                                acc[g] = ff_add(acc[g], in_exact ? e : ff{-e.hi, -e.lo});
                            }
                    });
                });
        }
    }
    // the cap, once every chunk's correction is in (the sweep wrote these
    // nodes' sums, uncapped, before the CTA's barriers)
    for (uint32_t jb = tid; jb < n_fn * NG; jb += THREADS) {
        const uint32_t f = jb / NG;
        const int g = (int)(jb % NG);
        if (!(fmask[f] & (1u << g))) continue;
        const uint32_t node = fnode[f];
        int jx, jy, jz0;
        thread_nodes((int)(node >> 2), jx, jy, jz0);
        const size_t idx = (size_t)(z0 + jz0 + (node & 3)) * plane + (size_t)(y0 + jy) * nx + (x0 + jx);
        double& e = tables[(size_t)g * per_table + idx];
        if (kEnergyCap < e) e = kEnergyCap;
    }
}

// One brick of the sweep (the body of the sweep kernels). Every thread of the
// block calls it; no copy of this CTA is in flight when it returns.
template <int NG, int TRUNC>
__device__ __forceinline__ void sweep_brick(const GridGeom& geo, const F32GridArgs& A, int brick,
                                            unsigned char* smem,
                                            unsigned long long* __restrict__ executed,
                                            unsigned* flags) {
    SmemCarve sc{smem};
    ImageRecF* raw = sc.take<ImageRecF>(TILE);         // the gathered tile (cp.async)
    ulonglong2* cxy = sc.take<ulonglong2>(2 * TILE);   // converted tiles: {x, x}, {y, y}
    ulonglong2* czt = sc.take<ulonglong2>(2 * TILE);   // {z, z}, {type, 0}
    uint32_t* row_begin = sc.take<uint32_t>(MAX_ROWS);
    uint32_t* row_off = sc.take<uint32_t>(MAX_ROWS + 1);
    uint32_t* warp_tot = sc.take<uint32_t>(THREADS / 32);
    F32Params<NG, TRUNC>& P = *sc.take<F32Params<NG, TRUNC>>(1);
    // double-float sweep sums (touched once per tile): hi at [(g NPT + k) 2 + 0]
    // x THREADS + tid, lo at [... + 1]
    float* accs = sc.take<float>(2 * NG * NPT * THREADS);
    float4* wsph = sc.take<float4>(THREADS / 32);  // per warp: sphere centre, cull2
    float2* wlim = sc.take<float2>(THREADS / 32);  // per warp: near2, inner2
    uint16_t* amask = sc.take<uint16_t>(2 * TILE); // per atom: 2-bit class per warp
    uint16_t* wlist = sc.take<uint16_t>((THREADS / 32) * TILE);  // per warp: atom lists
    const ImageRecF* __restrict__ images = A.images;
    const uint32_t* __restrict__ bin_start = A.bin_start;
    double* __restrict__ tables = A.tables;

    const int tid = threadIdx.x;
    const int nx = geo.n[0], ny = geo.n[1], nz = geo.n[2];
    const int bxn = geo.bricks[0], byn = geo.bricks[1];
    const int bx = brick % bxn, by = (brick / bxn) % byn, bz = brick / (bxn * byn);
    const int x0 = bx * BX, y0 = by * BY, z0 = bz * BZ;
    const float rc2f = geo.rc2f, rcf = geo.rcf;
    auto acc_hi = [&](int g, int k) -> float& { return accs[((g * NPT + k) * 2) * THREADS + tid]; };
    auto acc_lo = [&](int g, int k) -> float& { return accs[((g * NPT + k) * 2 + 1) * THREADS + tid]; };

    load_f32_params(P, A.pab, A.pff, geo.n_types, rcf);
    int nr;
    if (A.plans) {  // the brick's plan, made ahead by grid_plan_kernel
        const uint32_t* __restrict__ pl = A.plans + (size_t)brick * A.plan_stride;
        const uint32_t n = pl[0];
        if (n == ~0u) return;  // capacity flag raised; the other bricks go on
        nr = (int)n;
        for (int i = tid; i < nr; i += THREADS) row_begin[i] = pl[1 + i];
        for (int i = tid; i <= nr; i += THREADS) row_off[i] = pl[1 + nr + i];
        __syncthreads();
    } else {
        nr = plan_rows(geo, geo.hf, geo.keep2f, bin_start, x0, y0, z0, row_begin, row_off, warp_tot,
                       flags);
        if (nr < 0) return;  // capacity flag raised; the other bricks go on
    }
    const uint32_t n_cand = row_off[nr];

    int tx, ty, tz0;
    thread_nodes(tid, tx, ty, tz0);
    const int ixn = x0 + tx, iyn = y0 + ty;
    ff org[3];
    brick_origin(geo, x0, y0, z0, org);
    constexpr int NP = NPT / 2;  // node pairs per thread: nodes 2q and 2q + 1
    f2 NX[NP], NY[NP], NZ[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) {
        ff v0[3], v1[3];
        node_local(geo, tx - 0.5f * (BX - 1), ty - 0.5f * (BY - 1), tz0 + 2 * q - 0.5f * (BZ - 1), v0);
        node_local(geo, tx - 0.5f * (BX - 1), ty - 0.5f * (BY - 1), tz0 + 2 * q + 1 - 0.5f * (BZ - 1), v1);
        NX[q] = f2_pack(v0[0].hi, v1[0].hi);
        NY[q] = f2_pack(v0[1].hi, v1[1].hi);
        NZ[q] = f2_pack(v0[2].hi, v1[2].hi);
    }
    // the warp's bounding sphere: centre of its 8x4x4 sub-box, radius over its
    // nodes; 1e-3 A of margin covers FP32 rounding in the two reach tests
    {
        float wcx, wcy, wcz;
        const int w = tid >> 5;
        const float wd0 = (w & 1) * 8 + 3.5f - 0.5f * (BX - 1);
        const float wd1 = ((w >> 1) & 1) * 4 + 1.5f - 0.5f * (BY - 1);
        const float wd2 = (w >> 2) * 4 + 1.5f - 0.5f * (BZ - 1);
        wcx = wd0 * geo.sh[0] + wd1 * geo.sh[3] + wd2 * geo.sh[6];
        wcy = wd0 * geo.sh[1] + wd1 * geo.sh[4] + wd2 * geo.sh[7];
        wcz = wd0 * geo.sh[2] + wd1 * geo.sh[5] + wd2 * geo.sh[8];
        float r2max = 0.f;
#pragma unroll
        for (int k = 0; k < NPT; ++k) {
            float px, py, pz, d0, d1, d2;
            f2_unpack(NX[k / 2], d0, px);
            f2_unpack(NY[k / 2], d1, py);
            f2_unpack(NZ[k / 2], d2, pz);
            if ((k & 1) == 0) {
                px = d0;
                py = d1;
                pz = d2;
            }
            const float ex = px - wcx, ey = py - wcy, ez = pz - wcz;
            r2max = fmaxf(r2max, fmaf(ex, ex, fmaf(ey, ey, ez * ez)));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r2max = fmaxf(r2max, __shfl_xor_sync(0xffffffffu, r2max, o));
        const float rad = sqrtf(r2max) + 1e-3f;
        if ((tid & 31) == 0) {
            wsph[w] = make_float4(wcx, wcy, wcz, (geo.rcf + rad) * (geo.rcf + rad) * (1.0f + 1e-5f));
            // near: within sigma_max of some node; inner: every node within the cutoff
            const float in = geo.rcf - rad;
            wlim[w] = make_float2((geo.smaxf + rad) * (geo.smaxf + rad) * (1.0f + 1e-5f),
                                  in > 0.f ? in * in * (1.0f - 1e-5f) : -1.f);
        }
    }
    // every warp's sphere is read by every thread in the conversion of tile 0
    __syncthreads();

    float ce[NG][NPT];               // FP32 close-pair estimates
    uint32_t has_close = 0;  // bit k: node k has a close pair; bit NPT + k: a pair at rc (truncated)
    const float amb2 = CUT_AMBIGUITY * geo.rc2f;
#pragma unroll
    for (int g = 0; g < NG; ++g)
#pragma unroll
        for (int k = 0; k < NPT; ++k) {
            acc_hi(g, k) = acc_lo(g, k) = 0.f;
            ce[g][k] = 0.f;
        }
    uint32_t passes = 0;  // atoms this warp evaluated

    const unsigned char* img = reinterpret_cast<const unsigned char*>(images);
    unsigned char* rawb = reinterpret_cast<unsigned char*>(raw);
    const uint32_t n_tiles = (n_cand + TILE - 1) / TILE;
    // One staging buffer, in which thread tid's slot holds the record that
    // thread tid gathered and converts, and two converted-tile buffers: the
    // conversion of tile t writes buffer t & 1, last read by the main loop of
    // tile t - 2, which every warp finished before the barrier of tile t - 1;
    // so one barrier per tile.
    if (n_tiles > 0) gather_tile(0, n_cand, nr, row_begin, row_off, img, rawb);
    for (uint32_t t = 0; t < n_tiles; ++t) {
        const uint32_t cnt = min((uint32_t)TILE, n_cand - t * TILE);
        ulonglong2* cxy_t = cxy + (t & 1) * TILE;
        ulonglong2* czt_t = czt + (t & 1) * TILE;
        uint16_t* amask_t = amask + (t & 1) * TILE;
        cp_async_wait_all();  // this thread's record of tile t
        static_assert(TILE == THREADS, "one record per thread in the conversion pass");
        static_assert(TILE <= 32768 && THREADS / 32 <= 8, "list entry and class-mask widths");
        if ((uint32_t)tid < cnt) {
            ff v[3];
            const ImageRecF r = raw[tid];
            atom_local(r, org, v);
            cxy_t[tid] = make_ulonglong2(f2_pack(v[0].hi, v[0].hi), f2_pack(v[1].hi, v[1].hi));
            czt_t[tid] = make_ulonglong2(f2_pack(v[2].hi, v[2].hi), (unsigned long long)r.type);
            // this atom's class for each warp (2 bits per warp): 0 beyond the
            // warp's reach, 1 inner, 2 boundary, 3 near
            uint32_t m = 0;
#pragma unroll
            for (int w = 0; w < THREADS / 32; ++w) {
                const float4 c = wsph[w];
                const float2 lim = wlim[w];
                const float ex = v[0].hi - c.x, ey = v[1].hi - c.y, ez = v[2].hi - c.z;
                const float d2w = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
                const uint32_t cls = d2w > c.w ? 0u : d2w < lim.x ? 3u : d2w <= lim.y ? 1u : 2u;
                m |= cls << (2 * w);
            }
            amask_t[tid] = (uint16_t)m;
        }
        __syncthreads();
        // the staging buffer is free again: gather tile t + 1 while computing
        if (t + 1 < n_tiles) gather_tile(t + 1, n_cand, nr, row_begin, row_off, img, rawb);
        // this warp's atoms: inner ones from the front of its list (tile
        // order), the others from the back; the shift sum over both (every
        // lane of the warp needs the same sum)
        uint32_t n_in = 0, n_out = 0;
        uint16_t* mine_list = wlist + (tid >> 5) * TILE;
        float shift_sum[NG];
        {
            const int w = tid >> 5, lane = tid & 31;
            const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
            for (int g = 0; g < NG; ++g) shift_sum[g] = 0.f;
#pragma unroll 4  // the class loads and ballots of several chunks in flight
            for (uint32_t c0 = 0; c0 < cnt; c0 += 32) {
                const uint32_t j = c0 + lane;
                const uint32_t cls = j < cnt ? (amask_t[j] >> (2 * w)) & 3u : 0u;
                const uint32_t b_in = __ballot_sync(0xffffffffu, cls == 1u);
                const uint32_t b_out = __ballot_sync(0xffffffffu, cls >= 2u);
                if (cls == 1u) mine_list[n_in + __popc(b_in & lt)] = (uint16_t)j;
                if (cls >= 2u)
                    mine_list[TILE - 1 - (n_out + __popc(b_out & lt))] = (uint16_t)((j << 1) | (cls & 1u));
                if (TRUNC != ALEA_TRUNCATED && cls) {
                    const int type = (int)(uint32_t)czt_t[j].y;
#pragma unroll
                    for (int g = 0; g < NG; ++g) shift_sum[g] += P.shift[type * NG + g];
                }
                n_in += __popc(b_in);
                n_out += __popc(b_out);
            }
            if (TRUNC != ALEA_TRUNCATED) {
#pragma unroll
                for (int g = 0; g < NG; ++g)
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1)
                        shift_sum[g] += __shfl_xor_sync(0xffffffffu, shift_sum[g], o);
            }
            __syncwarp();
        }
        passes += n_in + n_out;
        f2 part[NG][NP];
#pragma unroll
        for (int g = 0; g < NG; ++g)
#pragma unroll
            for (int q = 0; q < NP; ++q) part[g][q] = 0ull;  // {+0, +0}
        // one atom against this thread's nodes; LO: clamp r^2 from below at
        // sigma_t^2, HI: clamp (or cut) at the cutoff
        auto add_atom = [&](uint32_t j, auto lo_tag, auto hi_tag) {
            constexpr bool LO = decltype(lo_tag)::value, HI = decltype(hi_tag)::value;
            const ulonglong2 xy = cxy_t[j];
            const ulonglong2 zt = czt_t[j];
            const int type = (int)(uint32_t)zt.y;
            float close2 = 0.f;
            if (LO) close2 = P.close2[type];
            ulonglong2 AB[NG];
#pragma unroll
            for (int g = 0; g < NG; ++g) AB[g] = P.ab[type * NG + g];
            if (LO) {  // this atom may be closer than sigma_t to a node
                float ax, ay, az, dummy;
                f2_unpack(xy.x, ax, dummy);
                f2_unpack(xy.y, ay, dummy);
                f2_unpack(zt.x, az, dummy);
#pragma unroll
                for (int k = 0; k < NPT; ++k) {
                    float p[2][3];
                    f2_unpack(NX[k / 2], p[0][0], p[1][0]);
                    f2_unpack(NY[k / 2], p[0][1], p[1][1]);
                    f2_unpack(NZ[k / 2], p[0][2], p[1][2]);
                    const float r2 = r2_f32(ax, ay, az, p[k & 1][0], p[k & 1][1], p[k & 1][2]);
                    if (r2 < close2) {
                        has_close |= 1u << k;
                        const float ir2 = rcp_approx(fmaxf(r2, 1e-4f));
                        const float ir6 = ir2 * ir2 * ir2;
#pragma unroll
                        for (int g = 0; g < NG; ++g) {
                            float a, nb, dm;
                            f2_unpack(AB[g].x, a, dm);
                            f2_unpack(AB[g].y, nb, dm);
                            float v = ir6 * fmaf(a, ir6, nb) - P.vclose[type * NG + g];
                            if (TRUNC == ALEA_LINEAR_FORCE_SHIFTED)
                                v -= (sqrtf(fmaxf(r2, 1e-4f)) - rcf) * P.dvdrc[type * NG + g];
                            ce[g][k] += v;
                        }
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < NP; ++q) {
                const f2 dx = f2_sub(xy.x, NX[q]);
                const f2 dy = f2_sub(xy.y, NY[q]);
                const f2 dz = f2_sub(zt.x, NZ[q]);
                const f2 r2 = f2_fma(dx, dx, f2_fma(dy, dy, f2_mul(dz, dz)));
                float r2a, r2b;
                f2_unpack(r2, r2a, r2b);
                float ia, ib;
                if (TRUNC == ALEA_TRUNCATED) {
                    ia = rcp_approx(LO ? fmaxf(r2a, close2) : r2a);
                    ib = rcp_approx(LO ? fmaxf(r2b, close2) : r2b);
                    if (HI) {
                        ia = r2a > rc2f ? 0.f : ia;
                        ib = r2b > rc2f ? 0.f : ib;
                        // V jumps at rc: a pair this near it may lie on the
                        // other side in exact arithmetic (node to correction)
                        if (fabsf(r2a - rc2f) <= amb2) has_close |= 1u << (NPT + 2 * q);
                        if (fabsf(r2b - rc2f) <= amb2) has_close |= 1u << (NPT + 2 * q + 1);
                    }
                } else {
                    if (LO) {
                        r2a = fmaxf(r2a, close2);
                        r2b = fmaxf(r2b, close2);
                    }
                    if (HI) {
                        r2a = fminf(r2a, rc2f);
                        r2b = fminf(r2b, rc2f);
                    }
                    ia = rcp_approx(r2a);
                    ib = rcp_approx(r2b);
                }
                const f2 ir2 = f2_pack(ia, ib);
                const f2 ir6 = f2_mul(ir2, f2_mul(ir2, ir2));
#pragma unroll
                for (int g = 0; g < NG; ++g) part[g][q] = f2_fma(ir6, f2_fma(AB[g].x, ir6, AB[g].y), part[g][q]);
                if (TRUNC == ALEA_LINEAR_FORCE_SHIFTED) {
                    const f2 dr = f2_pack(__fsub_rn(__fmul_rn(r2a, rsqrtf(r2a)), rcf),
                                          __fsub_rn(__fmul_rn(r2b, rsqrtf(r2b)), rcf));
#pragma unroll
                    for (int g = 0; g < NG; ++g) {
                        const float md = -P.dvdrc[type * NG + g];
                        part[g][q] = f2_fma(f2_pack(md, md), dr, part[g][q]);
                    }
                }
            }
        };
        using yes = std::true_type;
        using no = std::false_type;
        // inner atoms: every node of the warp within the cutoff and none
        // closer than sigma_t, so neither clamp can act
        for (uint32_t u = 0; u < n_in; ++u) add_atom(mine_list[u], no{}, no{});
        for (uint32_t u = TILE - n_out; u < TILE; ++u) {
            const uint32_t e = mine_list[u];
            if (e & 1u)  // warp-uniform
                add_atom(e >> 1, yes{}, yes{});
            else
                add_atom(e >> 1, no{}, yes{});
        }
#pragma unroll
        for (int g = 0; g < NG; ++g)
#pragma unroll
            for (int q = 0; q < NP; ++q) {
                float pa, pb;
                f2_unpack(part[g][q], pa, pb);
                const ff sa = ff_add_f(ff{acc_hi(g, 2 * q), acc_lo(g, 2 * q)}, pa - shift_sum[g]);
                const ff sb = ff_add_f(ff{acc_hi(g, 2 * q + 1), acc_lo(g, 2 * q + 1)}, pb - shift_sum[g]);
                acc_hi(g, 2 * q) = sa.hi;
                acc_lo(g, 2 * q) = sa.lo;
                acc_hi(g, 2 * q + 1) = sb.hi;
                acc_lo(g, 2 * q + 1) = sb.lo;
            }
    }

    // per node and guest: sweep sum, cap, sweep sum + FP32 estimate, or the
    // sweep sum flagged for the double-float correction
    // (the cap: framework_energy_grid.cc:22, 243)
    const size_t plane = (size_t)nx * ny;
    const size_t per_table = plane * nz;
    uint32_t mine = 0;
    uint32_t gm[NPT];  // per node: guests flagged for the correction
#pragma unroll
    for (int k = 0; k < NPT; ++k) {
        gm[k] = 0;
        const int izn = z0 + tz0 + k;
        if (ixn < nx && iyn < ny && izn < nz) {
            const size_t idx = (size_t)izn * plane + (size_t)iyn * nx + ixn;
#pragma unroll
            for (int g = 0; g < NG; ++g) {
                const double e = (double)acc_hi(g, k) + (double)acc_lo(g, k);
                double out = e;
                bool f = false;
                // (truncated) a pair at rc: the correction redoes its cutoff
                // decision, and the node's close pairs with it
                const bool amb = TRUNC == ALEA_TRUNCATED && ((has_close >> (NPT + k)) & 1u);
                if (has_close & (1u << k)) {
                    const double est = e + (double)ce[g][k];
                    if (est > 1.01 * kEnergyCap)
                        out = kEnergyCap;
                    else if (!amb && fabsf(ce[g][k]) <= CLOSE_FP32_RATIO * fmaxf(CLOSE_FP32_FLOOR, (float)fabs(est)))
                        out = est;
                    else
                        f = true;
                } else {
                    f = amb;
                }
                tables[(size_t)g * per_table + idx] = (!f && kEnergyCap < out) ? kEnergyCap : out;
                gm[k] |= (uint32_t)f << g;
                if (f && amb) gm[k] |= FIX_AT_CUTOFF;
            }
            mine += passes;
        }
    }
    // node-image pairs evaluated: atoms past the warp cull x nodes in the grid
    mine = __reduce_add_sync(0xffffffffu, mine);
    __syncthreads();  // warp_tot is free after the tile loop
    if ((tid & 31) == 0) warp_tot[tid >> 5] = mine;
    __syncthreads();
    if (tid == 0) {
        unsigned long long sum = 0;
        for (int w = 0; w < THREADS / 32; ++w) sum += warp_tot[w];
        atomicAdd(executed, sum);
    }
    // the flagged nodes' close pairs; the staging and converted-tile buffers
    // and the accumulators are free now (the vote in fix_flagged is the
    // barrier after the last reads of warp_tot and the accumulators)
    static_assert(fix_buf_bytes<NG>() <= carve(TILE * sizeof(ImageRecF)) + 2 * carve(2 * TILE * sizeof(ulonglong2)),
                  "correction buffers fit the tile buffers");
    static_assert(64 * NG * sizeof(ParamFF) <= 2 * NG * NPT * THREADS * sizeof(float),
                  "double-float parameters fit the accumulators");
    fix_flagged<NG, TRUNC>(geo, A, P, org, x0, y0, z0, gm, smem, reinterpret_cast<ParamFF*>(accs),
                           row_begin, row_off, warp_tot, flags);
    __syncthreads();  // shared memory is reused by the next brick
}

// 4 CTAs per SM fit in shared memory up to two guests, 3 beyond
template <int NG, int TRUNC>
__global__ void __launch_bounds__(THREADS, NG <= 2 ? 4 : 3)
grid_build_f32_kernel(GridGeom geo, F32GridArgs args, unsigned long long* __restrict__ executed,
                      unsigned* flags) {
    extern __shared__ __align__(128) unsigned char smem[];
    sweep_brick<NG, TRUNC>(geo, args, geo.brick0 + (int)blockIdx.x, smem, executed, flags);
}

template <int NG, int TRUNC>
constexpr size_t f32_smem_bytes() {
    return carve(TILE * sizeof(ImageRecF)) + carve(2 * TILE * sizeof(ulonglong2)) +
           carve(2 * TILE * sizeof(ulonglong2)) + carve(MAX_ROWS * sizeof(uint32_t)) +
           carve((MAX_ROWS + 1) * sizeof(uint32_t)) + carve((THREADS / 32) * sizeof(uint32_t)) +
           carve(sizeof(F32Params<NG, TRUNC>)) + carve(2 * NG * NPT * THREADS * sizeof(float)) +
           carve((THREADS / 32) * sizeof(float4)) + carve((THREADS / 32) * sizeof(float2)) +
           carve(2 * TILE * sizeof(uint16_t)) + carve((THREADS / 32) * TILE * sizeof(uint16_t));
}

// ---------------------------------------------------------------- batched FP32 build
// Many independent grids (uneven frameworks: their own cells, atoms, force
// fields and node counts) in one persistent launch per kernel: every CTA takes
// (grid, brick) work items from a global counter (dynamic, so uneven grids
// balance) and runs the same per-brick code as the single-grid kernels, with
// the item's geometry copied into shared memory. The results are those of
// building each grid alone, bit for bit: every brick is computed the same way
// whichever CTA takes it.
struct BatchItem {
    GridGeom geo;
    F32GridArgs args;
    uint64_t brick0;  // first work item of this grid
};

__device__ __forceinline__ bool next_item(const BatchItem* __restrict__ items, int n_items,
                                          uint64_t total, unsigned long long* next,
                                          unsigned long long& work, int& item, GridGeom& geo) {
    if (threadIdx.x == 0) {
        work = atomicAdd(next, 1ull);
        if (work < total) {
            int lo = 0, hi = n_items - 1;  // last grid with brick0 <= work
            while (lo < hi) {
                const int mid = (lo + hi + 1) / 2;
                if (items[mid].brick0 <= work) lo = mid; else hi = mid - 1;
            }
            item = lo;
        }
    }
    __syncthreads();
    if (work >= total) return false;
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&items[item].geo);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&geo);
    for (int i = threadIdx.x; i < (int)(sizeof(GridGeom) / 4); i += THREADS) dst[i] = src[i];
    __syncthreads();
    return true;
}

template <int NG, int TRUNC, int MINB>
__global__ void __launch_bounds__(THREADS, MINB)
grid_build_f32_batch_kernel(const BatchItem* __restrict__ items, int n_items, uint64_t total,
                            unsigned long long* next, unsigned long long* __restrict__ executed,
                            unsigned* flags) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ unsigned long long work;
    __shared__ int item;
    GridGeom& geo = *reinterpret_cast<GridGeom*>(smem);
    unsigned char* body = smem + carve(sizeof(GridGeom));
    static_assert(sizeof(GridGeom) % 4 == 0, "geometry copied as words");
    while (next_item(items, n_items, total, next, work, item, geo)) {
        const BatchItem& it = items[item];
        sweep_brick<NG, TRUNC>(geo, it.args, (int)(work - it.brick0), body, executed, flags);
        __syncthreads();  // work, item and geo are rewritten next
    }
}

// The batched launch shapes the autotuner chooses between.
constexpr int BATCH_VARIANTS = 2;  // 0: 3 sweep blocks per SM, 1: 4

template <int NG, int TRUNC>
void batch_launch_t(int variant, int sms, cudaStream_t s, const BatchItem* items, int n_items,
                    uint64_t total, unsigned long long* counters, unsigned long long* executed,
                    unsigned* flags) {
    const size_t sb = carve(sizeof(GridGeom)) + f32_smem_bytes<NG, TRUNC>();
    auto sweep = variant == 0 ? grid_build_f32_batch_kernel<NG, TRUNC, 3>
                              : grid_build_f32_batch_kernel<NG, TRUNC, 4>;
    ALEA_CUDA(cudaFuncSetAttribute(sweep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb));
    int per_sm = 1;
    ALEA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep, THREADS, sb));
    const unsigned gs = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(total, (uint64_t)sms * std::max(per_sm, 1)));
    ALEA_CUDA(cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned long long), s));
    sweep<<<gs, THREADS, sb, s>>>(items, n_items, total, counters, executed, flags);
    ALEA_CUDA(cudaGetLastError());
}

void batch_launch(int ng, int trunc, int variant, int sms, cudaStream_t s, const BatchItem* items,
                  int n_items, uint64_t total, unsigned long long* counters,
                  unsigned long long* executed, unsigned* flags) {
#define ALEA_BATCH_T(NGV)                                                                          \
    if (trunc == ALEA_TRUNCATED)                                                                   \
        batch_launch_t<NGV, ALEA_TRUNCATED>(variant, sms, s, items, n_items, total, counters, executed, flags); \
    else if (trunc == ALEA_SHIFTED)                                                                \
        batch_launch_t<NGV, ALEA_SHIFTED>(variant, sms, s, items, n_items, total, counters, executed, flags);   \
    else                                                                                           \
        batch_launch_t<NGV, ALEA_LINEAR_FORCE_SHIFTED>(variant, sms, s, items, n_items, total, counters, executed, flags);
    switch (ng) {
        case 1: ALEA_BATCH_T(1) break;
        case 2: ALEA_BATCH_T(2) break;
        case 3: ALEA_BATCH_T(3) break;
        default: ALEA_BATCH_T(4) break;
    }
#undef ALEA_BATCH_T
}

// ---------------------------------------------------------------- interpolation
// framework_energy_grid.cc:251-288, with non-contracted FP64 arithmetic so the
// result matches the reference's rounding sequence.
__global__ void grid_interpolate_kernel(Lattice L, int nx, int ny, int nz,
                                        const double* __restrict__ table,
                                        const double* __restrict__ xyz, uint64_t n,
                                        double* __restrict__ out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = grid_interp_ref(L, nx, ny, nz, table, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
}

// Grids built in the FP32 form: the same trilinear interpolation with the
// fractional transform as multiplies by the inverse cell (no IEEE divisions)
// and fused lerps: about 40 FP64 operations per query instead of about 100,
// within ~1e-12 relative of the reference form's value (not bit-equal).
// FP32-form grids: a persistent grid-stride loop, one query per thread and
// turn: locate in double-float, the eight corner loads issued together
// (predicated, no early exit, so the warp's gathers stay in flight together),
// then the blend; a query outside the double-float range goes to FP64.
__global__ void __launch_bounds__(256)
grid_interpolate_fast_kernel(Lattice L, InvFF inv, int nx, int ny, int nz,
                             const double* __restrict__ table, const double* __restrict__ xyz,
                             uint64_t n, double* __restrict__ out) {
    const int cnt[3] = {nx, ny, nz};
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double px = xyz[3 * i], py = xyz[3 * i + 1], pz = xyz[3 * i + 2];
        int i0[3], i1[3];
        ff t[3];
        const bool ok = grid_ff_locate(inv, cnt, px, py, pz, i0, i1, t);
        double c[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int ix = (k & 1) ? i1[0] : i0[0], iy = (k & 2) ? i1[1] : i0[1],
                      iz = (k & 4) ? i1[2] : i0[2];
            c[k] = ok ? __ldg(&table[((size_t)iz * ny + iy) * nx + ix]) : 0.0;
        }
        double r;
        if (!ok || !grid_ff_blend(c, t, r)) r = grid_interp_fast(L, nx, ny, nz, table, px, py, pz);
        out[i] = r;
    }
}

// The corner blocks of an FP32-form table: node i's eight corners (k = x + 2y
// + 4z, 0 the node, 1 the next node along that axis with wrap) as four
// double2, grid_ff_blend's order.
__global__ void grid_corners_kernel(int nx, int ny, int nz, const double* __restrict__ t,
                                    double2* __restrict__ out) {
    const uint64_t nodes = (uint64_t)nx * ny * nz;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nodes; i += stride) {
        const int ix = (int)(i % nx);
        const uint64_t r = i / nx;
        const int iy = (int)(r % ny), iz = (int)(r / ny);
        const int jx = ix + 1 == nx ? 0 : ix + 1, jy = iy + 1 == ny ? 0 : iy + 1,
                  jz = iz + 1 == nz ? 0 : iz + 1;
        auto V = [&](int x, int y, int z) { return __ldg(&t[((size_t)z * ny + y) * nx + x]); };
        out[4 * i] = make_double2(V(ix, iy, iz), V(jx, iy, iz));
        out[4 * i + 1] = make_double2(V(ix, jy, iz), V(jx, jy, iz));
        out[4 * i + 2] = make_double2(V(ix, iy, jz), V(jx, iy, jz));
        out[4 * i + 3] = make_double2(V(ix, jy, jz), V(jx, jy, jz));
    }
}

// FP32-form grids with their corner blocks: as grid_interpolate_fast_kernel,
// the eight corners read as one aligned 64-byte block (one DRAM row) instead
// of four 16-byte pairs in four rows.
__global__ void __launch_bounds__(256)
grid_interpolate_corners_kernel(Lattice L, InvFF inv, int nx, int ny, int nz,
                                const double2* __restrict__ corners,
                                const double* __restrict__ table, const double* __restrict__ xyz,
                                uint64_t n, double* __restrict__ out) {
    const int cnt[3] = {nx, ny, nz};
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double px = xyz[3 * i], py = xyz[3 * i + 1], pz = xyz[3 * i + 2];
        int i0[3], i1[3];
        ff t[3];
        const bool ok = grid_ff_locate(inv, cnt, px, py, pz, i0, i1, t);
        const uint64_t node = ok ? ((uint64_t)i0[2] * ny + i0[1]) * nx + i0[0] : 0;
        double c[8];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const double2 v = __ldg(&corners[4 * node + k]);
            c[2 * k] = v.x;
            c[2 * k + 1] = v.y;
        }
        double r;
        if (!ok || !grid_ff_blend(c, t, r)) r = grid_interp_fast(L, nx, ny, nz, table, px, py, pz);
        out[i] = r;
    }
}

struct BuildArgs {
    const ImageRec* images;      // FP64 form
    const ImageRecF* images_f;   // FP32 form
    const uint32_t* bins;
    const PairParams* params;    // FP64 form: mixed table, indexed through guests
    const uint32_t* guests;
    const ParamAB* pab;          // FP32 form: [guest of this launch][type]
    const ParamFF* pff;
    double* tables;
    unsigned long long* executed;
    unsigned* flags;
    unsigned tile_wait;          // FP64 form: polls before a tile wait gives up
    const uint32_t* plans;       // FP32 form: the row plans of grid_plan_kernel
    uint32_t plan_stride;
};

template <int NG, int TRUNC>
void launch_one(bool f32, dim3 grid, cudaStream_t s, const GridGeom& geo, const BuildArgs& a) {
    if (f32) {
        constexpr size_t bytes = f32_smem_bytes<NG, TRUNC>();
        // opt in to more than 48 KB of dynamic shared memory (per device, cheap)
        ALEA_CUDA(cudaFuncSetAttribute(grid_build_f32_kernel<NG, TRUNC>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
        const F32GridArgs fa{a.images_f, a.bins, a.pab, a.pff, a.tables, a.plans, a.plan_stride};
        grid_build_f32_kernel<NG, TRUNC><<<grid, THREADS, bytes, s>>>(geo, fa, a.executed, a.flags);
    } else {
        constexpr size_t bytes = f64_smem_bytes<NG>();
        ALEA_CUDA(cudaFuncSetAttribute(grid_build_f64_kernel<NG, TRUNC>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
        grid_build_f64_kernel<NG, TRUNC><<<grid, THREADS, bytes, s>>>(
            geo, a.images, a.bins, a.params, a.guests, a.tables, a.executed, a.flags, a.tile_wait);
    }
}

template <int NG>
void launch_trunc(int trunc, bool f32, dim3 grid, cudaStream_t s, const GridGeom& geo,
                  const BuildArgs& a) {
    if (trunc == ALEA_TRUNCATED)
        launch_one<NG, ALEA_TRUNCATED>(f32, grid, s, geo, a);
    else if (trunc == ALEA_SHIFTED)
        launch_one<NG, ALEA_SHIFTED>(f32, grid, s, geo, a);
    else
        launch_one<NG, ALEA_LINEAR_FORCE_SHIFTED>(f32, grid, s, geo, a);
}

void launch_build(int ng, int trunc, bool f32, dim3 grid, cudaStream_t s, const GridGeom& geo,
                  const BuildArgs& a) {
    switch (ng) {
        case 1: launch_trunc<1>(trunc, f32, grid, s, geo, a); break;
        case 2: launch_trunc<2>(trunc, f32, grid, s, geo, a); break;
        case 3: launch_trunc<3>(trunc, f32, grid, s, geo, a); break;
        default: launch_trunc<4>(trunc, f32, grid, s, geo, a); break;
    }
}

}  // namespace

// ---------------------------------------------------------------- host plan
struct GridImpl {
    GridGeom geo{};
    int precision = ALEA_FP64;
    int truncation = ALEA_SHIFTED;
    double spacing = 0;
    uint64_t n_atoms = 0;
    std::vector<uint32_t> species;  // sorted distinct guest species
    DevBuf<ImageRec> images;     // FP64 form
    DevBuf<ImageRecF> images_f;  // FP32 form
    DevBuf<ParamAB> pab;         // FP32 form, [guest][type]
    DevBuf<ParamFF> pff;
    DevBuf<uint32_t> bin_start;
    DevBuf<uint32_t> plans;      // FP32 form: the bricks' row plans (grid_plan_kernel)
    uint32_t plan_stride = 0;    // words a brick: 2 + 2 x the most rows a brick can touch
    DevBuf<PairParams> params;
    DevBuf<uint32_t> guests;
    DevBuf<double> tables;
    DevBuf<unsigned long long> executed;
    DevBuf<unsigned> flags;
    uint64_t n_images = 0;
    uint64_t executed_pairs = 0;
    bool min_image = false;  // rc > L_perp/2: the reference's minimum-image loop (MiGeom)
    MiGeom mg{};
    float last_ms = 0.f;
    int launches = 0;
    // FP32-form grids: per species, the eight trilinear corners of every node
    // stored together (64 B a node), made on the first device interpolation of
    // that species and remade after a build (gen counts the builds)
    uint64_t gen = 0;
    std::vector<DevBuf<double2>> corners;
    std::vector<uint64_t> corners_gen;
    // recorded after each species' corner kernel: an interpolation on another
    // stream waits on it before reading the blocks
    struct EventDel {
        void operator()(CUevent_st* e) const { cudaEventDestroy(e); }
    };
    std::vector<std::unique_ptr<CUevent_st, EventDel>> corners_ev;
    bool corners_off = false;  // their allocation failed once: the plain table serves
    std::mutex corners_mu;     // interpolations from several host threads share them
};

// Initial bin width (A). The FP64 kernel evaluates every candidate against
// every node of its brick, so narrow bins (fewer candidates) pay; the FP32
// sweep culls per warp and gathers each record on its own, so its cost is per
// bin row (planning, list building) and wider bins pay: 4 A bins build the
// 4x4x4 supercell's 0.2 A grid in 19.4 ms against 21.9 ms with 2 A bins.
static double bin_width(int precision) { return precision == ALEA_FP32 ? 4.0 : 2.0; }

static void build_plan(GridImpl& g, const alea_lennard_jones& lj, const alea_particles& fw,
                       const alea_lattice& lat, const uint32_t* guest, uint32_t n_guest,
                       double spacing, int precision, double bin_width) {
    require(spacing > 0.0, ALEA_ERR_INVALID_ARGUMENT,
            "FrameworkEnergyGrid: spacingAngstrom must be positive");
    require(lj.cutoff > 0.0, ALEA_ERR_INVALID_ARGUMENT, "LennardJones: cutoff must be positive");
    require(lj.n_species > 0 && lj.n_species <= 64, ALEA_ERR_INVALID_ARGUMENT,
            "alea_grid_build: 1..64 LJ species supported");
    require(precision == ALEA_FP64 || precision == ALEA_FP32, ALEA_ERR_INVALID_ARGUMENT,
            "alea_grid_build: precision must be ALEA_FP64 or ALEA_FP32");
    require(lj.truncation >= 0 && lj.truncation <= 2, ALEA_ERR_INVALID_ARGUMENT,
            "alea_grid_build: unknown truncation");
    require(fw.n == 0 || (fw.x && fw.y && fw.z), ALEA_ERR_INVALID_ARGUMENT,
            "alea_grid_build: framework coordinates missing");
    g.geo.L = make_lattice(lat.m);
    // the reference's constructor takes any cutoff: above L_perp/2 its
    // minimum-image sum is restated by grid_build_mi_kernel (FP64)
    for (int a = 0; a < 3; ++a) g.min_image |= lj.cutoff > 0.5 * g.geo.L.perp[a];
    g.precision = g.min_image ? ALEA_FP64 : precision;
    g.truncation = lj.truncation;
    g.spacing = spacing;
    g.n_atoms = fw.n;
    for (int a = 0; a < 3; ++a) {
        const long n = lround(g.geo.L.perp[a] / spacing);  // framework_energy_grid.cc:207-211
        g.geo.n[a] = n < 1 ? 1 : (int)n;
    }
    std::vector<uint32_t> sp(guest, guest + n_guest);
    std::sort(sp.begin(), sp.end());
    sp.erase(std::unique(sp.begin(), sp.end()), sp.end());
    for (uint32_t s : sp)
        require(s < lj.n_species, ALEA_ERR_OUT_OF_RANGE,
                "FrameworkEnergyGrid: guest species id out of range of the force field");
    for (uint64_t i = 0; i < fw.n; ++i)
        require(!fw.species || fw.species[i] < lj.n_species, ALEA_ERR_OUT_OF_RANGE,
                "FrameworkEnergyGrid: framework species id out of range of the force field");
    g.species = sp;
    const int ng = (int)sp.size();
    require_device();  // every check above runs without a GPU
    if (g.min_image) {
        MiGeom& G = g.mg;
        for (int i = 0; i < 9; ++i) G.m[i] = g.geo.L.m[i];
        G.ortho = g.geo.L.ortho;
        reduced_basis(G.m, G.r);
        auto cross = [](const double* a, const double* b, double* o) {
            o[0] = a[1] * b[2] - a[2] * b[1];
            o[1] = a[2] * b[0] - a[0] * b[2];
            o[2] = a[0] * b[1] - a[1] * b[0];
        };
        cross(G.r + 3, G.r + 6, G.t0);
        cross(G.r + 6, G.r, G.t1);
        cross(G.r, G.r + 3, G.t2);
        G.rvol = G.r[0] * G.t0[0] + G.r[1] * G.t0[1] + G.r[2] * G.t0[2];
        for (int a = 0; a < 3; ++a) G.n[a] = g.geo.n[a];
        G.rc = lj.cutoff;
        G.trunc = lj.truncation;
        G.n_species = lj.n_species;
        std::vector<ImageRec> at(fw.n);
        for (uint64_t i = 0; i < fw.n; ++i)
            at[i] = ImageRec{fw.x[i], fw.y[i], fw.z[i], fw.species ? fw.species[i] : 0u, 0u};
        g.images.alloc(std::max<size_t>(fw.n, 1));
        g.images.upload(at.data(), fw.n);
        g.n_images = fw.n;
        std::vector<PairParams> tab((size_t)lj.n_species * lj.n_species);
        mixed_table(lj, tab.data());
        g.params.alloc(tab.size());
        g.params.upload(tab.data(), tab.size());
        g.guests.alloc(std::max(ng, 1));
        g.guests.upload(sp.data(), sp.size());
        g.tables.alloc((size_t)g.geo.n[0] * g.geo.n[1] * g.geo.n[2] * std::max(ng, 1));
        g.executed.alloc(1);
        g.flags.alloc(1);
        ALEA_CUDA(cudaMemset(g.flags.p, 0, sizeof(unsigned)));
        return;
    }

    // metric tensor and extents
    const double* m = g.geo.L.m;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            g.geo.Gf[3 * i + j] = (float)(m[3 * i] * m[3 * j] + m[3 * i + 1] * m[3 * j + 1] +
                                          m[3 * i + 2] * m[3 * j + 2]);
    for (int i = 0; i < 3; ++i) g.geo.Ginvf[i] = 1.0f / g.geo.Gf[4 * i];
    g.geo.rc = lj.cutoff;
    g.geo.rc2 = lj.cutoff * lj.cutoff;
    g.geo.rcf = (float)lj.cutoff;
    g.geo.rc2f = (float)g.geo.rc2;
    g.geo.irc2f = (float)(1.0 / g.geo.rc2);
    g.geo.keep2f = (float)(g.geo.rc2 * (1.0 + 1e-3) + 1e-2);
    for (int a = 0; a < 3; ++a) {
        g.geo.inv_nf[a] = (float)(1.0 / g.geo.n[a]);
        g.geo.hf[a] = (float)(lj.cutoff / g.geo.L.perp[a]);
        for (int c = 0; c < 3; ++c) {
            const double v = m[3 * a + c] / g.geo.n[a];
            g.geo.sh[3 * a + c] = (float)v;
            g.geo.sl[3 * a + c] = (float)(v - (double)g.geo.sh[3 * a + c]);
        }
    }
    // widen the bins until no brick can touch more than MAX_ROWS bin rows
    int span_bins[3] = {0, 0, 0};
    for (int attempt = 0; attempt < 64; ++attempt) {
        for (int a = 0; a < 3; ++a) {
            const double h = lj.cutoff / g.geo.L.perp[a];
            const double span = (double)(g.geo.n[a] - 1) / g.geo.n[a] + 2 * h + 2e-7;
            const int nb = std::max(1, (int)std::ceil(span * g.geo.L.perp[a] / bin_width));
            const double bw = span / nb;
            const int bd = a == 0 ? BX : a == 1 ? BY : BZ;
            span_bins[a] = std::min(nb, (int)std::ceil(((double)(bd - 1) / g.geo.n[a] + 2 * h) / bw) + 4);
        }
        if (span_bins[1] * span_bins[2] <= MAX_ROWS) break;
        bin_width *= 1.25;
    }
    // plan_rows spans at most span_bins[a] bins on axes 1 and 2 (its margins
    // are a bin narrower than the 4 added here)
    g.plan_stride = 2 + 2 * (uint32_t)std::min(span_bins[1] * span_bins[2], MAX_ROWS);
    for (int a = 0; a < 3; ++a) {
        const double h = lj.cutoff / g.geo.L.perp[a];
        g.geo.lo[a] = -h - 1e-7;
        g.geo.hi[a] = (double)(g.geo.n[a] - 1) / g.geo.n[a] + h + 1e-7;
        const double span = g.geo.hi[a] - g.geo.lo[a];
        g.geo.nb[a] = std::max(1, (int)std::ceil(span * g.geo.L.perp[a] / bin_width));
        g.geo.binw[a] = span / g.geo.nb[a];
        g.geo.lof[a] = (float)g.geo.lo[a];
        g.geo.binwf[a] = (float)g.geo.binw[a];
        g.geo.inv_binwf[a] = (float)(1.0 / g.geo.binw[a]);
        g.geo.bricks[a] = (g.geo.n[a] + (a == 0 ? BX : a == 1 ? BY : BZ) - 1) /
                          (a == 0 ? BX : a == 1 ? BY : BZ);
    }
    g.geo.n_types = (int)lj.n_species;

    // periodic images within the extended fractional range, binned
    std::vector<ImageRec> recs;
    std::vector<uint32_t> keys;
    recs.reserve(fw.n * 2 + 16);
    const double* inv = g.geo.L.inv;
    for (uint64_t i = 0; i < fw.n; ++i) {
        const double c[3] = {fw.x[i], fw.y[i], fw.z[i]};
        double f[3];
        for (int a = 0; a < 3; ++a) f[a] = c[0] * inv[a] + c[1] * inv[3 + a] + c[2] * inv[6 + a];
        int nlo[3], nhi[3];
        for (int a = 0; a < 3; ++a) {
            nlo[a] = (int)std::ceil(g.geo.lo[a] - f[a]);
            nhi[a] = (int)std::floor(g.geo.hi[a] - f[a]);
        }
        for (int k0 = nlo[0]; k0 <= nhi[0]; ++k0)
            for (int k1 = nlo[1]; k1 <= nhi[1]; ++k1)
                for (int k2 = nlo[2]; k2 <= nhi[2]; ++k2) {
                    const double fi[3] = {f[0] + k0, f[1] + k1, f[2] + k2};
                    int b[3];
                    for (int a = 0; a < 3; ++a) {
                        int v = (int)std::floor((fi[a] - g.geo.lo[a]) / g.geo.binw[a]);
                        b[a] = std::min(std::max(v, 0), g.geo.nb[a] - 1);
                    }
                    ImageRec r;
                    r.x = c[0] + (k0 * m[0] + k1 * m[3] + k2 * m[6]);
                    r.y = c[1] + (k0 * m[1] + k1 * m[4] + k2 * m[7]);
                    r.z = c[2] + (k0 * m[2] + k1 * m[5] + k2 * m[8]);
                    r.type = fw.species ? fw.species[i] : 0u;
                    r.pad = 0;
                    recs.push_back(r);
                    keys.push_back((uint32_t)(((size_t)b[2] * g.geo.nb[1] + b[1]) * g.geo.nb[0] + b[0]));
                }
    }
    const size_t nbins = (size_t)g.geo.nb[0] * g.geo.nb[1] * g.geo.nb[2];
    require(nbins < (1u << 31) && recs.size() < (1u << 31), ALEA_ERR_INVALID_ARGUMENT,
            "FrameworkEnergyGrid: framework too large for one grid plan");
    std::vector<uint32_t> start(nbins + 1, 0);
    for (uint32_t k : keys) start[k + 1]++;
    for (size_t b = 0; b < nbins; ++b) start[b + 1] += start[b];
    std::vector<ImageRec> sorted(recs.size());
    {
        std::vector<uint32_t> fill(start.begin(), start.end() - 1);
        for (size_t i = 0; i < recs.size(); ++i) sorted[fill[keys[i]]++] = recs[i];
    }
    g.n_images = sorted.size();
    if (precision == ALEA_FP32) {
        std::vector<ImageRecF> sf(sorted.size());
        for (size_t i = 0; i < sorted.size(); ++i) {
            const ImageRec& r = sorted[i];
            ImageRecF& q = sf[i];
            q.xh = (float)r.x;
            q.yh = (float)r.y;
            q.zh = (float)r.z;
            q.xl = (float)(r.x - (double)q.xh);
            q.yl = (float)(r.y - (double)q.yh);
            q.zl = (float)(r.z - (double)q.zh);
            q.type = r.type;
            q.pad = 0.f;
        }
        g.images_f.alloc(std::max<size_t>(sf.size(), 1));
        g.images_f.upload(sf.data(), sf.size());
    } else {
        g.images.alloc(std::max<size_t>(sorted.size(), 1));
        g.images.upload(sorted.data(), sorted.size());
    }
    g.bin_start.alloc(start.size());
    g.bin_start.upload(start.data(), start.size());

    std::vector<PairParams> table((size_t)lj.n_species * lj.n_species);
    mixed_table(lj, table.data());
    // FP32 form: per (guest, framework type) the A/B coefficients and the
    // shift terms, and the double-float parameters of the close pairs; the
    // close-pair reach is the largest mixed sigma of these guests
    {
        const uint32_t nt = lj.n_species;
        std::vector<ParamAB> ab((size_t)ng * nt);
        std::vector<ParamFF> pf((size_t)ng * nt);
        double smax = 0.0;
        for (int gi = 0; gi < ng; ++gi)
            for (uint32_t t = 0; t < nt; ++t) {
                const PairParams& p = table[(size_t)sp[gi] * nt + t];
                smax = std::max(smax, p.sigma);
                const double s2 = p.sigma * p.sigma, s6 = s2 * s2 * s2, e4 = 4.0 * p.eps;
                ab[(size_t)gi * nt + t] = ParamAB{(float)(e4 * s6 * s6), (float)(e4 * s6),
                                                  (float)p.shift, (float)p.dvdrc};
                const float s2h = (float)s2, e4h = (float)e4, shh = (float)p.shift;
                pf[(size_t)gi * nt + t] = ParamFF{s2h, (float)(s2 - s2h), e4h, (float)(e4 - e4h), shh,
                                                  (float)(p.shift - shh), (float)p.dvdrc, 0.f};
            }
        g.geo.smaxf = (float)(smax * (1.0 + 1e-5));
        // reach of the close-pair correction: pairs closer than the largest
        // sigma (FP32 classification, so a relative margin on top)
        const double reach = smax * (1.0 + 1e-4) + 1e-3;
        for (int a = 0; a < 3; ++a) g.geo.hf_near[a] = (float)(reach / g.geo.L.perp[a]);
        g.geo.keep2_near = (float)(reach * reach * (1.0 + 1e-3) + 1e-2);
        if (precision == ALEA_FP32) {
            g.pab.alloc(std::max<size_t>(ab.size(), 1));
            g.pab.upload(ab.data(), ab.size());
            g.pff.alloc(std::max<size_t>(pf.size(), 1));
            g.pff.upload(pf.data(), pf.size());
        }
    }
    g.params.alloc(table.size());
    g.params.upload(table.data(), table.size());
    g.guests.alloc(std::max(ng, 1));
    g.guests.upload(sp.data(), sp.size());
    const size_t nodes = (size_t)g.geo.n[0] * g.geo.n[1] * g.geo.n[2];
    g.tables.alloc(nodes * std::max(ng, 1));
    g.executed.alloc(1);
    g.flags.alloc(1);
    ALEA_CUDA(cudaMemset(g.flags.p, 0, sizeof(unsigned)));
}

// Test support (alea_test_grid_tile_wait_limit): when set (>= 0), the poll limit
// of every tile wait of the next FP64-form build, consumed by that build; the
// waits for the copies still in flight when a CTA gives up keep WAIT_LIMIT.
// (The FP32 form's gathers complete on cp.async.wait_all: no polled wait.)
static std::atomic<int64_t> g_next_tile_wait{-1};

void grid_test_set_tile_wait_limit(int64_t limit) { g_next_tile_wait.store(limit); }

// host: null, or per table one host array the build's rows are copied into as
// the build goes: the bricks run in z-slabs on s, and each finished slab's
// rows (contiguous, z being the slowest index) are copied on a second stream
// while the next slab computes.
static void run_build(GridImpl& g, cudaStream_t s, double* const* host = nullptr) {
    ++g.gen;
    if (g.min_image) {  // rc > L_perp/2: the reference's loop, every node x atom
        const size_t nodes = (size_t)g.geo.n[0] * g.geo.n[1] * g.geo.n[2];
        cudaEvent_t e0, e1;
        ALEA_CUDA(cudaEventCreate(&e0));
        ALEA_CUDA(cudaEventCreate(&e1));
        ALEA_CUDA(cudaEventRecord(e0, s));
        grid_build_mi_kernel<<<(unsigned)((nodes + MI_THREADS - 1) / MI_THREADS), MI_THREADS, 0, s>>>(
            g.mg, g.images.p, g.n_images, g.params.p, g.guests.p, (int)g.species.size(), g.tables.p);
        ALEA_CUDA(cudaGetLastError());
        ALEA_CUDA(cudaEventRecord(e1, s));
        ALEA_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        ALEA_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        g.last_ms = ms;
        g.launches = 1;
        g.executed_pairs = (uint64_t)nodes * g.n_atoms;
        if (host)
            for (size_t k = 0; k < g.species.size(); ++k)
                if (host[k])
                    ALEA_CUDA(cudaMemcpy(host[k], g.tables.p + k * nodes, nodes * sizeof(double),
                                         cudaMemcpyDeviceToHost));
        return;
    }
    const int ng = (int)g.species.size();
    const size_t nodes = (size_t)g.geo.n[0] * g.geo.n[1] * g.geo.n[2];
    const uint64_t nbricks = (uint64_t)g.geo.bricks[0] * g.geo.bricks[1] * g.geo.bricks[2];
    require(nbricks < (1ull << 31), ALEA_ERR_INVALID_ARGUMENT, "grid too large");
    ALEA_CUDA(cudaMemsetAsync(g.executed.p, 0, sizeof(unsigned long long), s));
    const bool f32 = g.precision == ALEA_FP32;
    const int64_t knob = f32 ? -1 : g_next_tile_wait.exchange(-1);
    const unsigned tile_wait = knob >= 0 ? (unsigned)std::min<int64_t>(knob, WAIT_LIMIT) : WAIT_LIMIT;
    // one launch per chunk of up to MAX_NG guests, timed by events on the stream
    const int chunks = (ng + MAX_NG - 1) / MAX_NG;
    cudaEvent_t ev[2];
    for (auto& e : ev) ALEA_CUDA(cudaEventCreate(&e));
    ALEA_CUDA(cudaEventRecord(ev[0], s));
    const int layers = g.geo.bricks[2];
    const int slabs = host ? std::min(8, layers) : 1;
    const uint64_t per_layer = (uint64_t)g.geo.bricks[0] * g.geo.bricks[1];
    const size_t row = (size_t)g.geo.n[0] * g.geo.n[1];
    cudaStream_t cs = nullptr;
    std::vector<cudaEvent_t> done(slabs);
    if (host) {
        ALEA_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        for (auto& e : done) ALEA_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    if (f32 && !g.plans.p) g.plans.alloc((size_t)per_layer * layers * g.plan_stride);
    for (int sl = 0; sl < slabs; ++sl) {
        const int z0 = (int)((int64_t)layers * sl / slabs), z1 = (int)((int64_t)layers * (sl + 1) / slabs);
        GridGeom geo = g.geo;
        geo.brick0 = (int)(per_layer * z0);
        if (f32 && z1 > z0) {  // the slab's row plans, shared by its guest chunks
            grid_plan_kernel<<<(unsigned)(per_layer * (z1 - z0)), THREADS, 0, s>>>(
                geo, g.bin_start.p, g.plans.p, g.plan_stride, g.flags.p);
            ALEA_CUDA(cudaGetLastError());
        }
        for (int c = 0; c < chunks; ++c) {
            const int g0 = c * MAX_NG;
            const int cnt = std::min(MAX_NG, ng - g0);
            dim3 grid((unsigned)(per_layer * (z1 - z0)));
            const size_t pofs = (size_t)g0 * g.geo.n_types;
            const BuildArgs args{g.images.p, g.images_f.p, g.bin_start.p, g.params.p, g.guests.p + g0,
                                 f32 ? g.pab.p + pofs : nullptr, f32 ? g.pff.p + pofs : nullptr,
                                 g.tables.p + (size_t)g0 * nodes, g.executed.p, g.flags.p,
                                 tile_wait, g.plans.p, g.plan_stride};
            launch_build(cnt, g.truncation, f32, grid, s, geo, args);
            ALEA_CUDA(cudaGetLastError());
        }
        if (host) {  // this slab's node rows z in [BZ z0, BZ z1) of every table
            ALEA_CUDA(cudaEventRecord(done[sl], s));
            ALEA_CUDA(cudaStreamWaitEvent(cs, done[sl], 0));
            const size_t a = (size_t)BZ * z0 * row;
            const size_t b = std::min((size_t)BZ * z1, (size_t)g.geo.n[2]) * row;
            for (int k = 0; k < ng; ++k)
                if (host[k] && b > a)
                    ALEA_CUDA(cudaMemcpyAsync(host[k] + a, g.tables.p + (size_t)k * nodes + a,
                                              (b - a) * sizeof(double), cudaMemcpyDeviceToHost, cs));
        }
    }
    ALEA_CUDA(cudaEventRecord(ev[1], s));
    ALEA_CUDA(cudaEventSynchronize(ev[1]));
    if (host) {
        ALEA_CUDA(cudaStreamSynchronize(cs));
        for (auto& e : done) cudaEventDestroy(e);
        cudaStreamDestroy(cs);
    }
    float ms = 0.f;
    ALEA_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
    for (auto& e : ev) cudaEventDestroy(e);
    g.last_ms = ms;
    g.launches = slabs * chunks + (f32 ? slabs : 0);
    unsigned long long ex = 0;
    ALEA_CUDA(cudaMemcpy(&ex, g.executed.p, sizeof(ex), cudaMemcpyDeviceToHost));
    g.executed_pairs = ex;
    check_device_flags(g.flags.p, s, "grid build kernel");
}

GridImpl* grid_build(const alea_lennard_jones& lj, const alea_particles& fw,
                     const alea_lattice& lat, const uint32_t* guest, uint32_t n_guest,
                     double spacing, int precision) {
    auto* g = new GridImpl();
    try {
        build_plan(*g, lj, fw, lat, guest, n_guest, spacing, precision, bin_width(precision));
        run_build(*g, 0);
    } catch (...) {
        delete g;
        throw;
    }
    return g;
}

void grid_rebuild(GridImpl* g, cudaStream_t s) { run_build(*g, s); }

GridImpl* grid_build_to_host(const alea_lennard_jones& lj, const alea_particles& fw,
                             const alea_lattice& lat, const uint32_t* guest, uint32_t n_guest,
                             double spacing, int precision, double* const* host) {
    auto* g = new GridImpl();
    try {
        build_plan(*g, lj, fw, lat, guest, n_guest, spacing, precision, bin_width(precision));
        // host arrays in the order of `guest`, tables in the grid's (sorted) order
        std::vector<double*> per_table(g->species.size(), nullptr);
        for (uint32_t k = 0; k < n_guest; ++k) {
            const size_t t = (size_t)(std::lower_bound(g->species.begin(), g->species.end(), guest[k]) -
                                      g->species.begin());
            if (!per_table[t]) per_table[t] = host[k];
        }
        run_build(*g, 0, per_table.data());
        // a species listed twice: its other arrays get the copy made above
        for (uint32_t k = 0; k < n_guest; ++k) {
            const size_t t = (size_t)(std::lower_bound(g->species.begin(), g->species.end(), guest[k]) -
                                      g->species.begin());
            const size_t nodes = (size_t)g->geo.n[0] * g->geo.n[1] * g->geo.n[2];
            if (host[k] != per_table[t]) std::memcpy(host[k], per_table[t], nodes * sizeof(double));
        }
    } catch (...) {
        delete g;
        throw;
    }
    return g;
}
void grid_destroy(GridImpl* g) { delete g; }

static int table_index(const GridImpl* g, uint32_t species) {
    const auto it = std::lower_bound(g->species.begin(), g->species.end(), species);
    if (it == g->species.end() || *it != species)
        throw Error(ALEA_ERR_OUT_OF_RANGE,
                    "FrameworkEnergyGrid::interpolate: no table for guest species " +
                        std::to_string(species));
    return (int)(it - g->species.begin());
}

const double* grid_table(const GridImpl* g, uint32_t species) {
    const size_t nodes = (size_t)g->geo.n[0] * g->geo.n[1] * g->geo.n[2];
    return g->tables.p + (size_t)table_index(g, species) * nodes;
}

GridView grid_view(const GridImpl* g, uint32_t species) {
    GridView v{};
    v.L = g->geo.L;
    for (int a = 0; a < 3; ++a) v.n[a] = g->geo.n[a];
    v.table = grid_table(g, species);  // out_of_range as FrameworkEnergyGrid::interpolate
    v.fast = g->precision == ALEA_FP32;
    return v;
}

// The corner blocks of an FP32-form grid's species table, made (on stream s)
// when missing or older than the table; null when they cannot be allocated.
// Every caller's stream s waits on the event recorded after the corner kernel,
// so an interpolation on another stream never reads blocks still being made.
static const double2* grid_corners(GridImpl* g, uint32_t species, cudaStream_t s) {
    std::lock_guard<std::mutex> lock(g->corners_mu);
    if (g->corners_off) return nullptr;
    const int k = table_index(g, species);
    const size_t nodes = (size_t)g->geo.n[0] * g->geo.n[1] * g->geo.n[2];
    if (g->corners.size() != g->species.size()) {
        g->corners.resize(g->species.size());
        g->corners_gen.assign(g->species.size(), 0);
        g->corners_ev.resize(g->species.size());
    }
    if (!g->corners[k].p || g->corners_gen[k] != g->gen) {
        if (!g->corners[k].p) {
            try {
                g->corners[k].alloc(4 * nodes);
            } catch (const Error&) {
                (void)cudaGetLastError();  // out of memory: not sticky
                g->corners[k].release();
                g->corners_off = true;
                return nullptr;
            }
        }
        if (!g->corners_ev[k]) {
            cudaEvent_t ev = nullptr;
            ALEA_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            g->corners_ev[k].reset(ev);
        }
        int dev = 0, sms = 0;
        ALEA_CUDA(cudaGetDevice(&dev));
        ALEA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        grid_corners_kernel<<<(unsigned)sms * 8, 256, 0, s>>>(g->geo.n[0], g->geo.n[1], g->geo.n[2],
                                                              grid_table(g, species), g->corners[k].p);
        ALEA_CUDA(cudaGetLastError());
        ALEA_CUDA(cudaEventRecord(g->corners_ev[k].get(), s));
        g->corners_gen[k] = g->gen;
    } else {
        ALEA_CUDA(cudaStreamWaitEvent(s, g->corners_ev[k].get(), 0));
    }
    return g->corners[k].p;
}

void grid_interpolate_device(const GridImpl* g, uint32_t species, const double* xyz, uint64_t n,
                             double* out, cudaStream_t s) {
    const double* tab = grid_table(g, species);
    if (n == 0) return;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    // the FP64 form reproduces the reference's arithmetic bit for bit
    if (g->precision == ALEA_FP32) {
        InvFF inv;
        for (int k = 0; k < 9; ++k) {
            const ff v = ff_from(g->geo.L.inv[k]);
            inv.h[k] = v.hi;
            inv.l[k] = v.lo;
        }
        int dev = 0, sms = 0;  // resident work for a persistent loop: 24 blocks per SM
        ALEA_CUDA(cudaGetDevice(&dev));
        ALEA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const unsigned fb = (unsigned)std::min<uint64_t>(blocks, (uint64_t)sms * 24);
        const double2* cb = grid_corners(const_cast<GridImpl*>(g), species, s);
        if (cb)
            grid_interpolate_corners_kernel<<<fb, 256, 0, s>>>(g->geo.L, inv, g->geo.n[0],
                                                              g->geo.n[1], g->geo.n[2], cb, tab,
                                                              xyz, n, out);
        else
            grid_interpolate_fast_kernel<<<fb, 256, 0, s>>>(g->geo.L, inv, g->geo.n[0], g->geo.n[1],
                                                           g->geo.n[2], tab, xyz, n, out);
    } else
        grid_interpolate_kernel<<<blocks, 256, 0, s>>>(g->geo.L, g->geo.n[0], g->geo.n[1],
                                                      g->geo.n[2], tab, xyz, n, out);
    ALEA_CUDA(cudaGetLastError());
}

void grid_interpolate_host(const GridImpl* g, uint32_t species, const double* xyz, uint64_t n,
                           double* out) {
    (void)grid_table(g, species);
    if (n == 0) return;
    DevBuf<double> dx(3 * n), dout(n);
    dx.upload(xyz, 3 * n);
    grid_interpolate_device(g, species, dx.p, n, dout.p, 0);
    dout.download(out, n);
    ALEA_CUDA(cudaStreamSynchronize(0));
}

void grid_download(const GridImpl* g, uint32_t species, double* out, uint64_t n) {
    const size_t nodes = (size_t)g->geo.n[0] * g->geo.n[1] * g->geo.n[2];
    require(n >= nodes, ALEA_ERR_INVALID_ARGUMENT, "alea_grid_download: output too small");
    ALEA_CUDA(cudaMemcpy(out, grid_table(g, species), nodes * sizeof(double),
                         cudaMemcpyDeviceToHost));
}

void grid_counts(const GridImpl* g, int32_t* out) {
    for (int a = 0; a < 3; ++a) out[a] = g->geo.n[a];
}
double grid_spacing(const GridImpl* g) { return g->spacing; }
const std::vector<uint32_t>& grid_species(const GridImpl* g) { return g->species; }

void grid_stats(const GridImpl* g, alea_grid_stats* out) {
    const uint64_t nodes = (uint64_t)g->geo.n[0] * g->geo.n[1] * g->geo.n[2];
    out->nodes = nodes;
    out->algorithmic_pairs = nodes * g->n_atoms * (uint64_t)g->species.size();
    out->executed_pairs = g->executed_pairs * (uint64_t)g->species.size();
    out->images = g->n_images;
    out->bricks = (uint64_t)g->geo.bricks[0] * g->geo.bricks[1] * g->geo.bricks[2];
    out->last_kernel_ms = g->last_ms;
    out->launches = (uint32_t)g->launches;
}

// ---------------------------------------------------------------- batch of grids
struct GridBatchImpl {
    std::vector<GridImpl*> grids;
    int ng = 0, truncation = ALEA_SHIFTED;
    uint64_t total = 0;
    DevBuf<BatchItem> items;
    DevBuf<unsigned long long> counters, executed;
    DevBuf<unsigned> flags;
    cudaStream_t own = nullptr;  // capture stream (graphs cannot be captured on stream 0)
    int sms = 0;
    int variant = -1;            // chosen by the autotuner on the first build
    float tune_ms[BATCH_VARIANTS] = {};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint32_t graph_launches = 0;
    float last_ms = 0.f;
    uint64_t executed_pairs = 0;
    ~GridBatchImpl() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (own) cudaStreamDestroy(own);
        for (auto* g : grids) delete g;
    }
};

GridBatchImpl* grid_batch_create(uint32_t n, const alea_lennard_jones* lj, const alea_particles* fw,
                                 const alea_lattice* lat, const uint32_t* guests, uint32_t n_guest,
                                 double spacing) {
    require(n >= 1, ALEA_ERR_INVALID_ARGUMENT, "alea_grid_batch_create: at least one grid");
    require(n_guest >= 1 && n_guest <= (uint32_t)MAX_NG, ALEA_ERR_INVALID_ARGUMENT,
            "alea_grid_batch_create: 1..4 guest species per grid");
    auto* b = new GridBatchImpl();
    try {
        std::vector<BatchItem> items(n);
        for (uint32_t i = 0; i < n; ++i) {
            auto* g = new GridImpl();
            b->grids.push_back(g);
            // the batched kernel sums image lists: every cutoff must fit (rc <= L_perp/2)
            validate_cutoff(make_lattice(lat[i].m), lj[i].cutoff, "alea_grid_batch_create");
            build_plan(*g, lj[i], fw[i], lat[i], guests + (size_t)i * n_guest, n_guest, spacing,
                       ALEA_FP32, bin_width(ALEA_FP32));
            if (i == 0) {
                b->ng = (int)g->species.size();
                b->truncation = g->truncation;
            }
            require((int)g->species.size() == b->ng && g->truncation == b->truncation,
                    ALEA_ERR_INVALID_ARGUMENT,
                    "alea_grid_batch_create: every grid needs the same number of distinct guests "
                    "and the same truncation");
            const uint64_t nodes = (uint64_t)g->geo.n[0] * g->geo.n[1] * g->geo.n[2];
            (void)nodes;
            items[i].geo = g->geo;
            items[i].args = F32GridArgs{g->images_f.p, g->bin_start.p, g->pab.p, g->pff.p,
                                        g->tables.p, nullptr, 0u};
            items[i].brick0 = b->total;
            b->total += (uint64_t)g->geo.bricks[0] * g->geo.bricks[1] * g->geo.bricks[2];
        }
        b->items.alloc(n);
        b->items.upload(items.data(), n);
        b->counters.alloc(2);
        b->executed.alloc(1);
        b->flags.alloc(1);
        ALEA_CUDA(cudaMemset(b->flags.p, 0, sizeof(unsigned)));
        ALEA_CUDA(cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking));
        int dev = 0;
        ALEA_CUDA(cudaGetDevice(&dev));
        ALEA_CUDA(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev));
        ALEA_CUDA(cudaDeviceSynchronize());
    } catch (...) {
        delete b;
        throw;
    }
    return b;
}

static void batch_sequence(GridBatchImpl* b, int variant, cudaStream_t s) {
    ALEA_CUDA(cudaMemsetAsync(b->executed.p, 0, sizeof(unsigned long long), s));
    batch_launch(b->ng, b->truncation, variant, b->sms, s, b->items.p, (int)b->grids.size(), b->total,
                 b->counters.p, b->executed.p, b->flags.p);
}

// One build of every grid. The first call times each launch variant on the
// whole batch (the autotuner; every variant writes the same tables), keeps the
// fastest and captures its launch sequence into a CUDA graph; every call then
// replays the graph on the caller's stream.
void grid_batch_build(GridBatchImpl* b, cudaStream_t s) {
    cudaStream_t run = s ? s : b->own;
    cudaEvent_t e0, e1;
    ALEA_CUDA(cudaEventCreate(&e0));
    ALEA_CUDA(cudaEventCreate(&e1));
    if (b->variant < 0) {
        for (int v = 0; v < BATCH_VARIANTS; ++v) {
            ALEA_CUDA(cudaEventRecord(e0, run));
            batch_sequence(b, v, run);
            ALEA_CUDA(cudaEventRecord(e1, run));
            ALEA_CUDA(cudaEventSynchronize(e1));
            ALEA_CUDA(cudaEventElapsedTime(&b->tune_ms[v], e0, e1));
            check_device_flags(b->flags.p, run, "batched grid build");
        }
        b->variant = (int)(std::min_element(b->tune_ms, b->tune_ms + BATCH_VARIANTS) - b->tune_ms);
        ALEA_CUDA(cudaStreamBeginCapture(b->own, cudaStreamCaptureModeThreadLocal));
        batch_sequence(b, b->variant, b->own);
        ALEA_CUDA(cudaStreamEndCapture(b->own, &b->graph));
        ALEA_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
    }
    ALEA_CUDA(cudaEventRecord(e0, run));
    ALEA_CUDA(cudaGraphLaunch(b->exec, run));
    ALEA_CUDA(cudaEventRecord(e1, run));
    ALEA_CUDA(cudaEventSynchronize(e1));
    ALEA_CUDA(cudaEventElapsedTime(&b->last_ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ++b->graph_launches;
    unsigned long long ex = 0;
    ALEA_CUDA(cudaMemcpy(&ex, b->executed.p, sizeof(ex), cudaMemcpyDeviceToHost));
    b->executed_pairs = ex;
    check_device_flags(b->flags.p, run, "batched grid build");
}

void grid_batch_stats(const GridBatchImpl* b, alea_grid_batch_stats* out) {
    out->grids = (uint32_t)b->grids.size();
    out->nodes = 0;
    out->algorithmic_pairs = 0;
    for (const auto* g : b->grids) {
        const uint64_t nodes = (uint64_t)g->geo.n[0] * g->geo.n[1] * g->geo.n[2];
        out->nodes += nodes;
        out->algorithmic_pairs += nodes * g->n_atoms * (uint64_t)g->species.size();
    }
    out->executed_pairs = b->executed_pairs * (uint64_t)b->ng;
    out->bricks = b->total;
    out->last_ms = b->last_ms;
    out->variant = b->variant;
    for (int v = 0; v < BATCH_VARIANTS && v < 2; ++v) out->tune_ms[v] = b->tune_ms[v];
    out->graph_launches = b->graph_launches;
}

const GridImpl* grid_batch_item(const GridBatchImpl* b, uint32_t i) {
    require(i < b->grids.size(), ALEA_ERR_OUT_OF_RANGE, "grid batch: grid index");
    return b->grids[i];
}

void grid_batch_destroy(GridBatchImpl* b) { delete b; }

GridImpl* grid_from_tables(const alea_lattice& lat, double spacing, const int32_t counts[3],
                           const std::vector<uint32_t>& species,
                           const std::vector<std::vector<double>>& tables) {
    require_device();
    auto* g = new GridImpl();
    g->geo.L = make_lattice(lat.m);
    for (int a = 0; a < 3; ++a) g->geo.n[a] = counts[a];
    g->spacing = spacing;
    g->species = species;
    const size_t nodes = (size_t)counts[0] * counts[1] * counts[2];
    g->tables.alloc(nodes * std::max<size_t>(species.size(), 1));
    for (size_t i = 0; i < species.size(); ++i) {
        require(tables[i].size() == nodes, ALEA_ERR_RUNTIME, "grid cache: table size mismatch");
        ALEA_CUDA(cudaMemcpy(g->tables.p + i * nodes, tables[i].data(), nodes * sizeof(double),
                             cudaMemcpyHostToDevice));
    }
    return g;
}

}  // namespace alea
