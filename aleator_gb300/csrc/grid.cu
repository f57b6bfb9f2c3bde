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
// range, and streams the ranges through shared memory in 256-record tiles
// with cp.async.bulk (TMA) copies completed on an mbarrier, double-buffered.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "common.cuh"
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

struct GridGeom {
    Lattice L;
    int n[3];
    double lo[3], hi[3];   // fractional extent of the binned image range
    int nb[3];             // bins per axis
    double binw[3];        // fractional bin width
    double G[9];           // metric tensor a_i . a_j
    float Gf[9];           // the same in FP32 (bin culling)
    float lof[3], binwf[3];  // lo and binw in FP32 (bin culling)
    float near2;           // (largest sigma + brick half-diagonal)^2: close-pass reach
    double rc, rc2;
    int bricks[3];
    int n_types;           // framework LJ species in the table
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
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, unsigned* flags) {
    for (unsigned it = 0; it < WAIT_LIMIT; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if (it > 64) __nanosleep(64);
    }
    flag_error(flags, DEV_ERR_WAIT);
    return false;
}

// Lower bound on min |D . M|^2 over the fractional box D = [dlo, dhi]:
// a few coordinate-descent sweeps of the convex quadratic D^T G D, then the
// first-order bound f(x) + min_{y in box} grad(x).(y - x), which never exceeds
// the true minimum. Exact for orthorhombic cells. FP32 (FP64 issues at a small
// fraction of the FP32 rate on this part); the caller compares against rc^2
// with a relative margin far above FP32 rounding, so culling stays conservative.
__device__ __forceinline__ float box_min_dist2_lb(const float* G, const float* dlo,
                                                  const float* dhi) {
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
            x[i] = fminf(fmaxf(-s / G[4 * i], dlo[i]), dhi[i]);
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

// ---------------------------------------------------------------- double-float
// Two-float ("double-float") arithmetic for the rare close pairs of the FP32
// form: the repulsive terms there reach 1e4 K, where FP32's ~1e-6 relative
// rounding would leave ~1e-2 K of error in a node energy. Error-free
// transformations (Knuth two-sum, FMA two-product); the _rn intrinsics keep
// the compiler from contracting or reassociating them.
struct ff {
    float hi, lo;
};
__device__ __forceinline__ ff ff_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
__device__ __forceinline__ ff ff_fast(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = ff_two_sum(a.hi, b.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return ff_fast(s.hi, s.lo);
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
    return ff_fast(p, e);
}
__device__ __forceinline__ ff ff_rcp(ff a) {  // one Newton step from the FP32 reciprocal
    const float y = __frcp_rn(a.hi);
    const ff ay = ff_mul(a, ff{y, 0.f});
    const ff r = ff_add(ff{1.f, 0.f}, ff{-ay.hi, -ay.lo});
    const ff c = ff_mul(ff{y, 0.f}, r);
    return ff_add(ff{y, 0.f}, c);
}

struct alignas(16) ParamFF {
    float sig2_hi, sig2_lo, eps4_hi, eps4_lo, shift_hi, shift_lo, dvdrc, pad;
};

struct alignas(16) ParamF {
    float sig2, eps4, shift, dvdrc;
};

template <typename Real>
struct KernelSmem;

// ---------------------------------------------------------------- build kernel
// Real = float: pair terms in FP32 on brick-local coordinates, per-tile FP32
// partial sums folded into FP64. Real = double: the FP64 parity form on the
// reference's global Cartesian coordinates.
template <typename Real, int NG, int TRUNC>
__global__ void __launch_bounds__(THREADS)
grid_build_kernel(GridGeom geo, const ImageRec* __restrict__ images,
                  const uint32_t* __restrict__ bin_start, const PairParams* __restrict__ params,
                  const uint32_t* __restrict__ guests, double* __restrict__ tables,
                  unsigned long long* __restrict__ executed, unsigned* flags) {
    // dynamic shared memory (above the 48 KB static limit), carved by hand;
    // the layout is mirrored by grid_smem_bytes<Real>() on the host
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char* sp = smem;
    auto take = [&](size_t bytes) {
        unsigned char* q = sp;
        sp += (bytes + 127) & ~(size_t)127;
        return q;
    };
    ImageRec* raw = reinterpret_cast<ImageRec*>(take(2 * TILE * sizeof(ImageRec)));
    float4* conv = reinterpret_cast<float4*>(take(TILE * sizeof(float4)));
    float4* convlo = reinterpret_cast<float4*>(take((sizeof(Real) == 4 ? TILE : 1) * sizeof(float4)));
    float* nlo = reinterpret_cast<float*>(take((sizeof(Real) == 4 ? NPT * 3 * THREADS : 1) * sizeof(float)));
    uint64_t* bars = reinterpret_cast<uint64_t*>(take(2 * sizeof(uint64_t)));
    uint32_t* row_begin = reinterpret_cast<uint32_t*>(take(MAX_ROWS * sizeof(uint32_t)));
    uint32_t* row_off = reinterpret_cast<uint32_t*>(take((MAX_ROWS + 1) * sizeof(uint32_t)));
    uint32_t* warp_tot = reinterpret_cast<uint32_t*>(take((THREADS / 32) * sizeof(uint32_t)));
    ParamF* pf = reinterpret_cast<ParamF*>(take(64 * MAX_NG * sizeof(ParamF)));
    float* rcl2 = reinterpret_cast<float*>(take(64 * sizeof(float)));
    uint16_t* close_idx = reinterpret_cast<uint16_t*>(take(TILE * sizeof(uint16_t)));
    PairParams* pd = reinterpret_cast<PairParams*>(take(64 * MAX_NG * sizeof(PairParams)));
    ParamFF* pff = reinterpret_cast<ParamFF*>(pd);  // the FP32 form uses this slot instead

    const int tid = threadIdx.x;
    const int nx = geo.n[0], ny = geo.n[1], nz = geo.n[2];
    const int brick = blockIdx.x;
    const int bxn = geo.bricks[0], byn = geo.bricks[1];
    const int bx = brick % bxn, by = (brick / bxn) % byn, bz = brick / (bxn * byn);
    const int x0 = bx * BX, y0 = by * BY, z0 = bz * BZ;

    // pair parameters for (framework type, guest g)
    for (int i = tid; i < geo.n_types * NG; i += THREADS) {
        const int t = i / NG, g = i % NG;
        const PairParams p = params[(size_t)guests[g] * geo.n_types + t];
        const double s2 = p.sigma * p.sigma;
        pf[i] = ParamF{(float)s2, (float)(4.0 * p.eps), (float)p.shift, (float)p.dvdrc};
        if (sizeof(Real) == 8) {
            pd[i] = p;
        } else {
            const double e4 = 4.0 * p.eps;
            const float s2h = (float)s2, e4h = (float)e4, shh = (float)p.shift;
            pff[i] = ParamFF{s2h, (float)(s2 - s2h), e4h, (float)(e4 - e4h), shh,
                             (float)(p.shift - shh), (float)p.dvdrc, 0.f};
        }
    }
    __syncthreads();
    // close-pair radius per framework type: r < sigma for some guest (s^2 > 1)
    if (sizeof(Real) == 4)
        for (int t = tid; t < geo.n_types; t += THREADS) {
            float m = 0.f;
            for (int g = 0; g < NG; ++g) m = fmaxf(m, pf[t * NG + g].sig2);
            rcl2[t] = m;
        }
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_barrier_init();
    }

    // fractional extent of the brick's nodes
    const int xe = min(x0 + BX, nx) - 1, ye = min(y0 + BY, ny) - 1, ze = min(z0 + BZ, nz) - 1;
    double flo[3] = {(double)x0 / nx, (double)y0 / ny, (double)z0 / nz};
    double fhi[3] = {(double)xe / nx, (double)ye / ny, (double)ze / nz};
    int blo[3], bhi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double h = geo.rc / geo.L.perp[a];
        blo[a] = max(0, (int)floor((flo[a] - h - geo.lo[a]) / geo.binw[a]) - 1);
        bhi[a] = min(geo.nb[a] - 1, (int)floor((fhi[a] + h - geo.lo[a]) / geo.binw[a]) + 1);
    }
    const int rows_y = bhi[1] - blo[1] + 1, rows_z = bhi[2] - blo[2] + 1;
    const int total_rows = rows_y * rows_z;
    __syncthreads();

    // one thread per bin row: find the first and last bins within reach.
    // Row slots follow the row enumeration, so the candidate order (and the
    // floating-point summation order) is the same on every run.
    if (total_rows > MAX_ROWS) {
        if (tid == 0) flag_error(flags, DEV_ERR_CAPACITY);
        return;
    }
    const float keep2 = (float)(geo.rc2 * (1.0 + 1e-3) + 1e-2);
    const float flof[3] = {(float)flo[0], (float)flo[1], (float)flo[2]};
    const float fhif[3] = {(float)fhi[0], (float)fhi[1], (float)fhi[2]};
    for (int r = tid; r < total_rows; r += THREADS) {
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
            if (box_min_dist2_lb(geo.Gf, dlo, dhi) <= keep2) {
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
    const int nr = total_rows;
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
    const uint32_t n_cand = row_off[nr];

    // this thread's nodes
    const int tx = tid % BX, ty = (tid / BX) % BY, tz = tid / (BX * BY);
    const int ixn = x0 + tx, iyn = y0 + ty;
    double acc[NG][NPT];
#pragma unroll
    for (int g = 0; g < NG; ++g)
#pragma unroll
        for (int k = 0; k < NPT; ++k) acc[g][k] = 0.0;

    // Brick centre (origin of the FP32 form's local coordinates: the atoms
    // that matter most, the close ones, then have the smallest coordinates and
    // the smallest rounding) and node coordinates.
    const double* M = geo.L.m;
    double ox = 0, oy = 0, oz = 0;
    Real nxr[NPT], nyr[NPT], nzr[NPT];
    {
        const double cx = x0 + 0.5 * (BX - 1), cy = y0 + 0.5 * (BY - 1), cz = z0 + 0.5 * (BZ - 1);
        const double f0o = cx / nx, f1o = cy / ny, f2o = cz / nz;
        ox = f0o * M[0] + f1o * M[3] + f2o * M[6];
        oy = f0o * M[1] + f1o * M[4] + f2o * M[7];
        oz = f0o * M[2] + f1o * M[5] + f2o * M[8];
#pragma unroll
        for (int k = 0; k < NPT; ++k) {
            const int izn = z0 + tz + 2 * k;
            if (sizeof(Real) == 4) {
                const double d0 = (ixn - cx) / nx, d1 = (iyn - cy) / ny, d2 = (izn - cz) / nz;
                const double lx = d0 * M[0] + d1 * M[3] + d2 * M[6];
                const double ly = d0 * M[1] + d1 * M[4] + d2 * M[7];
                const double lz = d0 * M[2] + d1 * M[5] + d2 * M[8];
                nxr[k] = (Real)lx;
                nyr[k] = (Real)ly;
                nzr[k] = (Real)lz;
                nlo[(k * 3 + 0) * THREADS + tid] = (float)(lx - (double)nxr[k]);
                nlo[(k * 3 + 1) * THREADS + tid] = (float)(ly - (double)nyr[k]);
                nlo[(k * 3 + 2) * THREADS + tid] = (float)(lz - (double)nzr[k]);
                continue;
            }
            // framework_energy_grid.cc:227-231 node position
            const double f0 = (double)ixn / nx, f1 = (double)iyn / ny, f2 = (double)izn / nz;
            double c[3];
#pragma unroll
            for (int cc = 0; cc < 3; ++cc)
                c[cc] = add_rn(add_rn(mul_rn(f0, M[cc]), mul_rn(f1, M[3 + cc])), mul_rn(f2, M[6 + cc]));
            {
                nxr[k] = (Real)c[0];
                nyr[k] = (Real)c[1];
                nzr[k] = (Real)c[2];
            }
        }
    }

    // stage tile `t` of the concatenated candidate list into raw[buf]
    auto issue = [&](uint32_t t, int buf) {
        const uint32_t a = t * TILE;
        const uint32_t b = min(a + (uint32_t)TILE, n_cand);
        mbar_expect_tx(&bars[buf], (b - a) * (uint32_t)sizeof(ImageRec));
        // rows overlapping [a, b)
        int r = 0;
        {
            int lo = 0, hi = nr - 1;  // last row with row_off[r] <= a
            while (lo < hi) {
                const int mid = (lo + hi + 1) / 2;
                if (row_off[mid] <= a) lo = mid; else hi = mid - 1;
            }
            r = lo;
        }
        for (; r < nr && row_off[r] < b; ++r) {
            const uint32_t s = max(row_off[r], a), e = min(row_off[r + 1], b);
            if (e > s)
                bulk_g2s(&raw[buf * TILE + (s - a)], images + row_begin[r] + (s - row_off[r]),
                         (e - s) * (uint32_t)sizeof(ImageRec), &bars[buf]);
        }
    };

    const uint32_t n_tiles = (n_cand + TILE - 1) / TILE;
    if (tid == 0) {
        if (n_tiles > 0) issue(0, 0);
        if (n_tiles > 1) issue(1, 1);
    }
    const float rc2f = (float)geo.rc2;
    const float rcf = (float)geo.rc;
    bool ok = true;
    uint32_t failed_tile = 0;

    for (uint32_t t = 0; t < n_tiles; ++t) {
        const int buf = t & 1;
        const uint32_t cnt = min((uint32_t)TILE, n_cand - t * TILE);
        // block-wide vote so that every thread takes the same path on a timeout
        const bool got = mbar_wait_bounded(&bars[buf], (t >> 1) & 1, flags);
        if (!__syncthreads_and(got)) {
            ok = false;
            failed_tile = t;
            break;
        }
        if (sizeof(Real) == 4) {
            // convert to brick-centred FP32 (hi + lo parts) and list, in atom
            // order, the atoms that can be closer than sigma to a node of this
            // brick (within reach of the brick centre)
            static_assert(TILE == THREADS, "one atom per thread in the conversion pass");
            bool near = false;
            if ((uint32_t)tid < cnt) {
                const ImageRec r = raw[buf * TILE + tid];
                const double lx = r.x - ox, ly = r.y - oy, lz = r.z - oz;
                const float hx = (float)lx, hy = (float)ly, hz = (float)lz;
                conv[tid] = make_float4(hx, hy, hz, __int_as_float((int)r.type));
                convlo[tid] = make_float4((float)(lx - hx), (float)(ly - hy), (float)(lz - hz), 0.f);
                near = fmaf(hx, hx, fmaf(hy, hy, hz * hz)) < geo.near2;
            }
            const unsigned ballot = __ballot_sync(0xffffffffu, near);
            if ((tid & 31) == 0) warp_tot[tid >> 5] = __popc(ballot);
            __syncthreads();
            if (near) {
                uint32_t off = __popc(ballot & ((1u << (tid & 31)) - 1u));
                for (int w = 0; w < (tid >> 5); ++w) off += warp_tot[w];
                close_idx[off] = (uint16_t)tid;
            }
            uint32_t n_close = 0;
            for (int w = 0; w < THREADS / 32; ++w) n_close += warp_tot[w];
            __syncthreads();
            // raw[buf] is free again: prefetch tile t + 2 while computing
            if (tid == 0 && t + 2 < n_tiles) {
                fence_proxy_async();
                issue(t + 2, buf);
            }
            float part[NG][NPT];
#pragma unroll
            for (int g = 0; g < NG; ++g)
#pragma unroll
                for (int k = 0; k < NPT; ++k) part[g][k] = 0.f;
#pragma unroll 2
            for (uint32_t j = 0; j < cnt; ++j) {
                const float4 a = conv[j];
                const int type = __float_as_int(a.w);
                const float close2 = rcl2[type];
                ParamF p[NG];
#pragma unroll
                for (int g = 0; g < NG; ++g) p[g] = pf[type * NG + g];
#pragma unroll
                for (int k = 0; k < NPT; ++k) {
                    const float dx = a.x - (float)nxr[k];
                    const float dy = a.y - (float)nyr[k];
                    const float dz = a.z - (float)nzr[k];
                    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    const float inv = __frcp_rn(fmaxf(r2, 1e-4f));
                    // pairs closer than sigma are left to the close pass below
                    const bool in = (r2 <= rc2f) && (r2 >= close2);
#pragma unroll
                    for (int g = 0; g < NG; ++g) {
                        const float s2 = p[g].sig2 * inv;
                        const float s6 = s2 * s2 * s2;
                        float e = fmaf(p[g].eps4, fmaf(s6, s6, -s6), -p[g].shift);
                        if (TRUNC == ALEA_LINEAR_FORCE_SHIFTED) {
                            const float r = r2 * rsqrtf(fmaxf(r2, 1e-4f));
                            e = fmaf(-(r - rcf), p[g].dvdrc, e);
                        }
                        part[g][k] += in ? e : 0.f;
                    }
                }
            }
            // close pass: the few listed atoms, pairs closer than sigma in
            // double-float, straight into the FP64 accumulators
            for (uint32_t c = 0; c < n_close; ++c) {
                const uint32_t j = close_idx[c];
                const float4 a = conv[j];
                const int type = __float_as_int(a.w);
                const float close2 = rcl2[type];
#pragma unroll
                for (int k = 0; k < NPT; ++k) {
                    const float dx = a.x - (float)nxr[k];
                    const float dy = a.y - (float)nyr[k];
                    const float dz = a.z - (float)nzr[k];
                    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    if (r2 < close2) {
                        const float4 al = convlo[j];
                        const ff ddx = ff_add(ff{a.x, al.x}, ff{-(float)nxr[k], -nlo[(k * 3 + 0) * THREADS + tid]});
                        const ff ddy = ff_add(ff{a.y, al.y}, ff{-(float)nyr[k], -nlo[(k * 3 + 1) * THREADS + tid]});
                        const ff ddz = ff_add(ff{a.z, al.z}, ff{-(float)nzr[k], -nlo[(k * 3 + 2) * THREADS + tid]});
                        ff rr = ff_add(ff_add(ff_mul(ddx, ddx), ff_mul(ddy, ddy)), ff_mul(ddz, ddz));
                        if (rr.hi < 1e-4f) rr = ff{1e-4f, 0.f};
                        const ff iv = ff_rcp(rr);
#pragma unroll
                        for (int g = 0; g < NG; ++g) {
                            const ParamFF q = pff[type * NG + g];
                            const ff s2 = ff_mul(ff{q.sig2_hi, q.sig2_lo}, iv);
                            const ff s6 = ff_mul(ff_mul(s2, s2), s2);
                            const ff t = ff_mul(s6, ff_add(s6, ff{-1.f, 0.f}));
                            ff e = ff_add(ff_mul(ff{q.eps4_hi, q.eps4_lo}, t), ff{-q.shift_hi, -q.shift_lo});
                            if (TRUNC == ALEA_LINEAR_FORCE_SHIFTED) {
                                const float r = sqrtf(rr.hi);
                                e = ff_add(e, ff{-(r - rcf) * q.dvdrc, 0.f});
                            }
                            acc[g][k] += (double)e.hi + (double)e.lo;
                        }
                    }
                }
            }
#pragma unroll
            for (int g = 0; g < NG; ++g)
#pragma unroll
                for (int k = 0; k < NPT; ++k) acc[g][k] += (double)part[g][k];
            __syncthreads();  // conv reused by the next tile
        } else {
            for (uint32_t j = 0; j < cnt; ++j) {
                const ImageRec a = raw[buf * TILE + j];
                const PairParams* pp = &pd[a.type * NG];
#pragma unroll
                for (int k = 0; k < NPT; ++k) {
                    const double dx = a.x - (double)nxr[k];
                    const double dy = a.y - (double)nyr[k];
                    const double dz = a.z - (double)nzr[k];
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
                issue(t + 2, buf);
            }
        }
    }
    if (!ok) {
        // Drain this block's copies still in flight (tiles failed_tile and
        // failed_tile + 1 are the only ones issued and not yet consumed),
        // each wait again bounded, before the block exits.
        if (tid == 0)
            for (uint32_t t = failed_tile; t < failed_tile + 2 && t < n_tiles; ++t)
                for (unsigned it = 0; it < WAIT_LIMIT && !mbar_try_wait(&bars[t & 1], (t >> 1) & 1);
                     ++it) {
                    __nanosleep(64);
                }
        __syncthreads();
        return;
    }

    // store min(E, cap) (framework_energy_grid.cc:22, 243)
    const size_t plane = (size_t)nx * ny;
    const size_t per_table = plane * nz;
#pragma unroll
    for (int k = 0; k < NPT; ++k) {
        const int izn = z0 + tz + 2 * k;
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
        const unsigned long long active =
            (unsigned long long)(xe - x0 + 1) * (ye - y0 + 1) * (ze - z0 + 1);
        atomicAdd(executed, active * n_cand);
    }
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
    const double px = xyz[3 * i], py = xyz[3 * i + 1], pz = xyz[3 * i + 2];
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
    out[i] = add_rn(mul_rn(c0, sub_rn(1.0, t[2])), mul_rn(c1, t[2]));
}

template <typename Real>
constexpr size_t grid_smem_bytes() {
    auto up = [](size_t b) { return (b + 127) & ~(size_t)127; };
    return up(2 * TILE * sizeof(ImageRec)) + up(TILE * sizeof(float4)) +
           up((sizeof(Real) == 4 ? TILE : 1) * sizeof(float4)) +
           up((sizeof(Real) == 4 ? NPT * 3 * THREADS : 1) * sizeof(float)) + up(2 * sizeof(uint64_t)) +
           up(MAX_ROWS * sizeof(uint32_t)) + up((MAX_ROWS + 1) * sizeof(uint32_t)) +
           up((THREADS / 32) * sizeof(uint32_t)) + up(64 * MAX_NG * sizeof(ParamF)) +
           up(64 * sizeof(float)) + up(TILE * sizeof(uint16_t)) +
           up(64 * MAX_NG * sizeof(PairParams));
}

template <typename Real, int NG, int TRUNC>
void launch_one(dim3 grid, cudaStream_t s, const GridGeom& geo, const ImageRec* images,
                const uint32_t* bins, const PairParams* params, const uint32_t* guests,
                double* tables, unsigned long long* executed, unsigned* flags) {
    constexpr size_t bytes = grid_smem_bytes<Real>();
    // opt in to more than 48 KB of dynamic shared memory (per device, cheap)
    ALEA_CUDA(cudaFuncSetAttribute(grid_build_kernel<Real, NG, TRUNC>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    grid_build_kernel<Real, NG, TRUNC>
        <<<grid, THREADS, bytes, s>>>(geo, images, bins, params, guests, tables, executed, flags);
}

template <typename Real, int NG>
void launch_build_t(int trunc, dim3 grid, cudaStream_t s, const GridGeom& geo,
                    const ImageRec* images, const uint32_t* bins, const PairParams* params,
                    const uint32_t* guests, double* tables, unsigned long long* executed,
                    unsigned* flags) {
    if (trunc == ALEA_TRUNCATED)
        launch_one<Real, NG, ALEA_TRUNCATED>(grid, s, geo, images, bins, params, guests, tables, executed, flags);
    else if (trunc == ALEA_SHIFTED)
        launch_one<Real, NG, ALEA_SHIFTED>(grid, s, geo, images, bins, params, guests, tables, executed, flags);
    else
        launch_one<Real, NG, ALEA_LINEAR_FORCE_SHIFTED>(grid, s, geo, images, bins, params, guests, tables, executed, flags);
}

template <typename Real>
void launch_build(int ng, int trunc, dim3 grid, cudaStream_t s, const GridGeom& geo,
                  const ImageRec* images, const uint32_t* bins, const PairParams* params,
                  const uint32_t* guests, double* tables, unsigned long long* executed,
                  unsigned* flags) {
    switch (ng) {
        case 1: launch_build_t<Real, 1>(trunc, grid, s, geo, images, bins, params, guests, tables, executed, flags); break;
        case 2: launch_build_t<Real, 2>(trunc, grid, s, geo, images, bins, params, guests, tables, executed, flags); break;
        case 3: launch_build_t<Real, 3>(trunc, grid, s, geo, images, bins, params, guests, tables, executed, flags); break;
        default: launch_build_t<Real, 4>(trunc, grid, s, geo, images, bins, params, guests, tables, executed, flags); break;
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
    DevBuf<ImageRec> images;
    DevBuf<uint32_t> bin_start;
    DevBuf<PairParams> params;
    DevBuf<uint32_t> guests;
    DevBuf<double> tables;
    DevBuf<unsigned long long> executed;
    DevBuf<unsigned> flags;
    uint64_t n_images = 0;
    uint64_t executed_pairs = 0;
    float last_ms = 0.f;
};

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
    validate_cutoff(g.geo.L, lj.cutoff, "FrameworkEnergyGrid");
    g.precision = precision;
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

    // metric tensor and extents
    const double* m = g.geo.L.m;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            g.geo.G[3 * i + j] = m[3 * i] * m[3 * j] + m[3 * i + 1] * m[3 * j + 1] + m[3 * i + 2] * m[3 * j + 2];
    for (int i = 0; i < 9; ++i) g.geo.Gf[i] = (float)g.geo.G[i];
    g.geo.rc = lj.cutoff;
    g.geo.rc2 = lj.cutoff * lj.cutoff;
    // widen the bins until no brick can touch more than MAX_ROWS bin rows
    for (int attempt = 0; attempt < 64; ++attempt) {
        int span_bins[3];
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
    for (int a = 0; a < 3; ++a) {
        const double h = lj.cutoff / g.geo.L.perp[a];
        g.geo.lo[a] = -h - 1e-7;
        g.geo.hi[a] = (double)(g.geo.n[a] - 1) / g.geo.n[a] + h + 1e-7;
        const double span = g.geo.hi[a] - g.geo.lo[a];
        g.geo.nb[a] = std::max(1, (int)std::ceil(span * g.geo.L.perp[a] / bin_width));
        g.geo.binw[a] = span / g.geo.nb[a];
        g.geo.lof[a] = (float)g.geo.lo[a];
        g.geo.binwf[a] = (float)g.geo.binw[a];
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
    g.images.alloc(std::max<size_t>(sorted.size(), 1));
    g.images.upload(sorted.data(), sorted.size());
    g.bin_start.alloc(start.size());
    g.bin_start.upload(start.data(), start.size());

    std::vector<PairParams> table((size_t)lj.n_species * lj.n_species);
    mixed_table(lj, table.data());
    // reach of the FP32 form's close pass: largest mixed sigma of these guests
    // plus the half-diagonal of a brick (triangle inequality bound)
    {
        double smax = 0.0;
        for (uint32_t gs : sp)
            for (uint32_t t = 0; t < lj.n_species; ++t)
                smax = std::max(smax, table[(size_t)gs * lj.n_species + t].sigma);
        double half = 0.0;
        const int bd[3] = {BX, BY, BZ};
        for (int a = 0; a < 3; ++a) {
            const double f = (double)(bd[a] - 1) / g.geo.n[a];
            half += 0.5 * f * std::sqrt(m[3 * a] * m[3 * a] + m[3 * a + 1] * m[3 * a + 1] + m[3 * a + 2] * m[3 * a + 2]);
        }
        const double reach = smax * (1.0 + 1e-5) + half + 1e-3;
        g.geo.near2 = (float)(reach * reach);
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

static void run_build(GridImpl& g, cudaStream_t s) {
    const int ng = (int)g.species.size();
    const size_t nodes = (size_t)g.geo.n[0] * g.geo.n[1] * g.geo.n[2];
    const uint64_t nbricks = (uint64_t)g.geo.bricks[0] * g.geo.bricks[1] * g.geo.bricks[2];
    require(nbricks < (1ull << 31), ALEA_ERR_INVALID_ARGUMENT, "grid too large");
    ALEA_CUDA(cudaMemsetAsync(g.executed.p, 0, sizeof(unsigned long long), s));
    cudaEvent_t e0, e1;
    ALEA_CUDA(cudaEventCreate(&e0));
    ALEA_CUDA(cudaEventCreate(&e1));
    ALEA_CUDA(cudaEventRecord(e0, s));
    for (int g0 = 0; g0 < ng; g0 += MAX_NG) {
        const int cnt = std::min(MAX_NG, ng - g0);
        dim3 grid((unsigned)nbricks);
        if (g.precision == ALEA_FP32)
            launch_build<float>(cnt, g.truncation, grid, s, g.geo, g.images.p, g.bin_start.p,
                                g.params.p, g.guests.p + g0, g.tables.p + (size_t)g0 * nodes,
                                g.executed.p, g.flags.p);
        else
            launch_build<double>(cnt, g.truncation, grid, s, g.geo, g.images.p, g.bin_start.p,
                                 g.params.p, g.guests.p + g0, g.tables.p + (size_t)g0 * nodes,
                                 g.executed.p, g.flags.p);
        ALEA_CUDA(cudaGetLastError());
    }
    ALEA_CUDA(cudaEventRecord(e1, s));
    ALEA_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    ALEA_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    g.last_ms = ms;
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
        build_plan(*g, lj, fw, lat, guest, n_guest, spacing, precision, 2.0);
        run_build(*g, 0);
    } catch (...) {
        delete g;
        throw;
    }
    return g;
}

void grid_rebuild(GridImpl* g, cudaStream_t s) { run_build(*g, s); }
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

void grid_interpolate_device(const GridImpl* g, uint32_t species, const double* xyz, uint64_t n,
                             double* out, cudaStream_t s) {
    const double* tab = grid_table(g, species);
    if (n == 0) return;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    grid_interpolate_kernel<<<blocks, 256, 0, s>>>(g->geo.L, g->geo.n[0], g->geo.n[1], g->geo.n[2],
                                                  tab, xyz, n, out);
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
}

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
