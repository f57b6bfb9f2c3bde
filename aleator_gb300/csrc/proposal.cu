// Learned insertion proposal: a Fourier-feature MLP log-density over the
// unit cell, trained on Boltzmann-weighted Widom samples, tabulated into an
// exactly normalised piecewise-constant density that Widom and GCMC sample
// from.
//
// No counterpart in the reference (its insertions are uniform,
// monte_carlo_engine.cc:572-574, 882-884). The network: fractional position
// s in [0, 1)^3 -> 2 n_freq periodic features (sin, cos)(2 pi k_j . s) with
// integer wave vectors k_j -> depth hidden layers of `width` with SiLU ->
// one output f(s), an unnormalised log-density. Weights are rounded to BF16
// (the copy the kernels read) from FP32 master weights that Adam updates;
// activations and gradients are FP32. The hidden layers' products run on the
// tensor cores (mma.sync m16n8k16, BF16 operands, FP32 accumulation) with each
// FP32 operand split into BF16 hi + lo parts (tc_gemm_kernel); the one-unit
// output layer, the loss and Adam stay in FP32 on the CUDA cores.
//
// Training rows {s0, s1, s2, l, lq}: a position, its log-weight l = -dU/T and
// the log density lq of the proposal it was drawn from (relative to uniform;
// 0 for uniform trials). Objective on a batch: the cross-entropy between the
// Boltzmann distribution (tempered by tau) and the model, both importance
// weighted by 1/q,
//     L = -sum_i softmax(tau l - lq)_i f_i + log mean_i exp(f_i - lq_i),
// whose gradient in f is softmax(f - lq)_i - softmax(tau l - lq)_i. The second
// term estimates log of the normaliser of exp f over the cell, so L is the
// weighted negative log-likelihood of the density exp f / Z; rows drawn from
// an earlier proposal refine it where the Boltzmann weight lies.
//
// The proposal actually sampled is the network tabulated on cells^3 cell
// centres, mixed with a uniform share: P_c = (1 - u) softmax(f)_c + u / N.
// A trial picks cell c from the CDF and a uniform point inside it, so its
// density relative to uniform, N P_c, is known exactly and enters the
// importance weight (Widom) and the acceptance ratio (GCMC).
//
// Layout (row-major): W_l is [out x in], then b_l; layers 64->w, w->w (depth-1
// times), w->1. Matrices of a batch are [batch x features].

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "grid.cuh"

namespace alea {

namespace {

constexpr int GT = 64, GK = 16;  // GEMM tile (M and N) and k-step
constexpr int GTHREADS = 256;    // 16 x 16 threads, 4 x 4 outputs each
constexpr int ROW = ALEA_SAMPLE_ROW;  // floats per training row {s0, s1, s2, l, lq}

enum { EPI_STORE = 0, EPI_BIAS = 1, EPI_BIAS_SILU = 2, EPI_SILU_GRAD = 3 };

__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }
template <typename T>
__device__ __forceinline__ T from_f(float v);
template <>
__device__ __forceinline__ float from_f<float>(float v) { return v; }
template <>
__device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

__device__ __forceinline__ float sigmoidf(float z) { return 1.0f / (1.0f + __expf(-z)); }

// C = op(A) op(B) with op(A)[m][k] = TA ? A[k lda + m] : A[m lda + k] and
// op(B)[k][n] = TB ? B[n ldb + k] : B[k ldb + n]. Split over k by blockIdx.z
// (k_chunk per slice): EPI_STORE slices write to C + z M ldc.
// Epilogues: EPI_BIAS: C = acc + bias[n]; EPI_BIAS_SILU: aux = acc + bias[n]
// (pre-activation), C = SiLU(aux); EPI_SILU_GRAD: C = acc SiLU'(aux).
template <bool TA, bool TB, typename AT, typename BT, typename CT, int EPI>
__global__ void __launch_bounds__(GTHREADS)
gemm_kernel(int M, int N, int K, const AT* __restrict__ A, int lda, const BT* __restrict__ B,
            int ldb, CT* __restrict__ C, int ldc, const float* __restrict__ bias,
            float* __restrict__ aux, int k_chunk) {
    __shared__ float As[GK][GT + 4];
    __shared__ float Bs[GK][GT + 4];
    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;
    const int m0 = blockIdx.y * GT, n0 = blockIdx.x * GT;
    const int kb = blockIdx.z * k_chunk;
    const int ke = min(K, kb + k_chunk);
    float acc[4][4] = {};
    for (int k0 = kb; k0 < ke; k0 += GK) {
        for (int e = tid; e < GT * GK; e += GTHREADS) {
            int mm, kk;
            if (TA) { mm = e % GT; kk = e / GT; } else { kk = e % GK; mm = e / GK; }
            const int m = m0 + mm, k = k0 + kk;
            As[kk][mm] = (m < M && k < ke) ? to_f(TA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k]) : 0.f;
        }
        for (int e = tid; e < GT * GK; e += GTHREADS) {
            int nn, kk;
            if (TB) { kk = e % GK; nn = e / GK; } else { nn = e % GT; kk = e / GT; }
            const int n = n0 + nn, k = k0 + kk;
            Bs[kk][nn] = (n < N && k < ke) ? to_f(TB ? B[(size_t)n * ldb + k] : B[(size_t)k * ldb + n]) : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
    CT* Cz = C + (EPI == EPI_STORE ? (size_t)blockIdx.z * M * ldc : 0);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + ty * 4 + i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int n = n0 + tx * 4 + j;
            if (n >= N) continue;
            const size_t o = (size_t)m * ldc + n;
            float v = acc[i][j];
            if (EPI == EPI_BIAS) {
                v += bias[n];
            } else if (EPI == EPI_BIAS_SILU) {
                v += bias[n];
                aux[o] = v;
                v = v * sigmoidf(v);
            } else if (EPI == EPI_SILU_GRAD) {
                const float z = aux[o], sg = sigmoidf(z);
                v *= sg * (1.0f + z * (1.0f - sg));
            }
            Cz[o] = from_f<CT>(v);
        }
    }
}

// ---------------------------------------------------------------- tensor-core GEMM
// C[M x N] = op(A) op(B) on the tensor cores (mma.sync m16n8k16, BF16 operands,
// FP32 accumulation), with the same op() convention and epilogues as
// gemm_kernel. An FP32 operand (the activations and gradients) is split into
// BF16 hi + lo parts when it is staged, and its products are summed from
// hi x hi, lo x hi and hi x lo MMAs: ~16 significant bits per operand, the
// FP32 activations' precision for these sums; a BF16 operand (the weights,
// which are BF16 by design) has no lo part. A 64 x 64 tile per CTA of 4 warps
// (each 32 x 32: 2 x 4 MMA tiles), k-steps of 32 staged in shared memory as
// As[m][k] and Bs[n][k] (k contiguous, whatever the global layout) and read
// with ldmatrix. EPI_STORE writes split-K partials to C + z M ldc; with bpart,
// the CTAs of the first column of tiles also write the row sums of op(A) over
// their k-slice to bpart[z M + m] (the bias gradient when op(A) = dz^T).
constexpr int TC_T = 64, TC_K = 32, TC_PAD = 8, TC_THREADS = 128;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16& hi, __nv_bfloat16& lo) {
    hi = __float2bfloat16_rn(x);
    lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}
__device__ __forceinline__ void split_bf16(__nv_bfloat16 x, __nv_bfloat16& hi, __nv_bfloat16& lo) {
    hi = x;
    lo = __float2bfloat16_rn(0.f);
}

__device__ __forceinline__ void ldm_x4(uint32_t (&r)[4], const __nv_bfloat16* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, "
        "{%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

template <bool TA, bool TB, typename AT, typename BT, typename CT, int EPI>
__global__ void __launch_bounds__(TC_THREADS)
tc_gemm_kernel(int M, int N, int K, const AT* __restrict__ A, int lda, const BT* __restrict__ B,
               int ldb, CT* __restrict__ C, int ldc, const float* __restrict__ bias,
               float* __restrict__ aux, int k_chunk, float* __restrict__ bpart) {
    constexpr bool SA = std::is_same<AT, float>::value;  // A has a lo part
    constexpr bool SB = std::is_same<BT, float>::value;  // B has a lo part
    __shared__ __align__(16) __nv_bfloat16 Ah[TC_T][TC_K + TC_PAD], Al[SA ? TC_T : 1][TC_K + TC_PAD];
    __shared__ __align__(16) __nv_bfloat16 Bh[TC_T][TC_K + TC_PAD], Bl[SB ? TC_T : 1][TC_K + TC_PAD];
    __shared__ float brow[TC_T];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp >> 1, wn = warp & 1;  // this warp's 32 x 32 quarter
    const int m0 = blockIdx.y * TC_T, n0 = blockIdx.x * TC_T;
    const int kb = blockIdx.z * k_chunk;
    const int ke = min(K, kb + k_chunk);
    const bool row_sums = bpart != nullptr && blockIdx.x == 0;
    float acc[2][4][4] = {};
    float rs = 0.f;  // row sum of op(A) over the slice (thread tid < 64 owns row tid)
    for (int k0 = kb; k0 < ke; k0 += TC_K) {
        // stage op(A)[m0.., k0..] as A[m][k] and op(B)[k0.., n0..] as B[n][k]
        for (int e = tid; e < TC_T * TC_K; e += TC_THREADS) {
            int mm, kk;
            if (TA) { mm = e % TC_T; kk = e / TC_T; } else { kk = e % TC_K; mm = e / TC_K; }
            const int m = m0 + mm, k = k0 + kk;
            const AT v = (m < M && k < ke) ? (TA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k]) : AT(0.f);
            __nv_bfloat16 hi, lo;
            split_bf16(v, hi, lo);
            Ah[mm][kk] = hi;
            if constexpr (SA) Al[mm][kk] = lo;
        }
        for (int e = tid; e < TC_T * TC_K; e += TC_THREADS) {
            int nn, kk;
            if (TB) { kk = e % TC_K; nn = e / TC_K; } else { nn = e % TC_T; kk = e / TC_T; }
            const int n = n0 + nn, k = k0 + kk;
            const BT v = (n < N && k < ke) ? (TB ? B[(size_t)n * ldb + k] : B[(size_t)k * ldb + n]) : BT(0.f);
            __nv_bfloat16 hi, lo;
            split_bf16(v, hi, lo);
            Bh[nn][kk] = hi;
            if constexpr (SB) Bl[nn][kk] = lo;
        }
        __syncthreads();
        if (row_sums && tid < TC_T) {
            const int m = m0 + tid;
            if (m < M)
                for (int k = k0; k < min(ke, k0 + TC_K); ++k)
                    rs += to_f(TA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k]);
        }
#pragma unroll
        for (int ks = 0; ks < TC_K; ks += 16) {
            uint32_t ah[2][4], al[2][4], bh[4][2], bl[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = wm * 32 + i * 16 + (lane & 15), c = ks + (lane >> 4) * 8;
                ldm_x4(ah[i], &Ah[r][c]);
                if constexpr (SA) ldm_x4(al[i], &Al[r][c]);
            }
#pragma unroll
            for (int j = 0; j < 4; j += 2) {
                // matrices: (n j8.., k ks), (n j8.., k ks+8), (n j8+8.., k ks), (n j8+8.., k ks+8)
                const int r = wn * 32 + j * 8 + (lane & 7) + ((lane >> 4) << 3);
                const int c = ks + ((lane >> 3) & 1) * 8;
                uint32_t t[4];
                ldm_x4(t, &Bh[r][c]);
                bh[j][0] = t[0]; bh[j][1] = t[1]; bh[j + 1][0] = t[2]; bh[j + 1][1] = t[3];
                if constexpr (SB) {
                    ldm_x4(t, &Bl[r][c]);
                    bl[j][0] = t[0]; bl[j][1] = t[1]; bl[j + 1][0] = t[2]; bl[j + 1][1] = t[3];
                }
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    mma_bf16(acc[i][j], ah[i], bh[j][0], bh[j][1]);
                    if constexpr (SA) mma_bf16(acc[i][j], al[i], bh[j][0], bh[j][1]);
                    if constexpr (SB) mma_bf16(acc[i][j], ah[i], bl[j][0], bl[j][1]);
                }
        }
        __syncthreads();
    }
    if (row_sums && tid < TC_T) brow[tid] = rs;
    CT* Cz = C + (EPI == EPI_STORE ? (size_t)blockIdx.z * M * ldc : 0);
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                // C fragment: rows lane/4 (+8 for h >= 2), columns 2 (lane % 4) + (h & 1)
                const int m = m0 + wm * 32 + i * 16 + (lane >> 2) + ((h >> 1) << 3);
                const int n = n0 + wn * 32 + j * 8 + 2 * (lane & 3) + (h & 1);
                if (m >= M || n >= N) continue;
                const size_t o = (size_t)m * ldc + n;
                float v = acc[i][j][h];
                if (EPI == EPI_BIAS) {
                    v += bias[n];
                } else if (EPI == EPI_BIAS_SILU) {
                    v += bias[n];
                    aux[o] = v;
                    v = v * sigmoidf(v);
                } else if (EPI == EPI_SILU_GRAD) {
                    const float z = aux[o], sg = sigmoidf(z);
                    v *= sg * (1.0f + z * (1.0f - sg));
                }
                Cz[o] = from_f<CT>(v);
            }
    if (row_sums) {
        __syncthreads();
        if (tid < TC_T && m0 + tid < M) bpart[(size_t)blockIdx.z * M + m0 + tid] = brow[tid];
    }
}

// out[i] = sum over slices of part[z][i], in slice order.
__global__ void reduce_slices_kernel(const float* __restrict__ part, int slices, size_t n,
                                     float* __restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = 0.f;
    for (int z = 0; z < slices; ++z) s += part[(size_t)z * n + i];
    out[i] = s;
}

// The weight and bias gradients of a layer from their split-K partials, in
// slice order: out_w[i] = sum_z pw[z][i] (cnt entries), out_b[i] = sum_z pb[z][i].
__global__ void reduce_wb_kernel(const float* __restrict__ pw, const float* __restrict__ pb,
                                 int slices, size_t cnt, size_t nb, float* __restrict__ out_w,
                                 float* __restrict__ out_b) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < cnt) {
        float s = 0.f;
        for (int z = 0; z < slices; ++z) s += pw[(size_t)z * cnt + i];
        out_w[i] = s;
    } else if (i < cnt + nb) {
        const size_t j = i - cnt;
        float s = 0.f;
        for (int z = 0; z < slices; ++z) s += pb[(size_t)z * nb + j];
        out_b[j] = s;
    }
}

// Column sums of X [rows x cols] in a fixed order: per column, rows are
// summed by slices of `chunk` into part[slice][col], then reduce_slices.
template <typename XT>
__global__ void colsum_part_kernel(const XT* __restrict__ X, int rows, int cols, int chunk,
                                   float* __restrict__ part) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    const int r0 = blockIdx.y * chunk, r1 = min(rows, r0 + chunk);
    float s = 0.f;
    for (int r = r0; r < r1; ++r) s += to_f(X[(size_t)r * cols + c]);
    part[(size_t)blockIdx.y * cols + c] = s;
}

// Fourier features of rows with stride `stride` floats (s at 0..2):
// phi[i][j] = sin(2 pi k_j . s_i), phi[i][nf + j] = cos(2 pi k_j . s_i).
// idx (optional) gathers rows: sample = idx ? idx(i) : i.
__global__ void features_kernel(const float* __restrict__ samples, int stride, uint64_t n,
                                uint64_t perm_a, uint64_t perm_c, uint64_t pool,
                                const float* __restrict__ kvec, int nf, float* __restrict__ phi) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t src = pool ? (perm_a * i + perm_c) % pool : i;
    const float* s = samples + src * stride;
    for (int j = 0; j < nf; ++j) {
        const float t = kvec[3 * j] * s[0] + kvec[3 * j + 1] * s[1] + kvec[3 * j + 2] * s[2];
        float sn, cs;
        sincospif(2.0f * (t - floorf(t)), &sn, &cs);
        phi[i * 2 * nf + j] = sn;
        phi[i * 2 * nf + nf + j] = cs;
    }
}

// Batch softmax statistics, stage 1: per block of 256 rows, with
// a = f - lq and t = tau l - lq (gathered like the features):
// {max a, sum e^(a - max a), max t, sum e^(t - max t), sum e^(t - max t) f}.
__global__ void loss_part_kernel(const float* __restrict__ f, const float* __restrict__ samples,
                                 int stride, uint64_t n, uint64_t perm_a, uint64_t perm_c,
                                 uint64_t pool, double tau, double* __restrict__ part) {
    __shared__ double sh[256];
    const uint64_t i = (uint64_t)blockIdx.x * 256 + threadIdx.x;
    const bool on = i < n;
    double fv = 0.0, av = -INFINITY, lv = -INFINITY;
    if (on) {
        const uint64_t src = pool ? (perm_a * i + perm_c) % pool : i;
        const double lq = (double)samples[src * stride + 4];
        fv = f[i];
        av = fv - lq;
        lv = tau * (double)samples[src * stride + 3] - lq;
    }
    auto bmax = [&](double v) {
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int s = 128; s > 0; s >>= 1) {
            if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
            __syncthreads();
        }
        const double r = sh[0];
        __syncthreads();
        return r;
    };
    auto bsum = [&](double v) {
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int s = 128; s > 0; s >>= 1) {
            if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
            __syncthreads();
        }
        const double r = sh[0];
        __syncthreads();
        return r;
    };
    const double mf = bmax(av), ml = bmax(lv);
    const double ef = on ? exp(av - mf) : 0.0;
    const double el = (on && ml > -INFINITY) ? exp(lv - ml) : 0.0;
    const double sf = bsum(ef), sl = bsum(el), tl = bsum(el * fv);
    if (threadIdx.x == 0) {
        double* p = part + 5 * blockIdx.x;
        p[0] = mf;
        p[1] = sf;
        p[2] = ml;
        p[3] = sl;
        p[4] = tl;
    }
}

// Stage 2 (one thread, block order): stats = {Mf, Sf, Ml, Sl, loss}.
__global__ void loss_combine_kernel(const double* __restrict__ part, int nb, uint64_t n,
                                    double* __restrict__ stats) {
    if (threadIdx.x || blockIdx.x) return;
    double mf = -INFINITY, ml = -INFINITY;
    for (int b = 0; b < nb; ++b) {
        mf = fmax(mf, part[5 * b]);
        ml = fmax(ml, part[5 * b + 2]);
    }
    double sf = 0, sl = 0, tl = 0;
    for (int b = 0; b < nb; ++b) {
        sf += part[5 * b + 1] * exp(part[5 * b] - mf);
        if (part[5 * b + 2] > -INFINITY) {
            const double r = exp(part[5 * b + 2] - ml);
            sl += part[5 * b + 3] * r;
            tl += part[5 * b + 4] * r;
        }
    }
    stats[0] = mf;
    stats[1] = sf;
    stats[2] = ml;
    stats[3] = sl;
    stats[4] = -(tl / sl) + (mf + log(sf / (double)n));
}

// g_i = softmax(f - lq)_i - softmax(tau l - lq)_i
__global__ void loss_grad_kernel(const float* __restrict__ f, const float* __restrict__ samples,
                                 int stride, uint64_t n, uint64_t perm_a, uint64_t perm_c,
                                 uint64_t pool, double tau, const double* __restrict__ stats,
                                 float* __restrict__ g) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t src = pool ? (perm_a * i + perm_c) % pool : i;
    const double lq = (double)samples[src * stride + 4];
    const double lv = tau * (double)samples[src * stride + 3] - lq;
    const double pf = exp((double)f[i] - lq - stats[0]) / stats[1];
    const double pl = exp(lv - stats[2]) / stats[3];
    g[i] = (float)(pf - pl);
}

// Adam on the FP32 master weights, then the BF16 copy the kernels read.
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v,
                            __nv_bfloat16* __restrict__ wb, uint64_t n, float lr, float b1,
                            float b2, float eps, float c1, float c2) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    wb[i] = __float2bfloat16_rn(wi);
}

__global__ void to_bf16_kernel(const float* __restrict__ w, __nv_bfloat16* __restrict__ wb, uint64_t n) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) wb[i] = __float2bfloat16_rn(w[i]);
}

// Cell centres of a cells^3 table as rows (stride ROW; x fastest).
__global__ void cell_centres_kernel(int cells, uint64_t first, uint64_t n, float* __restrict__ out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t c = first + i;
    const uint64_t ix = c % cells, iy = (c / cells) % cells, iz = c / ((uint64_t)cells * cells);
    float* o = out + ROW * i;
    o[0] = (ix + 0.5f) / cells;
    o[1] = (iy + 0.5f) / cells;
    o[2] = (iz + 0.5f) / cells;
    o[3] = 0.f;
    o[4] = 0.f;
}

unsigned blocks_for(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

struct ProposalImpl {
    int nf = 32, width = 128, depth = 3;
    int fmax = 6;
    uint64_t seed = 0;
    std::vector<int32_t> kint;
    DevBuf<float> kvec;
    uint64_t n_params = 0;
    std::vector<uint64_t> woff, boff;  // per layer: weight and bias offsets
    std::vector<int> lin, lout;        // per layer: in and out width
    DevBuf<float> w, m, v, g;
    DevBuf<__nv_bfloat16> wb;
    uint64_t adam_t = 0;
    // batch workspace
    uint64_t cap = 0;
    DevBuf<float> phi, f, gf, dz_a, dz_b, part, bpart;
    std::vector<DevBuf<float>> z, h;  // per hidden layer: pre-activation, SiLU output
    DevBuf<double> lpart, stats;
    // tabulated proposal
    int cells = 0;
    double uniform_share = 1.0;
    DevBuf<double> cdf;
    DevBuf<double> logp;
    std::vector<double> logp_host;
};

static void ensure_capacity(ProposalImpl& P, uint64_t n) {
    if (n <= P.cap) return;
    P.cap = n;
    P.phi.alloc(n * 2 * P.nf);
    P.f.alloc(n);
    P.gf.alloc(n);
    P.dz_a.alloc(n * P.width);
    P.dz_b.alloc(n * P.width);
    P.z.clear();
    P.h.clear();
    for (int l = 0; l < P.depth; ++l) {
        P.z.emplace_back(n * P.width);
        P.h.emplace_back(n * P.width);
    }
    P.lpart.alloc(blocks_for(n, 256) * 5);
}

template <bool TA, bool TB, int EPI, typename AT, typename BT, typename CT>
static void gemm(cudaStream_t s, int M, int N, int K, const AT* A, int lda, const BT* B, int ldb,
                 CT* C, int ldc, const float* bias = nullptr, float* aux = nullptr,
                 int slices = 1) {
    const int chunk = slices > 1 ? ((K + slices - 1) / slices + GK - 1) / GK * GK : K;
    dim3 grid((unsigned)((N + GT - 1) / GT), (unsigned)((M + GT - 1) / GT), (unsigned)slices);
    gemm_kernel<TA, TB, AT, BT, CT, EPI><<<grid, GTHREADS, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc,
                                                                  bias, aux, chunk);
    ALEA_CUDA(cudaGetLastError());
}

template <bool TA, bool TB, int EPI, typename AT, typename BT, typename CT>
static void tc_gemm(cudaStream_t s, int M, int N, int K, const AT* A, int lda, const BT* B, int ldb,
                    CT* C, int ldc, const float* bias = nullptr, float* aux = nullptr,
                    int slices = 1, float* bpart = nullptr) {
    const int chunk = slices > 1 ? ((K + slices - 1) / slices + TC_K - 1) / TC_K * TC_K : K;
    dim3 grid((unsigned)((N + TC_T - 1) / TC_T), (unsigned)((M + TC_T - 1) / TC_T), (unsigned)slices);
    tc_gemm_kernel<TA, TB, AT, BT, CT, EPI><<<grid, TC_THREADS, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc,
                                                               bias, aux, chunk, bpart);
    ALEA_CUDA(cudaGetLastError());
}

// Forward over n rows (stride ROW, gathered through the affine
// permutation when pool > 0): f[i] and the per-layer z, h.
static void forward(ProposalImpl& P, const float* samples, uint64_t n, uint64_t pa, uint64_t pc,
                    uint64_t pool, cudaStream_t s) {
    ensure_capacity(P, n);
    features_kernel<<<blocks_for(n, 256), 256, 0, s>>>(samples, ROW, n, pa, pc, pool, P.kvec.p, P.nf,
                                                       P.phi.p);
    ALEA_CUDA(cudaGetLastError());
    const float* in = P.phi.p;
    for (int l = 0; l < P.depth; ++l) {  // tensor cores: h_l = SiLU(h_{l-1} W_l^T + b_l)
        tc_gemm<false, true, EPI_BIAS_SILU>(s, (int)n, P.lout[l], P.lin[l], in, P.lin[l],
                                            P.wb.p + P.woff[l], P.lin[l], P.h[l].p, P.lout[l],
                                            P.w.p + P.boff[l], P.z[l].p);
        in = P.h[l].p;
    }
    const int L = P.depth;
    // the one-unit output layer on the CUDA cores; biases are read in FP32 (not rounded)
    gemm<false, true, EPI_BIAS>(s, (int)n, 1, P.width, in, P.width, P.wb.p + P.woff[L], P.width,
                                P.f.p, 1, P.w.p + P.boff[L]);
}

// Loss and gradient for a batch: fills P.g and returns the loss.
static double loss_grad(ProposalImpl& P, const float* samples, uint64_t n, uint64_t pa, uint64_t pc,
                        uint64_t pool, double tau, cudaStream_t s, bool want_loss = true) {
    forward(P, samples, n, pa, pc, pool, s);
    const unsigned nb = blocks_for(n, 256);
    loss_part_kernel<<<nb, 256, 0, s>>>(P.f.p, samples, ROW, n, pa, pc, pool, tau, P.lpart.p);
    loss_combine_kernel<<<1, 1, 0, s>>>(P.lpart.p, (int)nb, n, P.stats.p);
    loss_grad_kernel<<<nb, 256, 0, s>>>(P.f.p, samples, ROW, n, pa, pc, pool, tau, P.stats.p, P.gf.p);
    ALEA_CUDA(cudaGetLastError());
    const int W = P.width, L = P.depth;
    const int slices = (int)std::min<uint64_t>(64, std::max<uint64_t>(1, n / 1024));
    auto need_parts = [&](size_t cnt, size_t nb) {
        if ((size_t)slices * cnt > P.part.n) P.part.alloc((size_t)slices * cnt);
        if ((size_t)slices * nb > P.bpart.n) P.bpart.alloc((size_t)slices * nb);
    };
    // output layer (one unit, CUDA cores): dW_L = g^T h_{L-1}, db_L = sum g
    {
        const size_t cnt = (size_t)W;
        need_parts(cnt, 1);
        gemm<true, false, EPI_STORE>(s, 1, W, (int)n, P.gf.p, 1, P.h[L - 1].p, W, P.part.p, W,
                                     nullptr, nullptr, slices);
        const int chunk = (int)((n + slices - 1) / slices);
        colsum_part_kernel<<<dim3(1, slices), 128, 0, s>>>(P.gf.p, (int)n, 1, chunk, P.bpart.p);
        reduce_wb_kernel<<<blocks_for(cnt + 1, 256), 256, 0, s>>>(P.part.p, P.bpart.p, slices, cnt, 1,
                                                                  P.g.p + P.woff[L], P.g.p + P.boff[L]);
        ALEA_CUDA(cudaGetLastError());
    }
    // dz_{L-1} = (g W_L) SiLU'(z_{L-1}) (rank one, CUDA cores)
    float* dz = P.dz_a.p;
    float* dz_next = P.dz_b.p;
    gemm<false, false, EPI_SILU_GRAD>(s, (int)n, W, 1, P.gf.p, 1, P.wb.p + P.woff[L], W, dz, W,
                                      nullptr, P.z[L - 1].p);
    for (int l = L - 1; l >= 0; --l) {
        const float* hin = l > 0 ? P.h[l - 1].p : P.phi.p;
        // tensor cores: dW_l = dz_l^T h_{l-1} split over samples, with the bias
        // gradient (the row sums of dz_l^T) in the same launch; then both reduced
        // in slice order by one launch
        const size_t cnt = (size_t)P.lout[l] * P.lin[l];
        need_parts(cnt, (size_t)P.lout[l]);
        tc_gemm<true, false, EPI_STORE>(s, P.lout[l], P.lin[l], (int)n, dz, P.lout[l], hin, P.lin[l],
                                        P.part.p, P.lin[l], nullptr, nullptr, slices, P.bpart.p);
        reduce_wb_kernel<<<blocks_for(cnt + P.lout[l], 256), 256, 0, s>>>(
            P.part.p, P.bpart.p, slices, cnt, (size_t)P.lout[l], P.g.p + P.woff[l], P.g.p + P.boff[l]);
        ALEA_CUDA(cudaGetLastError());
        if (l > 0) {
            // dz_{l-1} = (dz_l W_l) SiLU'(z_{l-1}) on the tensor cores
            tc_gemm<false, false, EPI_SILU_GRAD>(s, (int)n, P.lin[l], P.lout[l], dz, P.lout[l],
                                                 P.wb.p + P.woff[l], P.lin[l], dz_next, P.lin[l],
                                                 nullptr, P.z[l - 1].p);
            std::swap(dz, dz_next);
        }
    }
    if (!want_loss) return 0.0;
    double st[5];
    ALEA_CUDA(cudaMemcpyAsync(st, P.stats.p, sizeof(st), cudaMemcpyDeviceToHost, s));
    ALEA_CUDA(cudaStreamSynchronize(s));
    return st[4];
}

ProposalImpl* proposal_create(const alea_proposal_config& c) {
    require(c.n_freq >= 1 && c.n_freq <= 256, ALEA_ERR_INVALID_ARGUMENT,
            "alea_proposal_create: n_freq must be 1..256");
    require(c.width >= 1 && c.width <= 1024, ALEA_ERR_INVALID_ARGUMENT,
            "alea_proposal_create: width must be 1..1024");
    require(c.depth >= 1 && c.depth <= 8, ALEA_ERR_INVALID_ARGUMENT,
            "alea_proposal_create: depth must be 1..8");
    require(c.freq_max >= 1 && c.freq_max <= 64, ALEA_ERR_INVALID_ARGUMENT,
            "alea_proposal_create: freq_max must be 1..64");
    require_device();
    auto* P = new ProposalImpl();
    P->nf = (int)c.n_freq;
    P->width = (int)c.width;
    P->depth = (int)c.depth;
    P->fmax = (int)c.freq_max;
    P->seed = c.seed;
    // wave vectors: components uniform in [-fmax, fmax], not all zero (Philox
    // stream 1 of the seed)
    uint64_t call = 0;
    const int span = 2 * P->fmax + 1;
    for (int j = 0; j < P->nf; ++j) {
        int k[3];
        do {
            for (int a = 0; a < 3; ++a) {
                const double u = philox_uniform(c.seed, 1, call++);
                k[a] = std::min(span - 1, (int)(u * span)) - P->fmax;
            }
        } while (k[0] == 0 && k[1] == 0 && k[2] == 0);
        for (int a = 0; a < 3; ++a) P->kint.push_back(k[a]);
    }
    std::vector<float> kf(P->kint.begin(), P->kint.end());
    P->kvec.alloc(kf.size());
    P->kvec.upload(kf.data(), kf.size());
    // layers
    int in = 2 * P->nf;
    uint64_t off = 0;
    for (int l = 0; l <= P->depth; ++l) {
        const int out = l < P->depth ? P->width : 1;
        P->lin.push_back(in);
        P->lout.push_back(out);
        P->woff.push_back(off);
        off += (uint64_t)in * out;
        P->boff.push_back(off);
        off += out;
        in = out;
    }
    P->n_params = off;
    // initialisation: W ~ U(-1/sqrt(in), 1/sqrt(in)) (the output layer 0.1x
    // that, so the untrained density is close to uniform), b = 0 (Philox
    // stream 2 of the seed)
    std::vector<float> w(off, 0.f);
    call = 0;
    for (int l = 0; l <= P->depth; ++l) {
        const double a = (l < P->depth ? 1.0 : 0.1) / std::sqrt((double)P->lin[l]);
        for (uint64_t i = 0; i < (uint64_t)P->lin[l] * P->lout[l]; ++i)
            w[P->woff[l] + i] = (float)(a * (2.0 * philox_uniform(c.seed, 2, call++) - 1.0));
    }
    P->w.alloc(off);
    P->w.upload(w.data(), off);
    P->m.alloc(off);
    P->v.alloc(off);
    P->g.alloc(off);
    ALEA_CUDA(cudaMemset(P->m.p, 0, off * sizeof(float)));
    ALEA_CUDA(cudaMemset(P->v.p, 0, off * sizeof(float)));
    P->wb.alloc(off);
    to_bf16_kernel<<<blocks_for(off, 256), 256>>>(P->w.p, P->wb.p, off);
    ALEA_CUDA(cudaGetLastError());
    P->stats.alloc(5);
    ALEA_CUDA(cudaDeviceSynchronize());
    return P;
}

void proposal_destroy(ProposalImpl* P) { delete P; }
uint64_t proposal_param_count(const ProposalImpl* P) { return P->n_params; }
const std::vector<int32_t>& proposal_wave_vectors(const ProposalImpl* P) { return P->kint; }

void proposal_get_params(const ProposalImpl* P, float* out) {
    P->w.download(out, P->n_params);
}

void proposal_set_params(ProposalImpl* P, const float* in) {
    P->w.upload(in, P->n_params);
    to_bf16_kernel<<<blocks_for(P->n_params, 256), 256>>>(P->w.p, P->wb.p, P->n_params);
    ALEA_CUDA(cudaGetLastError());
    ALEA_CUDA(cudaDeviceSynchronize());
}

void proposal_forward_host(ProposalImpl* P, const float* s, uint64_t n, float* out) {
    if (n == 0) return;
    std::vector<float> rows(ROW * n, 0.f);
    for (uint64_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) rows[ROW * i + a] = s[3 * i + a];
    DevBuf<float> d(ROW * n);
    d.upload(rows.data(), rows.size());
    forward(*P, d.p, n, 0, 0, 0, 0);
    P->f.download(out, n);
    ALEA_CUDA(cudaDeviceSynchronize());
}

double proposal_loss_grad_host(ProposalImpl* P, const float* samples, uint64_t n, double tau,
                               float* grad) {
    require(n >= 1, ALEA_ERR_INVALID_ARGUMENT, "alea_proposal_loss_grad: no samples");
    DevBuf<float> d(ROW * n);
    d.upload(samples, ROW * n);
    const double loss = loss_grad(*P, d.p, n, 0, 0, 0, tau, 0);
    P->g.download(grad, P->n_params);
    ALEA_CUDA(cudaDeviceSynchronize());
    return loss;
}

// Minibatch Adam over a pool of samples in device memory; each epoch visits
// the pool through the affine permutation i -> (a i + c) mod pool with a
// coprime to pool (a and c drawn from Philox stream 3 of the seed).
double proposal_train(ProposalImpl* P, const float* samples_dev, uint64_t pool,
                      const alea_proposal_train_config& c, cudaStream_t s) {
    require(pool >= 2, ALEA_ERR_INVALID_ARGUMENT, "alea_proposal_train: need at least 2 samples");
    require(c.batch >= 2 && c.epochs >= 1, ALEA_ERR_INVALID_ARGUMENT,
            "alea_proposal_train: batch >= 2 and epochs >= 1 required");
    require(c.lr > 0 && c.beta1 >= 0 && c.beta1 < 1 && c.beta2 >= 0 && c.beta2 < 1 && c.eps > 0,
            ALEA_ERR_INVALID_ARGUMENT, "alea_proposal_train: invalid Adam parameters");
    const uint64_t batch = std::min<uint64_t>(c.batch, pool);
    const uint64_t steps = pool / batch;
    double loss = 0.0;
    uint64_t call = 0;
    for (uint32_t e = 0; e < c.epochs; ++e) {
        uint64_t a;
        do {
            a = 1 + (uint64_t)(philox_uniform(c.seed, 3, call++) * (double)(pool - 1));
        } while (std::gcd(a, pool) != 1);
        const uint64_t cc = (uint64_t)(philox_uniform(c.seed, 3, call++) * (double)pool);
        for (uint64_t st = 0; st < steps; ++st) {
            const uint64_t pc = (cc + a * (st * batch % pool)) % pool;
            const bool last = e + 1 == c.epochs && st + 1 == steps;
            loss = loss_grad(*P, samples_dev, batch, a, pc, pool, c.tau, s, last);
            ++P->adam_t;
            const float c1 = 1.f - std::pow((float)c.beta1, (float)P->adam_t);
            const float c2 = 1.f - std::pow((float)c.beta2, (float)P->adam_t);
            adam_kernel<<<blocks_for(P->n_params, 256), 256, 0, s>>>(
                P->w.p, P->g.p, P->m.p, P->v.p, P->wb.p, P->n_params, (float)c.lr, (float)c.beta1,
                (float)c.beta2, (float)c.eps, c1, c2);
            ALEA_CUDA(cudaGetLastError());
        }
    }
    ALEA_CUDA(cudaStreamSynchronize(s));
    return loss;
}

// The sampled proposal: P_c = (1 - u) softmax(f(centre_c)) + u / N over the
// cells^3 cells (x fastest), its CDF in FP64, and log(N P_c).
void proposal_tabulate(ProposalImpl* P, uint32_t cells, double uniform_share) {
    require(cells >= 1 && cells <= 256, ALEA_ERR_INVALID_ARGUMENT,
            "alea_proposal_tabulate: cells per axis must be 1..256");
    require(uniform_share > 0.0 && uniform_share <= 1.0, ALEA_ERR_INVALID_ARGUMENT,
            "alea_proposal_tabulate: uniform share must be in (0, 1]");
    const uint64_t N = (uint64_t)cells * cells * cells;
    std::vector<float> f(N);
    const uint64_t chunk = 1u << 16;
    DevBuf<float> centres(ROW * chunk);
    for (uint64_t c0 = 0; c0 < N; c0 += chunk) {
        const uint64_t n = std::min(chunk, N - c0);
        cell_centres_kernel<<<blocks_for(n, 256), 256>>>((int)cells, c0, n, centres.p);
        ALEA_CUDA(cudaGetLastError());
        forward(*P, centres.p, n, 0, 0, 0, 0);
        P->f.download(f.data() + c0, n);
    }
    ALEA_CUDA(cudaDeviceSynchronize());
    double mx = -INFINITY;
    for (float v : f) mx = std::max(mx, (double)v);
    double z = 0.0;
    for (float v : f) z += std::exp((double)v - mx);
    std::vector<double> cdf(N);
    P->logp_host.assign(N, 0.0);
    double acc = 0.0;
    for (uint64_t i = 0; i < N; ++i) {
        const double p = (1.0 - uniform_share) * std::exp((double)f[i] - mx) / z + uniform_share / (double)N;
        acc += p;
        cdf[i] = acc;
        P->logp_host[i] = std::log(p * (double)N);
    }
    // exact normalisation: p_i is divided by the final sum, so the last CDF
    // entry is 1 and the densities integrate to 1
    for (uint64_t i = 0; i < N; ++i) {
        cdf[i] /= acc;
        P->logp_host[i] -= std::log(acc);
    }
    cdf[N - 1] = 1.0;
    P->cells = (int)cells;
    P->uniform_share = uniform_share;
    P->cdf.alloc(N);
    P->cdf.upload(cdf.data(), N);
    P->logp.alloc(N);
    P->logp.upload(P->logp_host.data(), N);
}

ProposalTable proposal_table(const ProposalImpl* P) {
    require(P->cells > 0, ALEA_ERR_RUNTIME, "proposal: tabulate before sampling from it");
    return ProposalTable{P->cells, P->cdf.p, P->logp.p};
}

double proposal_log_density_host(const ProposalImpl* P, const double* s) {
    require(P->cells > 0, ALEA_ERR_RUNTIME, "proposal: tabulate before sampling from it");
    int idx[3];
    for (int a = 0; a < 3; ++a) {
        double f = s[a] - std::floor(s[a]);
        int i = (int)(f * P->cells);
        idx[a] = std::min(std::max(i, 0), P->cells - 1);
    }
    const uint64_t c = ((uint64_t)idx[2] * P->cells + idx[1]) * P->cells + idx[0];
    return P->logp_host[c];
}

}  // namespace alea
