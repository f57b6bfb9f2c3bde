// Measurement helpers: sustained FP32 FMA throughput of this device, scalar
// (fmaf) and packed two-lane (fma.rn.f32x2), the roofline denominators for the
// FP32 pair kernels (the measured peaks file carries HBM and tensor-core
// figures only). Eight independent FMA chains per thread, every SM busy, timed
// with CUDA events; the best of five launches.
#include "common.cuh"
#include "ff.cuh"

namespace alea {
namespace {
__global__ void ffma_kernel(float* out, int iters, float a, float b) {
    float x[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = threadIdx.x * 1e-3f + i;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) x[i] = fmaf(x[i], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += x[i];
    if (s == 1234.5f) out[0] = s;  // keeps the chains live
}

// The same with the packed two-lane FMA (fma.rn.f32x2, sm_100 family), the
// instruction the FP32 grid sweep issues: 8 independent packed chains.
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b,
                                                   unsigned long long c) {
    unsigned long long d;
    asm volatile("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

__device__ __forceinline__ unsigned long long pack2(float lo, float hi) {
    return (unsigned long long)__float_as_uint(lo) | ((unsigned long long)__float_as_uint(hi) << 32);
}

__global__ void ffma2_kernel(float* out, int iters, float a, float b) {
    unsigned long long x[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = pack2(threadIdx.x * 1e-3f + i, threadIdx.x * 2e-3f - i);
    const unsigned long long a2 = pack2(a, a), b2 = pack2(b, b);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) x[i] = fma2(x[i], a2, b2);
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i)
        s += __uint_as_float((unsigned)x[i]) + __uint_as_float((unsigned)(x[i] >> 32));
    if (s == 1234.5f) out[0] = s;  // keeps the chains live
}

template <typename K>
double time_fma(K kernel, double flops_per_thread_iter) {
    int dev = 0, sms = 0;
    ALEA_CUDA(cudaGetDevice(&dev));
    ALEA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DevBuf<float> o(1);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    kernel<<<blocks, threads>>>(o.p, 64, 0.999f, 1e-3f);  // warm-up
    ALEA_CUDA(cudaGetLastError());
    cudaEvent_t e0, e1;
    ALEA_CUDA(cudaEventCreate(&e0));
    ALEA_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        ALEA_CUDA(cudaEventRecord(e0));
        kernel<<<blocks, threads>>>(o.p, iters, 0.999f, 1e-3f);
        ALEA_CUDA(cudaEventRecord(e1));
        ALEA_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        ALEA_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        best = ms < best ? ms : best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double flops = flops_per_thread_iter * iters * (double)blocks * threads;
    return flops / (best * 1e-3) / 1e12;
}
// Test support: the FP32 forms' double-float near-pair arithmetic, element by
// element. mode 0: erfc(x) (ff_erfc, x within its series); mode 1: q erfc(alpha
// r) / r of displacement (a, b, c) and charge q (near_coulomb_ff; NaN where it
// defers to FP64).
__global__ void ff_check_kernel(int mode, const double* in, double* out, uint64_t n, double alpha) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (mode == 0) {
        const ff r = ff_erfc(ff_from(in[i]));
        out[i] = (double)r.hi + (double)r.lo;
    } else {
        double v;
        const double* d = in + 4 * i;
        out[i] = near_coulomb_ff(ff_from(d[0]), ff_from(d[1]), ff_from(d[2]), ff_from(d[3]),
                                 ff_from(alpha), v) ? v : __longlong_as_double(0x7ff8000000000000ll);
    }
}
}  // namespace
}  // namespace alea

extern "C" alea_status alea_test_ff_near(int32_t mode, const double* in, double* out, uint64_t n,
                                         double alpha) {
    try {
        alea::require_device();
        alea::require(mode == 0 || mode == 1, ALEA_ERR_INVALID_ARGUMENT, "mode must be 0 or 1");
        if (n == 0) return ALEA_OK;
        const uint64_t w = mode == 0 ? 1 : 4;
        alea::DevBuf<double> din(n * w), dout(n);
        din.upload(in, n * w);
        alea::ff_check_kernel<<<(unsigned)((n + 255) / 256), 256>>>(mode, din.p, dout.p, n, alpha);
        ALEA_CUDA(cudaGetLastError());
        ALEA_CUDA(cudaMemcpy(out, dout.p, n * sizeof(double), cudaMemcpyDeviceToHost));
        return ALEA_OK;
    } catch (const alea::Error& e) {
        return e.status;
    }
}

extern "C" alea_status alea_probe_fp32x2_fma_tflops(double* out) {
    try {
        alea::require_device();
        *out = alea::time_fma(alea::ffma2_kernel, 2.0 * 2.0 * 8.0);
        return ALEA_OK;
    } catch (const alea::Error& e) {
        return e.status;
    }
}

extern "C" alea_status alea_probe_fp32_fma_tflops(double* out) {
    try {
        alea::require_device();
        *out = alea::time_fma(alea::ffma_kernel, 2.0 * 8.0);
        return ALEA_OK;
    } catch (const alea::Error& e) {
        return e.status;
    }
}
