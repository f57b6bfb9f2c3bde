// Measurement helper: sustained FP32 FFMA throughput of this device, the
// roofline denominator for the FP32 pair kernels (the measured peaks file
// carries HBM and tensor-core figures only). Eight independent FMA chains per
// thread, every SM busy, timed with CUDA events.
#include "common.cuh"

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
}  // namespace
}  // namespace alea

extern "C" alea_status alea_probe_fp32_fma_tflops(double* out) {
    try {
        alea::require_device();
        int dev = 0, sms = 0;
        ALEA_CUDA(cudaGetDevice(&dev));
        ALEA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        alea::DevBuf<float> o(1);
        const int blocks = sms * 8, threads = 256, iters = 4096;
        alea::ffma_kernel<<<blocks, threads>>>(o.p, 64, 0.999f, 1e-3f);  // warm-up
        cudaEvent_t e0, e1;
        ALEA_CUDA(cudaEventCreate(&e0));
        ALEA_CUDA(cudaEventCreate(&e1));
        float best = 1e30f;
        for (int rep = 0; rep < 5; ++rep) {
            ALEA_CUDA(cudaEventRecord(e0));
            alea::ffma_kernel<<<blocks, threads>>>(o.p, iters, 0.999f, 1e-3f);
            ALEA_CUDA(cudaEventRecord(e1));
            ALEA_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            ALEA_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            best = ms < best ? ms : best;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
        *out = flops / (best * 1e-3) / 1e12;
        return ALEA_OK;
    } catch (const alea::Error& e) {
        return e.status;
    }
}
