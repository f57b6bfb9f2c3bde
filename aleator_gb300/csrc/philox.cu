// Philox4x32-10 streams on the device, bit-exact to the reference's
// Philox4x32Rng (core/math/counter_based_rng.cc:42-79): each thread computes
// the draw at its own call index, so a stream is filled in one pass.
#include "common.cuh"
#include "grid.cuh"

namespace alea {

namespace {

__global__ void philox_raw_kernel(const uint4* __restrict__ ctr, const uint2* __restrict__ key,
                                  uint4* __restrict__ out, uint64_t n) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint4 c = ctr[i];
    const uint2 k = key[i];
    const U32x4 o = philox4x32_10(c.x, c.y, c.z, c.w, k.x, k.y);
    out[i] = make_uint4(o.v[0], o.v[1], o.v[2], o.v[3]);
}

__global__ void philox_u64_kernel(uint64_t seed, uint64_t stream, uint64_t first, uint64_t n,
                                  uint64_t* __restrict__ out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = philox_u64(seed, stream, first + i);
}

__global__ void philox_uniform_kernel(uint64_t seed, uint64_t stream, uint64_t first, uint64_t n,
                                      double* __restrict__ out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = philox_uniform(seed, stream, first + i);
}

unsigned fill_blocks(uint64_t n) {
    int sms = 152;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess)
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t want = (n + 255) / 256;
    const uint64_t cap = (uint64_t)sms * 8;
    return (unsigned)(want < cap ? (want ? want : 1) : cap);
}

}  // namespace

void philox_raw(const uint32_t* ctr, const uint32_t* key, uint32_t* out, uint64_t n) {
    require_device();
    if (n == 0) return;
    DevBuf<uint4> dc(n);
    DevBuf<uint2> dk(n);
    DevBuf<uint4> dout(n);
    ALEA_CUDA(cudaMemcpy(dc.p, ctr, n * 16, cudaMemcpyHostToDevice));
    ALEA_CUDA(cudaMemcpy(dk.p, key, n * 8, cudaMemcpyHostToDevice));
    philox_raw_kernel<<<(unsigned)((n + 255) / 256), 256>>>(dc.p, dk.p, dout.p, n);
    ALEA_CUDA(cudaGetLastError());
    ALEA_CUDA(cudaMemcpy(out, dout.p, n * 16, cudaMemcpyDeviceToHost));
}

void philox_fill_u64_device(uint64_t seed, uint64_t stream, uint64_t first, uint64_t n,
                            uint64_t* out, cudaStream_t s) {
    if (n == 0) return;
    philox_u64_kernel<<<fill_blocks(n), 256, 0, s>>>(seed, stream, first, n, out);
    ALEA_CUDA(cudaGetLastError());
}

void philox_fill_uniform_device(uint64_t seed, uint64_t stream, uint64_t first, uint64_t n,
                                double* out, cudaStream_t s) {
    if (n == 0) return;
    philox_uniform_kernel<<<fill_blocks(n), 256, 0, s>>>(seed, stream, first, n, out);
    ALEA_CUDA(cudaGetLastError());
}

}  // namespace alea
