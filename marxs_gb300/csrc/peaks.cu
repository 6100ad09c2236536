// FMA-chain throughput probe: the measured FP32 / FP64 FMA peaks that the
// intersect stage's pipe utilisation is reported against.  Each thread runs
// kChains independent dependent chains of fused multiply-adds; the chains
// are independent, so the pipe, not the FMA latency, bounds the rate.
#include <cuda_runtime.h>
#include "mgpu_device.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kChains = 8;

template <typename T>
__global__ void __launch_bounds__(kThreads) fma_chain_kernel(int iters, T b, T c, T* out) {
    T acc[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) acc[k] = (T)(threadIdx.x + k) * (T)1e-3;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) acc[k] = fma(acc[k], b, c);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += acc[k];
    out[(int64_t)blockIdx.x * kThreads + threadIdx.x] = s;
}

}  // namespace

extern "C" int mgpu_fma_probe(int32_t precision, int32_t blocks, int32_t iters, void* out,
                              void* stream) {
    if (blocks <= 0 || iters <= 0 || out == nullptr) return (int)cudaErrorInvalidValue;
    cudaStream_t s = (cudaStream_t)stream;
    if (precision == MGPU_FP64)
        fma_chain_kernel<double><<<blocks, kThreads, 0, s>>>(iters, 0.999999, 1e-7, (double*)out);
    else if (precision == MGPU_FP32LOCAL)
        fma_chain_kernel<float><<<blocks, kThreads, 0, s>>>(iters, 0.999999f, 1e-7f, (float*)out);
    else
        return (int)cudaErrorInvalidValue;
    return (int)cudaGetLastError();
}

namespace {

__global__ void __launch_bounds__(kThreads)
philox_probe_kernel(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    const uint32_t* a = in + 6 * i;
    const u4 r = philox4x32_10(u4{a[0], a[1], a[2], a[3]}, a[4], a[5]);
    uint32_t* o = out + 4 * i;
    o[0] = r.x;
    o[1] = r.y;
    o[2] = r.z;
    o[3] = r.w;
}

}  // namespace

// the device Philox4x32-10 on caller-given counters and keys (test access)
extern "C" int mgpu_philox4x32_10(const uint32_t* in, uint32_t* out, int64_t n, void* stream) {
    if (n < 0 || (n > 0 && (in == nullptr || out == nullptr))) return (int)cudaErrorInvalidValue;
    if (n == 0) return 0;
    const int64_t blocks = (n + kThreads - 1) / kThreads;
    if (blocks > (1 << 30)) return (int)cudaErrorInvalidValue;
    philox_probe_kernel<<<(unsigned)blocks, kThreads, 0, (cudaStream_t)stream>>>(in, out, n);
    return (int)cudaGetLastError();
}
