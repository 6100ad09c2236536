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
