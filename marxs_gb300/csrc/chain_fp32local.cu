// Fused element-chain kernel, FP32-local precision mode (placeholder until
// the mixed-precision kernel lands: the launch reports "not supported").
#include <cuda_runtime.h>
#include "mgpu_device.cuh"

cudaError_t mgpu_launch_chain_fp32local(const mgpu_chain& chain, const mgpu_photons& io,
                                        cudaStream_t stream, int sm_count) {
    (void)chain; (void)io; (void)stream; (void)sm_count;
    return cudaErrorNotSupported;
}
