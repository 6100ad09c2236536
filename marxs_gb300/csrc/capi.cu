// C ABI entry points (declared in include/marxs_gb300.h) and the unit
// kernels behind mgpu_plane_intersect / mgpu_cylinder_intersect /
// mgpu_parallel_transport.
#include <cuda_runtime.h>
#include "mgpu_device.cuh"

cudaError_t mgpu_launch_chain_fp64(const mgpu_chain& chain, const mgpu_photons& io,
                                   cudaStream_t stream, int sm_count);
cudaError_t mgpu_launch_chain_fp32local(const mgpu_chain& chain, const mgpu_photons& io,
                                        cudaStream_t stream, int sm_count);
cudaError_t mgpu_launch_grid_build(const mgpu_facet* facets, int n_facets, const mgpu_grid& g,
                                   int* counts, uint32_t* status, cudaStream_t stream);

namespace {

int sm_count_cached() {
    static int count = 0;
    if (count == 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) return 152;
        if (cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            count = 152;
    }
    return count;
}


__global__ void plane_intersect_kernel(const __grid_constant__ mgpu_stage fr, int64_t n,
                                       mgpu_vec pos, mgpu_vec dir, uint8_t* hit, mgpu_vec ip,
                                       mgpu_col l0, mgpu_col l1) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double* f = fr.frame;
        PlaneHit h = plane_intersect(arr3(f), arr3(f + 3), arr3(f + 6), arr3(f + 9), f[12], f[13],
                                     load3(pos, i), load3(dir, i));
        if (hit) hit[i] = h.hit ? 1 : 0;
        if (h.hit) {
            if (ip.ptr) store3(ip, i, h.ip);
            store_col(l0, i, h.ly);
            store_col(l1, i, h.lz);
        } else {
            if (ip.ptr) store3(ip, i, d3{kNaN, kNaN, kNaN});
            store_col(l0, i, kNaN);
            store_col(l1, i, kNaN);
        }
    }
}

__global__ void cylinder_intersect_kernel(const __grid_constant__ mgpu_stage fr, int64_t n,
                                          mgpu_vec pos, mgpu_vec dir, uint8_t* hit, mgpu_vec ip,
                                          mgpu_col l0, mgpu_col l1) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        CylHit h = cylinder_intersect_dev(fr.cyl, load3(pos, i), load3(dir, i));
        if (hit) hit[i] = h.hit ? 1 : 0;
        if (h.hit) {
            if (ip.ptr) store3(ip, i, h.ip);
            store_col(l0, i, h.phi);
            store_col(l1, i, h.zl);
        } else {
            if (ip.ptr) store3(ip, i, d3{kNaN, kNaN, kNaN});
            store_col(l0, i, kNaN);
            store_col(l1, i, kNaN);
        }
    }
}

__global__ void transport_kernel(int64_t n, mgpu_vec d0, mgpu_vec d1, mgpu_vec pol, mgpu_vec out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        store3(out, i, parallel_transport_dev(load3(d0, i), load3(d1, i), load3(pol, i)));
}

unsigned grid_for(int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    int64_t cap = (int64_t)sm_count_cached() * 16;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (unsigned)b;
}

}  // namespace

extern "C" {

int mgpu_abi_version(void) { return MGPU_ABI_VERSION; }

int mgpu_device_sm_count(void) { return sm_count_cached(); }

int mgpu_trace(const mgpu_chain* chain, const mgpu_photons* photons, void* stream) {
    if (chain == nullptr || photons == nullptr) return (int)cudaErrorInvalidValue;
    if (chain->n_stages < 0 || chain->n_stages > MGPU_MAX_STAGES) return (int)cudaErrorInvalidValue;
    if (chain->precision != MGPU_FP64 && chain->precision != MGPU_FP32LOCAL)
        return (int)cudaErrorInvalidValue;
    if (chain->rng != MGPU_RNG_PREDRAWN && chain->rng != MGPU_RNG_PHILOX)
        return (int)cudaErrorInvalidValue;
    if (photons->n < 0) return (int)cudaErrorInvalidValue;
    cudaStream_t s = (cudaStream_t)stream;
    const mgpu_chain* c = chain;
    mgpu_chain scan;
    if (chain->flags & MGPU_FLAG_NO_GRID) {
        // no candidate grids: every facet stage scans all its facets
        scan = *chain;
        for (int k = 0; k < scan.n_stages; ++k) scan.stages[k].grid.cell_start = nullptr;
        c = &scan;
    }
    cudaError_t e;
    if (c->precision == MGPU_FP32LOCAL)
        e = mgpu_launch_chain_fp32local(*c, *photons, s, sm_count_cached());
    else
        e = mgpu_launch_chain_fp64(*c, *photons, s, sm_count_cached());
    return (int)e;
}

int mgpu_facet_grid_build(const mgpu_facet* facets, int32_t n_facets, mgpu_grid* grid,
                          int32_t* counts, uint32_t* status, void* stream) {
    if (grid == nullptr || counts == nullptr || status == nullptr) return (int)cudaErrorInvalidValue;
    if (n_facets < 0 || (n_facets > 0 && facets == nullptr)) return (int)cudaErrorInvalidValue;
    if (grid->nu <= 0 || grid->nv <= 0 || grid->cell_start == nullptr || grid->cell_items == nullptr)
        return (int)cudaErrorInvalidValue;
    return (int)mgpu_launch_grid_build(facets, n_facets, *grid, counts, status, (cudaStream_t)stream);
}

int mgpu_plane_intersect(const double* frame14, int64_t n, mgpu_vec pos, mgpu_vec dir,
                         uint8_t* hit, mgpu_vec interpos, mgpu_col loc0, mgpu_col loc1,
                         void* stream) {
    if (frame14 == nullptr || n < 0) return (int)cudaErrorInvalidValue;
    if (n == 0) return 0;
    mgpu_stage fr = {};
    for (int k = 0; k < 14; ++k) fr.frame[k] = frame14[k];
    plane_intersect_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
        fr, n, pos, dir, hit, interpos, loc0, loc1);
    return (int)cudaGetLastError();
}

int mgpu_cylinder_intersect(const double* cyl32, int64_t n, mgpu_vec pos, mgpu_vec dir,
                            uint8_t* hit, mgpu_vec interpos, mgpu_col loc0, mgpu_col loc1,
                            void* stream) {
    if (cyl32 == nullptr || n < 0) return (int)cudaErrorInvalidValue;
    if (n == 0) return 0;
    mgpu_stage fr = {};
    for (int k = 0; k < 32; ++k) fr.cyl[k] = cyl32[k];
    cylinder_intersect_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
        fr, n, pos, dir, hit, interpos, loc0, loc1);
    return (int)cudaGetLastError();
}

int mgpu_parallel_transport(int64_t n, mgpu_vec dir_old, mgpu_vec dir_new, mgpu_vec pol,
                            mgpu_vec pol_out, void* stream) {
    if (n < 0) return (int)cudaErrorInvalidValue;
    if (n == 0) return 0;
    transport_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, dir_old, dir_new, pol,
                                                                        pol_out);
    return (int)cudaGetLastError();
}

}  // extern "C"
