// Photon generation on the device: point source through a CircleAperture.
//
// The arithmetic restates, per photon, the reference steps named in the
// header (RandomArbitraryPdf energies, uniform polarization angles,
// polarization_vectors, CircleAperture.generate_local_xy and its projected
// area factor), so that with the same uniforms the columns equal the
// reference's to rounding of the library sin/cos/sqrt.
#include <cuda_runtime.h>
#include "mgpu_device.cuh"
#include "mgpu_ff.cuh"

namespace {

constexpr int kThreads = 256;
// grid cap in blocks per SM (0: one block per 256 photons)
#ifndef MGPU_SOURCE_GRID_PER_SM
#define MGPU_SOURCE_GRID_PER_SM 8
#endif
constexpr int kGridPerSm = MGPU_SOURCE_GRID_PER_SM;
constexpr double kTwoPi = 6.283185307179586;
constexpr double kPi = 3.141592653589793;

__device__ __forceinline__ void uniforms(const mgpu_source& S, int64_t i, double* u) {
    if (S.rng == MGPU_RNG_PREDRAWN) {
#pragma unroll
        for (int k = 0; k < 5; ++k) u[k] = S.draws[(int64_t)k * S.n + i];
        return;
    }
    const uint64_t row = S.row_base + (uint64_t)i;
    philox_uniform2(S.seed, row, 0x5000u, 0u, &u[0], &u[1]);
    philox_uniform2(S.seed, row, 0x5001u, 0u, &u[2], &u[3]);
    double spare;
    philox_uniform2(S.seed, row, 0x5002u, 0u, &u[4], &spare);
}

__global__ void __launch_bounds__(kThreads)
generate_kernel(const __grid_constant__ mgpu_source S, mgpu_vec pos, mgpu_vec dir, mgpu_vec pol,
                mgpu_col energy, mgpu_col prob) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < S.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double u[5];
        uniforms(S, i, u);
        // energy: RandomArbitraryPdf.__call__ (random.py:79-95)
        double e = S.energy;
        if (S.n_bins > 0) {
            const int nb = S.n_bins;
            const double choice = S.e_cdf[nb - 1] * u[0];
            int lo = 0, hi = nb;                 // first i with cdf[i] >= choice (searchsorted left)
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (S.e_cdf[mid] < choice) lo = mid + 1;
                else hi = mid;
            }
            if (lo > nb - 1) lo = nb - 1;        // choice above cdf[last] cannot occur (u < 1)
            const int j = S.e_index[lo];
            const int jm = (j - 1 < 0) ? nb - 1 : j - 1;   // numpy x[-1]
            e = __dadd_rn(S.e_x[jm], __dmul_rn(S.e_width[j], u[1]));
        }
        // polarization angle and vector
        const double ang = S.pol_random ? __dmul_rn(kTwoPi, u[2]) : S.pol_angle;
        double sa, ca;
        sincos(ang, &sa, &ca);
        // position: CircleAperture.generate_local_xy
        const double phi = __dadd_rn(S.phi0, __dmul_rn(S.phi1 - S.phi0, u[3]));
        const double r = sqrt(__dadd_rn(S.r_inner2, __dmul_rn(1.0 - S.r_inner2, u[4])));
        double sp, cp;
        sincos(phi, &sp, &cp);
        const double x = __dmul_rn(r, cp), y = __dmul_rn(r, sp);
        d3 p{__dadd_rn(__dadd_rn(S.center[0], __dmul_rn(x, S.v_y[0])), __dmul_rn(y, S.v_z[0])),
             __dadd_rn(__dadd_rn(S.center[1], __dmul_rn(x, S.v_y[1])), __dmul_rn(y, S.v_z[1])),
             __dadd_rn(__dadd_rn(S.center[2], __dmul_rn(x, S.v_y[2])), __dmul_rn(y, S.v_z[2]))};
        d3 q{__dadd_rn(__dmul_rn(S.pol_v1[0], ca), __dmul_rn(S.pol_v2[0], sa)),
             __dadd_rn(__dmul_rn(S.pol_v1[1], ca), __dmul_rn(S.pol_v2[1], sa)),
             __dadd_rn(__dmul_rn(S.pol_v1[2], ca), __dmul_rn(S.pol_v2[2], sa))};
        store3(pos, i, p);
        store3(dir, i, arr3(S.dir));
        store3(pol, i, q);
        if (pos.stride == 4) pos.ptr[i * 4 + 3] = 1.0;        // homogeneous (N,4) columns
        if (dir.stride == 4) dir.ptr[i * 4 + 3] = 0.0;
        if (pol.stride == 4) pol.ptr[i * 4 + 3] = 0.0;
        energy.ptr[i * energy.stride] = e;
        prob.ptr[i * prob.stride] = S.prob;
    }
}

// Float32-local variant: the same distributions without float64 arithmetic
// on the FP64 pipe (which limits the float64 variant on this GPU).
__global__ void __launch_bounds__(kThreads)
generate_fast_kernel(const __grid_constant__ mgpu_source S, mgpu_vec pos, mgpu_vec dir,
                     mgpu_vec pol, mgpu_col energy, mgpu_col prob) {
    __shared__ float s_chi[3], s_clo[3], s_vy[3], s_vz[3], s_v1[3], s_v2[3];
    __shared__ float s_phi0, s_dphi, s_ri2, s_om, s_pc, s_ps;
    if (threadIdx.x == 0) {
        for (int k = 0; k < 3; ++k) {
            s_chi[k] = __double2float_rn(S.center[k]);
            s_clo[k] = __double2float_rn(S.center[k] - (double)s_chi[k]);
            s_vy[k] = __double2float_rn(S.v_y[k]);
            s_vz[k] = __double2float_rn(S.v_z[k]);
            s_v1[k] = __double2float_rn(S.pol_v1[k]);
            s_v2[k] = __double2float_rn(S.pol_v2[k]);
        }
        s_phi0 = __double2float_rn(S.phi0 / kPi);
        s_dphi = __double2float_rn((S.phi1 - S.phi0) / kPi);
        s_ri2 = __double2float_rn(S.r_inner2);
        s_om = __double2float_rn(1.0 - S.r_inner2);
        double sa, ca;
        sincos(S.pol_angle, &sa, &ca);
        s_pc = __double2float_rn(ca);
        s_ps = __double2float_rn(sa);
    }
    __syncthreads();
    const float k24 = 5.9604644775390625e-08f;   // 2^-24
    const d3 dd = arr3(S.dir);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < S.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t row = S.row_base + (uint64_t)i;
        const u4 w1 = philox4x32_10(u4{(uint32_t)row, (uint32_t)(row >> 32), 0x5003u, 0u},
                                    (uint32_t)S.seed, (uint32_t)(S.seed >> 32));
        const u4 w2 = philox4x32_10(u4{(uint32_t)row, (uint32_t)(row >> 32), 0x5004u, 0u},
                                    (uint32_t)S.seed, (uint32_t)(S.seed >> 32));
        const float u1 = (float)(w1.y >> 8) * k24, u2 = (float)(w1.z >> 8) * k24;
        const float u3 = (float)(w1.w >> 8) * k24, u4v = (float)(w2.x >> 8) * k24;
        double e = S.energy;
        if (S.n_bins > 0) {
            const uint64_t U = w1.x;
            int lo = 0, hi = S.n_bins;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (U >= S.e_thresh[mid]) lo = mid + 1;
                else hi = mid;
            }
            if (lo > S.n_bins - 1) lo = S.n_bins - 1;
            const int j = S.e_index[lo];
            const ff base{S.e_lo_ff[2 * j], S.e_lo_ff[2 * j + 1]};
            e = ff2d(ff_add(base, two_prod(S.e_width_f[j], u1)));
        }
        float ps = s_ps, pc = s_pc;
        if (S.pol_random) sincospif(2.0f * u2, &ps, &pc);
        float sp, cp;
        sincospif(s_phi0 + s_dphi * u3, &sp, &cp);
        const float r = sqrtf(s_ri2 + s_om * u4v);
        const float x = r * cp, y = r * sp;
        double pd[3], qd[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float off = fmaf(x, s_vy[k], y * s_vz[k]);
            pd[k] = ff2d(ff_add_f(ff{s_chi[k], s_clo[k]}, off));
            qd[k] = f2d_bits(fmaf(s_v1[k], pc, s_v2[k] * ps));
        }
        store3(pos, i, d3{pd[0], pd[1], pd[2]});
        store3(dir, i, dd);
        store3(pol, i, d3{qd[0], qd[1], qd[2]});
        if (pos.stride == 4) pos.ptr[i * 4 + 3] = 1.0;
        if (dir.stride == 4) dir.ptr[i * 4 + 3] = 0.0;
        if (pol.stride == 4) pol.ptr[i * 4 + 3] = 0.0;
        energy.ptr[i * energy.stride] = e;
        prob.ptr[i * prob.stride] = S.prob;
    }
}

}  // namespace

extern "C" int mgpu_generate_photons(const mgpu_source* src, mgpu_vec pos, mgpu_vec dir,
                                     mgpu_vec pol, mgpu_col energy, mgpu_col prob,
                                     void* stream) {
    if (src == nullptr || src->n < 0) return (int)cudaErrorInvalidValue;
    const mgpu_source& S = *src;
    if (S.n == 0) return 0;
    if (!pos.ptr || !dir.ptr || !pol.ptr || !energy.ptr || !prob.ptr)
        return (int)cudaErrorInvalidValue;
    if (S.rng != MGPU_RNG_PHILOX && S.rng != MGPU_RNG_PREDRAWN) return (int)cudaErrorInvalidValue;
    if (S.rng == MGPU_RNG_PREDRAWN && S.draws == nullptr) return (int)cudaErrorInvalidValue;
    if (S.precision != MGPU_FP64 && S.precision != MGPU_FP32LOCAL) return (int)cudaErrorInvalidValue;
    if (S.precision == MGPU_FP32LOCAL) {
        if (S.rng != MGPU_RNG_PHILOX) return (int)cudaErrorInvalidValue;
        if (S.n_bins < 0 || (S.n_bins > 0 && (!S.e_lo_ff || !S.e_width_f || !S.e_thresh ||
                                               !S.e_index)))
            return (int)cudaErrorInvalidValue;
    } else if (S.n_bins < 0 || (S.n_bins > 0 && (!S.e_x || !S.e_width || !S.e_cdf || !S.e_index))) {
        return (int)cudaErrorInvalidValue;
    }
    int dev = 0, sms = 0;
    cudaError_t e;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return (int)e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return (int)e;
    int64_t blocks = (S.n + kThreads - 1) / kThreads;
    if (kGridPerSm > 0) {
        const int64_t cap = (int64_t)sms * kGridPerSm;
        if (blocks > cap) blocks = cap;
    }
    if (blocks > (1 << 30)) blocks = 1 << 30;   // grid-stride beyond
    if (S.precision == MGPU_FP32LOCAL)
        generate_fast_kernel<<<(unsigned)blocks, kThreads, 0, (cudaStream_t)stream>>>(
            S, pos, dir, pol, energy, prob);
    else
        generate_kernel<<<(unsigned)blocks, kThreads, 0, (cudaStream_t)stream>>>(S, pos, dir, pol,
                                                                                 energy, prob);
    return (int)cudaGetLastError();
}
