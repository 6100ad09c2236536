// Facet poses of one Parallel recomputed on the device (tolerancing).
//
// Parallel.generate_elements (marxs/simulator/simulator.py:384-440) poses
// element i as
//   pos4d_i = G U T(t_i) T(c_i) R(a_i) M_i
// with G the Parallel's pos4d, U its global uncertainty, (t_i, a_i) the
// element uncertainty (a translation and an Euler sxyz rotation, as
// generate_facet_uncertainty builds it, design/uncertainties.py:8-39), c_i
// the element centre plus the common offset and M_i the element rotation,
// common rotation and zooms.  The caller passes O = G U and the
// uncertainty-free local poses (c_i, M_i); this kernel draws or takes
// (t_i, a_i), composes the pose and rewrites the facet's frame in the
// float64 table and the FP32-local table,
// exactly as the host lowering derives them from pos4d (frame of
// Geometry.__getitem__, math/geometry.py:108-160; groove frame of
// FlatGrating.e_groove_coos, optics/grating.py:186-207).  The candidate
// grid is rebuilt afterwards by mgpu_facet_grid_build.
#include <cuda_runtime.h>
#include "mgpu_device.cuh"

namespace {

constexpr int kThreads = 128;

// euler2mat(ax, ay, az, 'sxyz') = Rz(az) Ry(ay) Rx(ax), row-major
__device__ void euler_sxyz(double ax, double ay, double az, double* R) {
    double sx, cx, sy, cy, sz, cz;
    sincos(ax, &sx, &cx);
    sincos(ay, &sy, &cy);
    sincos(az, &sz, &cz);
    R[0] = cz * cy;
    R[1] = cz * sy * sx - sz * cx;
    R[2] = cz * sy * cx + sz * sx;
    R[3] = sz * cy;
    R[4] = sz * sy * sx + cz * cx;
    R[5] = sz * sy * cx - cz * sx;
    R[6] = -sy;
    R[7] = cy * sx;
    R[8] = cy * cx;
}

__device__ __forceinline__ void mat3_mul(const double* A, const double* B, double* C) {
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            C[3 * r + c] = A[3 * r] * B[c] + A[3 * r + 1] * B[3 + c] + A[3 * r + 2] * B[6 + c];
}

__device__ __forceinline__ void split_ff(double x, float& hi, float& lo) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(x - (double)hi);
}

__global__ void __launch_bounds__(kThreads)
pose_kernel(const __grid_constant__ mgpu_pose_update P) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n_facets) return;
    double q[6] = {0, 0, 0, 0, 0, 0};
    if (P.mode == MGPU_POSE_DRAW) {
        // numpy.random.normal(loc, scale): loc + scale * z
        philox_normal2(P.seed, (uint64_t)i, 0x6000u, 0u, &q[0], &q[1]);
        philox_normal2(P.seed, (uint64_t)i, 0x6001u, 0u, &q[2], &q[3]);
        philox_normal2(P.seed, (uint64_t)i, 0x6002u, 0u, &q[4], &q[5]);
        for (int k = 0; k < 6; ++k) q[k] = P.offset[k] + P.sigma[k] * q[k];
    } else if (P.mode == MGPU_POSE_GIVEN) {
        for (int k = 0; k < 6; ++k) q[k] = P.given[6 * (int64_t)i + k];
    }
    if (P.perturb_out)
        for (int k = 0; k < 6; ++k) P.perturb_out[6 * (int64_t)i + k] = q[k];
    const double* loc = P.local + 12 * (int64_t)i;   // c (3), M (3x3 row-major)
    double R[9], RM[9], L[9], Olin[9];
    euler_sxyz(q[3], q[4], q[5], R);
    mat3_mul(R, loc + 3, RM);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) Olin[3 * r + c] = P.outer[4 * r + c];
    mat3_mul(Olin, RM, L);
    const d3 tc{q[0] + loc[0], q[1] + loc[1], q[2] + loc[2]};
    d3 cen;
    cen.x = Olin[0] * tc.x + Olin[1] * tc.y + Olin[2] * tc.z + P.outer[3];
    cen.y = Olin[3] * tc.x + Olin[4] * tc.y + Olin[5] * tc.z + P.outer[7];
    cen.z = Olin[6] * tc.x + Olin[7] * tc.y + Olin[8] * tc.z + P.outer[11];
    const d3 vx{L[0], L[3], L[6]}, vy{L[1], L[4], L[7]}, vz{L[2], L[5], L[8]};
    const double nx = sqrt(dot3(vx, vx)), ny = sqrt(dot3(vy, vy)), nz = sqrt(dot3(vz, vz));
    const d3 ex{vx.x / nx, vx.y / nx, vx.z / nx};
    const d3 ey{vy.x / ny, vy.y / ny, vy.z / ny};
    const d3 ez{vz.x / nz, vz.y / nz, vz.z / nz};
    const double sn = P.groove[2 * (int64_t)i], cs = P.groove[2 * (int64_t)i + 1];
    const d3 l{sn * ey.x + cs * ez.x, sn * ey.y + cs * ez.y, sn * ey.z + cs * ez.z};
    const d3 dneg{-(cs * ey.x - sn * ez.x), -(cs * ey.y - sn * ez.y), -(cs * ey.z - sn * ez.z)};
    mgpu_facet& f = P.facets[i];
    f.c[0] = cen.x; f.c[1] = cen.y; f.c[2] = cen.z;
    f.ex[0] = ex.x; f.ex[1] = ex.y; f.ex[2] = ex.z;
    f.ey[0] = ey.x; f.ey[1] = ey.y; f.ey[2] = ey.z;
    f.ez[0] = ez.x; f.ez[1] = ez.y; f.ez[2] = ez.z;
    f.hy = ny;
    f.hz = nz;
    f.l[0] = l.x; f.l[1] = l.y; f.l[2] = l.z;
    f.dneg[0] = dneg.x; f.dneg[1] = dneg.y; f.dneg[2] = dneg.z;
    if (P.facets32) {
        mgpu_facet32& g = P.facets32[i];
        const double cv[3] = {cen.x, cen.y, cen.z};
        for (int k = 0; k < 3; ++k) split_ff(cv[k], g.c_hi[k], g.c_lo[k]);
        const double* src[5] = {f.ex, f.ey, f.ez, f.l, f.dneg};
        float* dst[5] = {g.ex, g.ey, g.ez, g.l, g.dneg};
        for (int v = 0; v < 5; ++v)
            for (int k = 0; k < 3; ++k) dst[v][k] = __double2float_rn(src[v][k]);
        g.hy = __double2float_rn(ny);
        g.hz = __double2float_rn(nz);
    }
}

}  // namespace

extern "C" int mgpu_facet_poses(const mgpu_pose_update* p, void* stream) {
    if (p == nullptr || p->n_facets < 0) return (int)cudaErrorInvalidValue;
    if (p->n_facets == 0) return 0;
    if (!p->local || !p->groove || !p->facets) return (int)cudaErrorInvalidValue;
    if (p->mode != MGPU_POSE_ZERO && p->mode != MGPU_POSE_DRAW && p->mode != MGPU_POSE_GIVEN)
        return (int)cudaErrorInvalidValue;
    if (p->mode == MGPU_POSE_GIVEN && !p->given) return (int)cudaErrorInvalidValue;
    if (p->facets32 && ((uintptr_t)p->facets32 & 15u) != 0) return (int)cudaErrorInvalidValue;
    const int blocks = (p->n_facets + kThreads - 1) / kThreads;
    pose_kernel<<<blocks, kThreads, 0, (cudaStream_t)stream>>>(*p);
    return (int)cudaGetLastError();
}
