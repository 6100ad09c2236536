// Pose adjoint: detector moments of frozen photons and their reverse mode
// (float64, sm_103a).
//
// Forward of one photon, stage by stage (each restates the reference formula
// with the photon's discrete choices frozen):
//   lens     PerfectLens, optics/mirror.py:53-82: plane crossing, then towards
//            centre - d_center_optical_axis e_z + f norm(dir)
//   scatter  RadialMirrorScatter, optics/scatter.py:49-77: R^T v about
//            dir x radial (angle alpha), then about radial (angle beta),
//            axangle2mat of math/rotations.py:50-87
//   grating  FlatGrating.diffract_photons, optics/grating.py:233-266 on the
//            photon's facet: p_d = p.d + sign m lambda / d,
//            p_n = sqrt(1 - p_d^2 - p_l^2), dir = p_d d + p_l l + nsign p_n n
//   detector FinitePlane.intersect (math/geometry.py:233-252) local (y, z), or
//            Cylinder.intersect (math/geometry.py:470-564) (phi R, z zoom_z)
// A stage's output ray (position, direction) is the checkpoint the reverse
// sweep starts that stage from: BACKWARD runs the forward keeping the stage
// outputs, then each stage's reverse step recomputes the stage's internals
// from its input ray and returns the adjoint of that input.
#include <cuda_runtime.h>
#include "mgpu_device.cuh"

namespace {

constexpr int kThreads = 256;
constexpr double kEnergy2Wave = 1.2398419292004202e-06;   // marxs/__init__.py:14

struct Ray {
    d3 p, d;
};

__device__ __forceinline__ d3 ld_soa(const double* a, int64_t i, int64_t n) {
    return d3{__ldg(a + i), __ldg(a + n + i), __ldg(a + 2 * n + i)};
}
__device__ __forceinline__ d3 mat_vec(const double* M, d3 v) {   // row-major 3x3
    return d3{M[0] * v.x + M[1] * v.y + M[2] * v.z, M[3] * v.x + M[4] * v.y + M[5] * v.z,
              M[6] * v.x + M[7] * v.y + M[8] * v.z};
}
__device__ __forceinline__ d3 mat_tvec(const double* M, d3 v) {  // M^T v
    return d3{M[0] * v.x + M[3] * v.y + M[6] * v.z, M[1] * v.x + M[4] * v.y + M[7] * v.z,
              M[2] * v.x + M[5] * v.y + M[8] * v.z};
}

// R = Rz(a2) Ry(a1) Rx(a0) and dR/da0, dR/da1, dR/da2 (4 x 9 doubles)
__global__ void pose_prep_kernel(const double* __restrict__ theta, int n_facets, double* rot) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j > n_facets) return;
    const double* a = theta + 1 + 6 * j + 3;
    double s0, c0, s1, c1, s2, c2;
    sincos(a[0], &s0, &c0);
    sincos(a[1], &s1, &c1);
    sincos(a[2], &s2, &c2);
    const double Rx[9] = {1, 0, 0, 0, c0, -s0, 0, s0, c0};
    const double dRx[9] = {0, 0, 0, 0, -s0, -c0, 0, c0, -s0};
    const double Ry[9] = {c1, 0, s1, 0, 1, 0, -s1, 0, c1};
    const double dRy[9] = {-s1, 0, c1, 0, 0, 0, -c1, 0, -s1};
    const double Rz[9] = {c2, -s2, 0, s2, c2, 0, 0, 0, 1};
    const double dRz[9] = {-s2, -c2, 0, c2, -s2, 0, 0, 0, 0};
    auto mul = [](const double* A, const double* B, double* C) {
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c)
                C[3 * r + c] = A[3 * r] * B[c] + A[3 * r + 1] * B[3 + c] + A[3 * r + 2] * B[6 + c];
    };
    double* out = rot + 36 * (size_t)j;
    double T[9], U[9];
    mul(Rz, Ry, T);
    mul(T, Rx, out);
    mul(T, dRx, out + 9);
    mul(Rz, dRy, U);
    mul(U, Rx, out + 18);
    mul(dRz, Ry, U);
    mul(U, Rx, out + 27);
}

// R^T v for R = axangle2mat(k, angle), k a unit vector
__device__ __forceinline__ d3 rot_t(d3 k, double c, double s, d3 v) {
    d3 kv = cross3(k, v);
    double kd = (1.0 - c) * dot3(k, v);
    return d3{c * v.x - s * kv.x + kd * k.x, c * v.y - s * kv.y + kd * k.y,
              c * v.z - s * kv.z + kd * k.z};
}
// adjoint of v in y = R^T(k, angle) v
__device__ __forceinline__ d3 rot_t_adj_v(d3 k, double c, double s, d3 yb) {
    d3 ky = cross3(k, yb);
    double kd = (1.0 - c) * dot3(k, yb);
    return d3{c * yb.x + s * ky.x + kd * k.x, c * yb.y + s * ky.y + kd * k.y,
              c * yb.z + s * ky.z + kd * k.z};
}
// adjoint of a unit vector k = u / |u| -> adjoint of u
__device__ __forceinline__ d3 normalize_adj(d3 k, double norm_u, d3 kb) {
    return (1.0 / norm_u) * (kb - dot3(k, kb) * k);
}

// ------------------------------------------------------------------ lens
__device__ __forceinline__ Ray lens_fwd(const mgpu_adjoint_problem& P, d3 P0, d3 d0, double f) {
    const d3 c = arr3(P.lens), n = arr3(P.lens + 3), ez = arr3(P.lens + 6);
    double k = dot3(c - P0, n) / dot3(d0, n);
    d3 PL = P0 + k * d0;
    d3 u = (c - P.lens[9] * ez) + f * normalize3(d0) - PL;
    return Ray{PL, normalize3(u)};
}
// adjoint of the output direction -> df (the output position does not depend on theta)
__device__ __forceinline__ double lens_bwd(const mgpu_adjoint_problem& P, d3 P0, d3 d0, double f,
                                           d3 dLb) {
    const d3 c = arr3(P.lens), n = arr3(P.lens + 3), ez = arr3(P.lens + 6);
    double k = dot3(c - P0, n) / dot3(d0, n);
    d3 PL = P0 + k * d0;
    d3 h0 = normalize3(d0);
    d3 u = (c - P.lens[9] * ez) + f * h0 - PL;
    double nu = sqrt(dot3(u, u));
    d3 ub = normalize_adj((1.0 / nu) * u, nu, dLb);
    return dot3(ub, h0);
}

// --------------------------------------------------------------- scatter
__device__ __forceinline__ Ray scatter_fwd(const mgpu_adjoint_problem& P, const Ray& L, double al,
                                           double be) {
    const d3 cS = arr3(P.scatter), nS = arr3(P.scatter + 3);
    double k = dot3(cS - L.p, nS) / dot3(L.d, nS);
    d3 radial = L.p - cS;
    d3 d = L.d;
    if (al != 0.0) {
        double s, c;
        sincos(al, &s, &c);
        d = rot_t(normalize3(cross3(L.d, radial)), c, s, d);
    }
    if (be != 0.0) {
        double s, c;
        sincos(be, &s, &c);
        d = rot_t(normalize3(radial), c, s, d);
    }
    return Ray{L.p + k * L.d, d};
}
// adjoints of the output ray -> adjoint of the input direction
__device__ __forceinline__ d3 scatter_bwd(const mgpu_adjoint_problem& P, const Ray& L, double al,
                                          double be, d3 PSb, d3 dSb) {
    const d3 cS = arr3(P.scatter), nS = arr3(P.scatter + 3);
    d3 radial = L.p - cS;
    d3 d1b = dSb;
    if (be != 0.0) {
        double s, c;
        sincos(be, &s, &c);
        d1b = rot_t_adj_v(normalize3(radial), c, s, dSb);
    }
    d3 dLb = d1b;
    if (al != 0.0) {
        double s, c;
        sincos(al, &s, &c);
        d3 perp = cross3(L.d, radial);
        double np_ = sqrt(dot3(perp, perp));
        d3 k = (1.0 / np_) * perp;
        dLb = rot_t_adj_v(k, c, s, d1b);
        // the axis depends on the direction: y = c v - s k x v + (1-c)(k.v) k
        d3 kb = (-s) * cross3(L.d, d1b) + (1.0 - c) * (dot3(d1b, k) * L.d + dot3(k, L.d) * d1b);
        dLb = dLb + cross3(radial, normalize_adj(k, np_, kb));
    }
    double den = dot3(L.d, nS);
    double k = dot3(cS - L.p, nS) / den;
    double kb = dot3(PSb, L.d);
    return dLb + k * PSb + (-kb * k / den) * nS;
}

// --------------------------------------------------------------- grating
struct Facet {
    d3 c, n, l, dn;
};

__device__ __forceinline__ Facet facet_at(const mgpu_adjoint_problem& P, const double* theta,
                                          int j) {
    const double* fb = P.facets + 13 * (size_t)j;
    const double* R = P.rot + 36 * (size_t)j;
    const double* t = theta + 1 + 6 * j;
    return Facet{d3{fb[0] + t[0], fb[1] + t[1], fb[2] + t[2]}, mat_vec(R, ldg3(fb + 3)),
                 mat_vec(R, ldg3(fb + 6)), mat_vec(R, ldg3(fb + 9))};
}

__device__ __forceinline__ Ray grating_fwd(const Facet& G, const Ray& S, double mterm,
                                           double nsign) {
    double k = dot3(G.c - S.p, G.n) / dot3(S.d, G.n);
    d3 p = normalize3(S.d);
    double pl = dot3(p, G.l), pd = dot3(p, G.dn) + mterm;
    double pn = sqrt(1.0 - pd * pd - pl * pl);
    return Ray{S.p + k * S.d, pd * G.dn + pl * G.l + (nsign * pn) * G.n};
}

// adjoints of the output ray -> adjoints of the input ray and of the facet pose
__device__ __forceinline__ void grating_bwd(const mgpu_adjoint_problem& P, int j, const Facet& G,
                                            const Ray& S, double mterm, double nsign, d3 Pgb,
                                            d3 dgb, d3& PSb, d3& dSb, double* fg) {
    double den = dot3(S.d, G.n);
    d3 cmp = G.c - S.p;
    double k = dot3(cmp, G.n) / den;
    double ns = sqrt(dot3(S.d, S.d));
    d3 p = (1.0 / ns) * S.d;
    double pl = dot3(p, G.l), pd = dot3(p, G.dn) + mterm;
    double pn = sqrt(1.0 - pd * pd - pl * pl);
    // dir = pd dn + pl l + nsign pn n
    double pdb = dot3(dgb, G.dn), plb = dot3(dgb, G.l), pnb = nsign * dot3(dgb, G.n);
    d3 dnb = pd * dgb, lb = pl * dgb, nb = (nsign * pn) * dgb;
    double qb = pnb / (2.0 * pn);
    pdb -= 2.0 * pd * qb;
    plb -= 2.0 * pl * qb;
    d3 pb = plb * G.l + pdb * G.dn;
    lb = lb + plb * p;
    dnb = dnb + pdb * p;
    dSb = normalize_adj(p, ns, pb);
    // position: S.p + k S.d, k = ((c - S.p) . n) / (S.d . n)
    PSb = Pgb;
    double kb = dot3(Pgb, S.d);
    dSb = dSb + k * Pgb;
    double numb = kb / den, denb = -kb * k / den;
    d3 cb = numb * G.n;
    PSb = PSb - numb * G.n;
    nb = nb + numb * cmp + denb * S.d;
    dSb = dSb + denb * G.n;
    // pose: c = c0 + t, (n, l, dn) = R (n0, l0, dn0)
    const double* fb = P.facets + 13 * (size_t)j;
    const double* R = P.rot + 36 * (size_t)j;
    const d3 n0 = ldg3(fb + 3), l0 = ldg3(fb + 6), dn0 = ldg3(fb + 9);
    fg[0] = cb.x;
    fg[1] = cb.y;
    fg[2] = cb.z;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double* dR = R + 9 * (a + 1);
        fg[3 + a] = dot3(nb, mat_vec(dR, n0)) + dot3(lb, mat_vec(dR, l0)) + dot3(dnb, mat_vec(dR, dn0));
    }
}

// -------------------------------------------------------------- detector
// FLAT det[]: centre, e_x, e_y, e_z (unit).  CYL det[]: centre, M, M^-1, R, zoom_z, b1, b2
__device__ __forceinline__ void flat_fwd(const mgpu_adjoint_problem& P, const double* R,
                                         const double* t, const Ray& g, double& x, double& y) {
    d3 c = arr3(P.det) + d3{t[0], t[1], t[2]};
    d3 n = mat_vec(R, arr3(P.det + 3)), ey = mat_vec(R, arr3(P.det + 6)),
       ez = mat_vec(R, arr3(P.det + 9));
    double k = dot3(c - g.p, n) / dot3(g.d, n);
    d3 v = g.p + k * g.d - c;
    x = dot3(v, ey);
    y = dot3(v, ez);
}

__device__ __forceinline__ void flat_bwd(const mgpu_adjoint_problem& P, const double* R,
                                         const double* t, const Ray& g, double xb, double yb,
                                         d3& Pgb, d3& dgb, double* dg6) {
    const d3 n0 = arr3(P.det + 3), ey0 = arr3(P.det + 6), ez0 = arr3(P.det + 9);
    d3 c = arr3(P.det) + d3{t[0], t[1], t[2]};
    d3 n = mat_vec(R, n0), ey = mat_vec(R, ey0), ez = mat_vec(R, ez0);
    double den = dot3(g.d, n);
    d3 cmp = c - g.p;
    double k = dot3(cmp, n) / den;
    d3 v = g.p + k * g.d - c;
    d3 vb = xb * ey + yb * ez;
    d3 eyb = xb * v, ezb = yb * v;
    d3 cb = d3{-vb.x, -vb.y, -vb.z};
    Pgb = vb;
    double kb = dot3(vb, g.d);
    dgb = k * vb;
    double numb = kb / den, denb = -kb * k / den;
    cb = cb + numb * n;
    Pgb = Pgb - numb * n;
    d3 nb = numb * cmp + denb * g.d;
    dgb = dgb + denb * n;
    dg6[0] = cb.x;
    dg6[1] = cb.y;
    dg6[2] = cb.z;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double* dR = R + 9 * (a + 1);
        dg6[3 + a] = dot3(nb, mat_vec(dR, n0)) + dot3(eyb, mat_vec(dR, ey0)) +
                     dot3(ezb, mat_vec(dR, ez0));
    }
}

struct CylLocal {
    d3 q, r, v;              // local position / direction, world offset from the centre
    double aq, bq, cq, sd;   // quadratic coefficients, sqrt of the discriminant
};

__device__ __forceinline__ CylLocal cyl_local(const mgpu_adjoint_problem& P, const double* R,
                                              const double* t, const Ray& g) {
    const double* Minv = P.det + 12;
    CylLocal L;
    L.v = g.p - (arr3(P.det) + d3{t[0], t[1], t[2]});
    L.q = mat_vec(Minv, mat_tvec(R, L.v));
    L.r = mat_vec(Minv, mat_tvec(R, g.d));
    L.aq = L.r.x * L.r.x + L.r.y * L.r.y;
    L.bq = 2.0 * (L.q.x * L.r.x + L.q.y * L.r.y);
    L.cq = L.q.x * L.q.x + L.q.y * L.q.y - 1.0;
    L.sd = sqrt(L.bq * L.bq - 4.0 * L.aq * L.cq);
    return L;
}

// root choice of Cylinder.intersect (geometry.py:526-540): +1 = (-b + sqrt) / 2a
__device__ __forceinline__ int cyl_freeze(const mgpu_adjoint_problem& P, const CylLocal& L,
                                          bool& ok) {
    double s1 = (-L.bq + L.sd) / (2.0 * L.aq), s2 = (-L.bq - L.sd) / (2.0 * L.aq);
    d3 h1 = L.q + s1 * L.r, h2 = L.q + s2 * L.r;
    bool hit1 = (s1 >= 0.0) && (fabs(h1.z) <= 1.0) &&
                angle_between_dev(atan2(h1.y, h1.x), P.det[23], P.det[24]);
    bool hit2 = (s2 >= 0.0) && (fabs(h2.z) <= 1.0) &&
                angle_between_dev(atan2(h2.y, h2.x), P.det[23], P.det[24]);
    ok = hit1 || hit2;
    if (hit1 && hit2) return (s2 < s1) ? -1 : 1;
    return hit2 ? -1 : 1;
}

__device__ __forceinline__ void cyl_fwd(const mgpu_adjoint_problem& P, const CylLocal& L,
                                        double root, double& x, double& y) {
    double s = (-L.bq + root * L.sd) / (2.0 * L.aq);
    d3 h = L.q + s * L.r;
    x = atan2(h.y, h.x) * P.det[21];
    y = h.z * P.det[22];
}

__device__ __forceinline__ void cyl_bwd(const mgpu_adjoint_problem& P, const double* R,
                                        const CylLocal& L, const Ray& g, double root, double xb,
                                        double yb, d3& Pgb, d3& dgb, double* dg6) {
    const double* Minv = P.det + 12;
    double s = (-L.bq + root * L.sd) / (2.0 * L.aq);
    d3 h = L.q + s * L.r;
    double rho2 = h.x * h.x + h.y * h.y;
    double phib = P.det[21] * xb;
    d3 hb = d3{-h.y * phib / rho2, h.x * phib / rho2, P.det[22] * yb};
    d3 qb = hb, rb = s * hb;
    double sb = dot3(hb, L.r);
    double bqb = sb * (-1.0 + root * L.bq / L.sd) / (2.0 * L.aq);
    double cqb = sb * (-root / L.sd);
    double aqb = sb * (-root * L.cq / (L.aq * L.sd) - s / L.aq);
    qb.x += 2.0 * (cqb * L.q.x + bqb * L.r.x);
    qb.y += 2.0 * (cqb * L.q.y + bqb * L.r.y);
    rb.x += 2.0 * (bqb * L.q.x + aqb * L.r.x);
    rb.y += 2.0 * (bqb * L.q.y + aqb * L.r.y);
    // q = M^-1 R^T v, r = M^-1 R^T dir
    d3 qm = mat_tvec(Minv, qb), rm = mat_tvec(Minv, rb);
    Pgb = mat_vec(R, qm);
    dgb = mat_vec(R, rm);
    dg6[0] = -Pgb.x;
    dg6[1] = -Pgb.y;
    dg6[2] = -Pgb.z;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double* dR = R + 9 * (a + 1);
        dg6[3 + a] = dot3(mat_vec(dR, qm), L.v) + dot3(mat_vec(dR, rm), g.d);
    }
}

__device__ __forceinline__ void add_shared(double* s, double v) {
    if (v != 0.0) atomicAdd(s, v);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(MGPU_FULL_MASK, v, off);
    return v;
}

template <int mode>
__global__ void __launch_bounds__(kThreads)
adjoint_kernel(const __grid_constant__ mgpu_adjoint_problem P, const double* __restrict__ theta,
               const double* __restrict__ seeds, double* moments, double* grad) {
    extern __shared__ double sh[];
    const int F = P.n_facets, G = P.n_groups;
    const int nsh = (mode == MGPU_ADJ_BACKWARD) ? 6 * F + 7
                                                : ((mode == MGPU_ADJ_FORWARD) ? 5 * G : 0);
    for (int k = threadIdx.x; k < nsh; k += blockDim.x) sh[k] = 0.0;
    __syncthreads();
    const double f = theta[0];
    const double* Rd = P.rot + 36 * (size_t)F;
    const double* td = theta + 1 + 6 * F;
    const bool cyl = P.det_kind == MGPU_ADJ_DET_CYL;
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    int cg = -1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int g = P.group[i];
        if (mode != MGPU_ADJ_FREEZE && g < 0) continue;
        const int j = P.facet[i];
        if (j < 0 || j >= F || (mode != MGPU_ADJ_FREEZE && g >= G)) {
            atomicOr(P.status, MGPU_STATUS_ADJ_RANGE);
            continue;
        }
        const d3 P0 = ld_soa(P.pos, i, P.n), d0 = ld_soa(P.dir, i, P.n);
        const double al = P.alpha[i], be = P.beta[i];
        const Ray L = lens_fwd(P, P0, d0, f);
        const Ray S = scatter_fwd(P, L, al, be);
        const Facet Fc = facet_at(P, theta, j);
        const double mwave = (double)P.order[i] * (kEnergy2Wave / P.energy[i]) /
                             __ldg(P.facets + 13 * (size_t)j + 12);
        if (mode == MGPU_ADJ_FREEZE) {
            const uint8_t fl = P.facet_flags[j];
            d3 p = normalize3(S.d);
            int sg = -1;                                    // FlatGrating, grating.py:145-172
            if (fl & MGPU_ADJ_FACET_CAT) sg = (dot3(p, Fc.dn) < 0.0) ? -1 : 1;   // grating.py:291-302
            double pn = dot3(p, Fc.n);
            int ns = (pn > 0.0) ? 1 : ((pn < 0.0) ? -1 : 0);
            if (!(fl & MGPU_ADJ_FACET_TRANSMISSION)) ns = -ns;
            P.sign[i] = (int8_t)sg;
            P.nsign[i] = (int8_t)ns;
            if (cyl) {
                const Ray Gr = grating_fwd(Fc, S, sg * mwave, (double)ns);
                bool ok;
                P.root[i] = (int8_t)cyl_freeze(P, cyl_local(P, Rd, td, Gr), ok);
                if (!ok) atomicOr(P.status, MGPU_STATUS_ADJ_RANGE);
            }
            continue;
        }
        const double sg = (double)P.sign[i], ns = (double)P.nsign[i];
        const Ray Gr = grating_fwd(Fc, S, sg * mwave, ns);
        double x, y, root = 0.0;
        CylLocal CL;
        if (cyl) {
            root = (double)P.root[i];
            CL = cyl_local(P, Rd, td, Gr);
            cyl_fwd(P, CL, root, x, y);
        } else {
            flat_fwd(P, Rd, td, Gr, x, y);
        }
        const double w = P.weight[i];
        const double xs = x - __ldg(P.ref + 2 * g), ys = y - __ldg(P.ref + 2 * g + 1);
        if (mode == MGPU_ADJ_FORWARD) {
            if (P.x_out) P.x_out[i] = x;
            if (P.y_out) P.y_out[i] = y;
            if (g != cg) {
                if (cg >= 0)
                    for (int k = 0; k < 5; ++k) add_shared(sh + 5 * cg + k, acc[k]);
                cg = g;
                for (int k = 0; k < 5; ++k) acc[k] = 0.0;
            }
            acc[0] += w;
            acc[1] += w * xs;
            acc[2] += w * ys;
            acc[3] += w * xs * xs;
            acc[4] += w * ys * ys;
            continue;
        }
        // ------------------------------------------------------- reverse sweep
        const double* sd = seeds + 4 * g;
        const double xb = w * (__ldg(sd) + 2.0 * __ldg(sd + 1) * xs);
        const double yb = w * (__ldg(sd + 2) + 2.0 * __ldg(sd + 3) * ys);
        d3 Pgb, dgb;
        double dg6[6];
        if (cyl) cyl_bwd(P, Rd, CL, Gr, root, xb, yb, Pgb, dgb, dg6);
        else flat_bwd(P, Rd, td, Gr, xb, yb, Pgb, dgb, dg6);
        d3 PSb, dSb;
        double fg[6];
        grating_bwd(P, j, Fc, S, sg * mwave, ns, Pgb, dgb, PSb, dSb, fg);
        const d3 dLb = scatter_bwd(P, L, al, be, PSb, dSb);
        acc[0] += lens_bwd(P, P0, d0, f, dLb);
#pragma unroll
        for (int k = 0; k < 6; ++k) acc[1 + k] += dg6[k];
#pragma unroll
        for (int k = 0; k < 6; ++k) add_shared(sh + 6 * j + k, fg[k]);
    }
    if (mode == MGPU_ADJ_FORWARD) {
        const unsigned peers = __match_any_sync(MGPU_FULL_MASK, cg);
        if (peers == MGPU_FULL_MASK) {
            if (cg >= 0) {
                for (int k = 0; k < 5; ++k) {
                    double v = warp_sum(acc[k]);
                    if ((threadIdx.x & 31) == 0) add_shared(sh + 5 * cg + k, v);
                }
            }
        } else if (cg >= 0) {
            for (int k = 0; k < 5; ++k) add_shared(sh + 5 * cg + k, acc[k]);
        }
        __syncthreads();
        for (int k = threadIdx.x; k < 5 * G; k += blockDim.x)
            if (sh[k] != 0.0) atomicAdd(moments + k, sh[k]);
    } else if (mode == MGPU_ADJ_BACKWARD) {
        for (int k = 0; k < 7; ++k) {
            double v = warp_sum(acc[k]);
            if ((threadIdx.x & 31) == 0) add_shared(sh + 6 * F + k, v);
        }
        __syncthreads();
        // grad layout: [f, facet 0 (6), ..., facet F-1 (6), detector (6)]
        for (int k = threadIdx.x; k < nsh; k += blockDim.x) {
            double v = sh[k];
            if (v == 0.0) continue;
            int o = (k < 6 * F) ? 1 + k : ((k == 6 * F) ? 0 : 1 + 6 * F + (k - 6 * F - 1));
            atomicAdd(grad + o, v);
        }
    }
}

template <int mode>
int launch_mode(const mgpu_adjoint_problem& P, const double* theta, const double* seeds,
                double* moments, double* grad, size_t smem, cudaStream_t s) {
    cudaError_t e;
    if (smem > 48 * 1024) {
        e = cudaFuncSetAttribute(adjoint_kernel<mode>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess) return (int)e;
    }
    int dev = 0, sms = 0, per_sm = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return (int)e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return (int)e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, adjoint_kernel<mode>, kThreads,
                                                           smem)) != cudaSuccess)
        return (int)e;
    if (per_sm < 1) return (int)cudaErrorInvalidConfiguration;
    // every block flushes its shared sums once: few blocks when the sums are large
    if (mode == MGPU_ADJ_BACKWARD && per_sm > 2) per_sm = 2;
    int64_t blocks = (P.n + kThreads - 1) / kThreads;
    const int64_t cap = (int64_t)sms * per_sm;
    if (blocks > cap) blocks = cap;
    adjoint_kernel<mode><<<(unsigned)blocks, kThreads, smem, s>>>(P, theta, seeds, moments, grad);
    return (int)cudaGetLastError();
}

}  // namespace

cudaError_t mgpu_pose_adjoint_fp32local(const mgpu_adjoint_problem& P, const double* theta,
                                        int mode, const double* seeds, double* moments,
                                        double* grad, cudaStream_t s);

extern "C" int mgpu_pose_adjoint(const mgpu_adjoint_problem* prob, const double* theta,
                                 int32_t mode, const double* seeds, double* moments, double* grad,
                                 void* stream) {
    if (prob == nullptr || theta == nullptr || prob->rot == nullptr || prob->status == nullptr)
        return (int)cudaErrorInvalidValue;
    const mgpu_adjoint_problem& P = *prob;
    if (P.n_facets < 1 || P.n_facets > MGPU_ADJ_MAX_FACETS || P.n_groups < 0 ||
        P.n_groups > MGPU_ADJ_MAX_GROUPS || P.n < 0)
        return (int)cudaErrorInvalidValue;
    if (P.det_kind != MGPU_ADJ_DET_FLAT && P.det_kind != MGPU_ADJ_DET_CYL)
        return (int)cudaErrorInvalidValue;
    if (P.precision != MGPU_FP64 && P.precision != MGPU_FP32LOCAL) return (int)cudaErrorInvalidValue;
    if (P.precision == MGPU_FP32LOCAL && P.det_kind != MGPU_ADJ_DET_FLAT && mode != MGPU_ADJ_FREEZE)
        return (int)cudaErrorInvalidValue;
    if (P.n > 0 && (!P.pos || !P.dir || !P.alpha || !P.beta || !P.energy || !P.weight ||
                    !P.facet || !P.order || !P.group || !P.facets || !P.facet_flags ||
                    !P.sign || !P.nsign || (P.det_kind == MGPU_ADJ_DET_CYL && !P.root)))
        return (int)cudaErrorInvalidValue;
    if (mode == MGPU_ADJ_FORWARD) {
        if (moments == nullptr || P.ref == nullptr) return (int)cudaErrorInvalidValue;
    } else if (mode == MGPU_ADJ_BACKWARD) {
        if (grad == nullptr || seeds == nullptr || P.ref == nullptr)
            return (int)cudaErrorInvalidValue;
    } else if (mode != MGPU_ADJ_FREEZE) {
        return (int)cudaErrorInvalidValue;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int F = P.n_facets;
    if (P.precision == MGPU_FP32LOCAL && mode != MGPU_ADJ_FREEZE)
        return (int)mgpu_pose_adjoint_fp32local(P, theta, mode, seeds, moments, grad, s);
    pose_prep_kernel<<<(F + 1 + 127) / 128, 128, 0, s>>>(theta, F, P.rot);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || P.n == 0) return (int)e;
    if (mode == MGPU_ADJ_FREEZE)
        return launch_mode<MGPU_ADJ_FREEZE>(P, theta, seeds, moments, grad, 0, s);
    if (mode == MGPU_ADJ_FORWARD)
        return launch_mode<MGPU_ADJ_FORWARD>(P, theta, seeds, moments, grad,
                                             sizeof(double) * 5 * (size_t)P.n_groups, s);
    return launch_mode<MGPU_ADJ_BACKWARD>(P, theta, seeds, moments, grad,
                                          sizeof(double) * (6 * (size_t)F + 7), s);
}
