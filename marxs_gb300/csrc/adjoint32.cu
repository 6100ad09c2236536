// Pose adjoint in FP32-local precision (flat detectors; sm_103a).
//
// The frozen photons, moments and reverse sweep of adjoint.cu (lens
// optics/mirror.py:53-82, scatter optics/scatter.py:49-77, grating
// optics/grating.py:233-266, flat detector math/geometry.py:233-252), with
// the arithmetic split the way the FP32-local chain kernel splits it:
//   * photon positions are float-float; every plane crossing is re-centred
//     on its element (pos - centre as an unnormalised TwoSum pair, the ray
//     parameter from a float32 solve, the local offset formed inside FMAs
//     and refined once), so the detector coordinates keep ~1e-8 of the
//     element's size instead of ~1e-7 of the path length;
//   * directions, frames and the whole reverse sweep are float32: the
//     adjoints are derivatives and need relative, not absolute, precision;
//   * the per-photon terms are summed in float64 (moments, gradient).
// A prep kernel writes each element's posed record once per launch from
// theta in float64: the centre as float-float, the rotated frame and, for
// the reverse sweep, dR/da_k applied to the base frame.
#include <cuda_runtime.h>
#include "mgpu_ff.cuh"

namespace {

constexpr int kThreads = 256;

// posed element record, 192 B: facets 0..F-1, the detector at F, the lens at
// F+1 (n = e_x, l = e_z, aux[0] = d_center_optical_axis, aux[1] = focal
// length), the scatter plane at F+2 (n = e_x)
struct Posed32 {
    float c_hi[3], c_lo[3];
    float n[3], l[3], dn[3];    // facet: normal, groove, -perp; detector: e_x, e_y, e_z
    float aux[2];               // facet: energy2wave / grating constant as float-float (keV)
    float dRn[9], dRl[9], dRdn[9];   // dR/da_k times the base n, l, dn (k-major)
    float pad[4];
};
static_assert(sizeof(Posed32) == 192, "posed record layout");

__device__ __forceinline__ void split3(const double* v, float* hi, float* lo) {
    for (int k = 0; k < 3; ++k) {
        hi[k] = __double2float_rn(v[k]);
        lo[k] = __double2float_rn(v[k] - (double)hi[k]);
    }
}
__device__ __forceinline__ void mv(const double* M, const double* v, double* out) {
    for (int r = 0; r < 3; ++r) out[r] = M[3 * r] * v[0] + M[3 * r + 1] * v[1] + M[3 * r + 2] * v[2];
}
__device__ __forceinline__ void to_f3(const double* v, float* out) {
    for (int k = 0; k < 3; ++k) out[k] = __double2float_rn(v[k]);
}

// R = Rz(a2) Ry(a1) Rx(a0) and dR/da0, dR/da1, dR/da2 (design/uncertainties.py:36-38)
__device__ void rot_and_derivs(const double* a, double* R /* 4 x 9 */) {
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
    double T[9], U[9];
    mul(Rz, Ry, T);
    mul(T, Rx, R);
    mul(T, dRx, R + 9);
    mul(Rz, dRy, U);
    mul(U, Rx, R + 18);
    mul(dRz, Ry, U);
    mul(U, Rx, R + 27);
}

// a posed frame: centre c0 + t, the three base vectors rotated, their
// derivatives
__device__ void posed_frame(const double* c0, const double* b0, const double* b1,
                            const double* b2, const double* t, const double* a, Posed32& o) {
    double R[36], c[3], v[3];
    rot_and_derivs(a, R);
    for (int k = 0; k < 3; ++k) c[k] = c0[k] + t[k];
    split3(c, o.c_hi, o.c_lo);
    mv(R, b0, v);
    to_f3(v, o.n);
    mv(R, b1, v);
    to_f3(v, o.l);
    mv(R, b2, v);
    to_f3(v, o.dn);
    for (int k = 0; k < 3; ++k) {
        mv(R + 9 * (k + 1), b0, v);
        to_f3(v, o.dRn + 3 * k);
        mv(R + 9 * (k + 1), b1, v);
        to_f3(v, o.dRl + 3 * k);
        mv(R + 9 * (k + 1), b2, v);
        to_f3(v, o.dRdn + 3 * k);
    }
}

__global__ void pose_prep32_kernel(const __grid_constant__ mgpu_adjoint_problem P,
                                   const double* __restrict__ theta, Posed32* rec) {
    const int F = P.n_facets;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j > F + 2) return;
    Posed32 o = {};
    if (j < F) {
        const double* fb = P.facets + 13 * (size_t)j;
        posed_frame(fb, fb + 3, fb + 6, fb + 9, theta + 1 + 6 * j, theta + 1 + 6 * j + 3, o);
        const double wd = 1.2398419292004202e-06 / fb[12];
        o.aux[0] = __double2float_rn(wd);
        o.aux[1] = __double2float_rn(wd - (double)o.aux[0]);
    } else if (j == F) {
        const double* t = theta + 1 + 6 * F;
        posed_frame(P.det, P.det + 3, P.det + 6, P.det + 9, t, t + 3, o);
    } else if (j == F + 1) {
        split3(P.lens, o.c_hi, o.c_lo);
        to_f3(P.lens + 3, o.n);
        to_f3(P.lens + 6, o.l);
        o.aux[0] = (float)P.lens[9];
        o.aux[1] = (float)theta[0];
    } else {
        split3(P.scatter, o.c_hi, o.c_lo);
        to_f3(P.scatter + 3, o.n);
    }
    rec[j] = o;
}

// ------------------------------------------------------------- forward
struct Cross {
    float k;     // ray parameter
    f3 v;        // crossing point - element centre
    f3 r0;       // ray start - element centre
    float kd;    // d . n
};

// FinitePlane.intersect without the bounds (the photon's element is frozen)
__device__ __forceinline__ Cross plane_cross(const ff3& p, f3 d, const ff3& c, f3 n) {
    Cross x;
    f3 s, e;
    ff3_rel(p, c, s, e);
    x.kd = dotf(d, n);
    float k = -(dotf(s, n) + dotf(e, n)) / x.kd;
    f3 v{fmaf(k, d.x, s.x) + e.x, fmaf(k, d.y, s.y) + e.y, fmaf(k, d.z, s.z) + e.z};
    const float dk = -dotf(v, n) / x.kd;
    if (isfinite(dk)) {
        k += dk;
        v = f3{fmaf(dk, d.x, v.x), fmaf(dk, d.y, v.y), fmaf(dk, d.z, v.z)};
    }
    x.k = k;
    x.v = v;
    x.r0 = s + e;
    return x;
}

__device__ __forceinline__ ff3 rec_centre(const Posed32* r) {
    return ff3{ff{__ldg(r->c_hi), __ldg(r->c_lo)}, ff{__ldg(r->c_hi + 1), __ldg(r->c_lo + 1)},
               ff{__ldg(r->c_hi + 2), __ldg(r->c_lo + 2)}};
}
__device__ __forceinline__ f3 ldg3f(const float* p) { return f3{__ldg(p), __ldg(p + 1), __ldg(p + 2)}; }

// R^T v for R = axangle2mat(k, angle), k a unit vector; 1 - cos as 2 sin^2(a/2)
__device__ __forceinline__ f3 rot_t_f(f3 k, float c, float s, float omc, f3 v) {
    const f3 kv = crossf(k, v);
    const float kd = omc * dotf(k, v);
    return f3{c * v.x - s * kv.x + kd * k.x, c * v.y - s * kv.y + kd * k.y,
              c * v.z - s * kv.z + kd * k.z};
}
// adjoint of v in y = R^T(k, angle) v
__device__ __forceinline__ f3 rot_t_adj_f(f3 k, float c, float s, float omc, f3 yb) {
    const f3 ky = crossf(k, yb);
    const float kd = omc * dotf(k, yb);
    return f3{c * yb.x + s * ky.x + kd * k.x, c * yb.y + s * ky.y + kd * k.y,
              c * yb.z + s * ky.z + kd * k.z};
}
// adjoint of u from the adjoint of k = u / |u|
__device__ __forceinline__ f3 normalize_adj_f(f3 k, float norm_u, f3 kb) {
    return (1.0f / norm_u) * (kb - dotf(k, kb) * k);
}
struct Turn {
    float c, s, omc;
};
__device__ __forceinline__ Turn turn(float a) {
    Turn t;
    sincosf(a, &t.s, &t.c);
    const float h = sinf(0.5f * a);
    t.omc = 2.0f * h * h;
    return t;
}

// one photon through the chain: the forward values the reverse sweep needs
struct Path {
    ff3 P0;
    f3 d0, h0, u, dL;
    float nu, f;
    Cross L, S, G, D;
    f3 radial, dS;
    float x, y;
    // grating
    f3 p;
    float ns, pl, pd, pn;
    f3 dG;
};

// one photon forward; ``sm`` = order sign * order, the grating term
// sign m lambda / d formed in float-float from the photon's energy
__device__ __forceinline__ void forward(const Posed32* rec, int F, int j, float al, float be,
                                        ff energy, float sm, float nsign, Path& q) {
    const Posed32* lens = rec + F + 1;
    const Posed32* sct = rec + F + 2;
    const Posed32* fac = rec + j;
    const Posed32* det = rec + F;
    // lens: crossing, then towards centre - d_off e_z + f norm(dir)
    const ff3 cL = rec_centre(lens);
    const f3 nL = ldg3f(lens->n), ezL = ldg3f(lens->l);
    q.f = __ldg(lens->aux + 1);
    q.L = plane_cross(q.P0, q.d0, cL, nL);
    q.h0 = normf(q.d0);
    q.u = (q.f * q.h0 - __ldg(lens->aux) * ezL) - q.L.v;
    q.nu = sqrtf(dotf(q.u, q.u));
    q.dL = (1.0f / q.nu) * q.u;
    // scatter: crossing of its plane from the lens point, R^T turns
    const ff3 PL = ff3_add_f3(cL, q.L.v);
    const ff3 cS = rec_centre(sct);
    const f3 nS = ldg3f(sct->n);
    q.S = plane_cross(PL, q.dL, cS, nS);
    q.radial = q.S.r0;
    f3 d = q.dL;
    if (al != 0.0f) {
        const Turn t = turn(al);
        d = rot_t_f(normf(crossf(q.dL, q.radial)), t.c, t.s, t.omc, d);
    }
    if (be != 0.0f) {
        const Turn t = turn(be);
        d = rot_t_f(normf(q.radial), t.c, t.s, t.omc, d);
    }
    q.dS = d;
    // grating: crossing of the facet plane, grating equation
    const ff3 PS = ff3_add_f3(cS, q.S.v);
    const ff3 cG = rec_centre(fac);
    const f3 n = ldg3f(fac->n), l = ldg3f(fac->l), dn = ldg3f(fac->dn);
    q.G = plane_cross(PS, q.dS, cG, n);
    q.ns = sqrtf(dotf(q.dS, q.dS));
    q.p = (1.0f / q.ns) * q.dS;
    q.pl = dotf(q.p, l);
    const float p_d = dotf(q.p, dn), p_n = dotf(q.p, n);
    // sign m lambda / d in float-float; the new components exactly as the
    // FP32-local chain forms them: pd = p.dn + term, and the change of the
    // normal component without cancellation when the side is kept
    const ff term = ff_mul_f(ff_div(ff{__ldg(fac->aux), __ldg(fac->aux + 1)}, energy), sm);
    const float tf = ff_f(term);
    q.pd = ff_f(ff_add_f(term, p_d));
    q.pn = sqrtf(1.0f - q.pd * q.pd - q.pl * q.pl);
    const float side = (p_n > 0.0f) ? 1.0f : ((p_n < 0.0f) ? -1.0f : 0.0f);
    const float dnc = (nsign == side) ? nsign * (-tf * (2.0f * p_d + tf)) / (q.pn + fabsf(p_n))
                                      : nsign * q.pn - p_n;
    q.dG = q.p + (tf * dn + dnc * n);
    // detector plane: local (y, z)
    const ff3 PG = ff3_add_f3(cG, q.G.v);
    q.D = plane_cross(PG, q.dG, rec_centre(det), ldg3f(det->n));
    q.x = dotf(q.D.v, ldg3f(det->l));
    q.y = dotf(q.D.v, ldg3f(det->dn));
}

// ------------------------------------------------------------- reverse
// detector: adjoints of the grating ray and the detector pose (6)
__device__ __forceinline__ void det_bwd(const Posed32* det, const Path& q, float xb, float yb,
                                        f3& Pgb, f3& dgb, float* dg6) {
    const f3 n = ldg3f(det->n), ey = ldg3f(det->l), ez = ldg3f(det->dn);
    const f3 v = q.D.v, cmp = -1.0f * q.D.r0;       // c - hit point of the grating
    const float k = q.D.k, den = q.D.kd;
    const f3 vb = xb * ey + yb * ez;
    const f3 eyb = xb * v, ezb = yb * v;
    f3 cb = -1.0f * vb;
    Pgb = vb;
    const float kb = dotf(vb, q.dG);
    dgb = k * vb;
    const float numb = kb / den, denb = -kb * k / den;
    cb = cb + numb * n;
    Pgb = Pgb - numb * n;
    const f3 nb = numb * cmp + denb * q.dG;
    dgb = dgb + denb * n;
    dg6[0] = cb.x;
    dg6[1] = cb.y;
    dg6[2] = cb.z;
#pragma unroll
    for (int a = 0; a < 3; ++a)
        dg6[3 + a] = dotf(nb, ldg3f(det->dRn + 3 * a)) + dotf(eyb, ldg3f(det->dRl + 3 * a)) +
                     dotf(ezb, ldg3f(det->dRdn + 3 * a));
}

// grating: adjoints of the scatter ray and the facet pose (6)
__device__ __forceinline__ void grating_bwd(const Posed32* fac, const Path& q, float nsign,
                                            f3 Pgb, f3 dgb, f3& PSb, f3& dSb, float* fg) {
    const f3 n = ldg3f(fac->n), l = ldg3f(fac->l), dn = ldg3f(fac->dn);
    const f3 cmp = -1.0f * q.G.r0;                  // facet centre - scatter point
    const float den = q.G.kd, k = q.G.k;
    float pdb = dotf(dgb, dn), plb = dotf(dgb, l);
    const float pnb = nsign * dotf(dgb, n);
    f3 dnb = q.pd * dgb, lb = q.pl * dgb, nb = (nsign * q.pn) * dgb;
    const float qb = pnb / (2.0f * q.pn);
    pdb -= 2.0f * q.pd * qb;
    plb -= 2.0f * q.pl * qb;
    const f3 pb = plb * l + pdb * dn;
    lb = lb + plb * q.p;
    dnb = dnb + pdb * q.p;
    dSb = normalize_adj_f(q.p, q.ns, pb);
    PSb = Pgb;
    const float kb = dotf(Pgb, q.dS);
    dSb = dSb + k * Pgb;
    const float numb = kb / den, denb = -kb * k / den;
    const f3 cb = numb * n;
    PSb = PSb - numb * n;
    nb = nb + numb * cmp + denb * q.dS;
    dSb = dSb + denb * n;
    fg[0] = cb.x;
    fg[1] = cb.y;
    fg[2] = cb.z;
#pragma unroll
    for (int a = 0; a < 3; ++a)
        fg[3 + a] = dotf(nb, ldg3f(fac->dRn + 3 * a)) + dotf(lb, ldg3f(fac->dRl + 3 * a)) +
                    dotf(dnb, ldg3f(fac->dRdn + 3 * a));
}

// scatter: adjoint of the lens direction
__device__ __forceinline__ f3 scatter_bwd(const Posed32* sct, const Path& q, float al, float be,
                                          f3 PSb, f3 dSb) {
    const f3 nS = ldg3f(sct->n);
    f3 d1b = dSb;
    if (be != 0.0f) {
        const Turn t = turn(be);
        d1b = rot_t_adj_f(normf(q.radial), t.c, t.s, t.omc, dSb);
    }
    f3 dLb = d1b;
    if (al != 0.0f) {
        const Turn t = turn(al);
        const f3 perp = crossf(q.dL, q.radial);
        const float np_ = sqrtf(dotf(perp, perp));
        const f3 k = (1.0f / np_) * perp;
        dLb = rot_t_adj_f(k, t.c, t.s, t.omc, d1b);
        // the axis depends on the direction: y = c v - s k x v + (1-c)(k.v) k
        const f3 kb = (-t.s) * crossf(q.dL, d1b) + t.omc * (dotf(d1b, k) * q.dL + dotf(k, q.dL) * d1b);
        dLb = dLb + crossf(q.radial, normalize_adj_f(k, np_, kb));
    }
    const float kb = dotf(PSb, q.dL);
    return dLb + q.S.k * PSb + (-kb * q.S.k / q.S.kd) * nS;
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
adjoint32_kernel(const __grid_constant__ mgpu_adjoint_problem P, const Posed32* __restrict__ rec,
                 const double* __restrict__ seeds, double* moments, double* grad) {
    extern __shared__ double sh[];
    const int F = P.n_facets, G = P.n_groups;
    const int nsh = (mode == MGPU_ADJ_BACKWARD) ? 6 * F + 7 : 5 * G;
    for (int k = threadIdx.x; k < nsh; k += blockDim.x) sh[k] = 0.0;
    __syncthreads();
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    int cg = -1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int g = P.group[i];
        if (g < 0) continue;
        const int j = P.facet[i];
        if (j < 0 || j >= F || g >= G) {
            atomicOr(P.status, MGPU_STATUS_ADJ_RANGE);
            continue;
        }
        Path q;
        q.P0 = ff3{d2ff_bits(P.pos[i]), d2ff_bits(P.pos[P.n + i]), d2ff_bits(P.pos[2 * P.n + i])};
        q.d0 = f3{__double2float_rn(P.dir[i]), __double2float_rn(P.dir[P.n + i]),
                  __double2float_rn(P.dir[2 * P.n + i])};
        const float al = __double2float_rn(P.alpha[i]), be = __double2float_rn(P.beta[i]);
        const float sg = (float)P.sign[i], nsign = (float)P.nsign[i];
        forward(rec, F, j, al, be, d2ff_bits(P.energy[i]), sg * (float)P.order[i], nsign, q);
        const double w = P.weight[i];
        const float xs = q.x - __double2float_rn(__ldg(P.ref + 2 * g));
        const float ys = q.y - __double2float_rn(__ldg(P.ref + 2 * g + 1));
        if (mode == MGPU_ADJ_FORWARD) {
            if (P.x_out) P.x_out[i] = (double)q.x;
            if (P.y_out) P.y_out[i] = (double)q.y;
            if (g != cg) {
                if (cg >= 0)
                    for (int k = 0; k < 5; ++k) add_shared(sh + 5 * cg + k, acc[k]);
                cg = g;
                for (int k = 0; k < 5; ++k) acc[k] = 0.0;
            }
            const double xd = (double)xs, yd = (double)ys;
            acc[0] += w;
            acc[1] += w * xd;
            acc[2] += w * yd;
            acc[3] += w * xd * xd;
            acc[4] += w * yd * yd;
            continue;
        }
        // ------------------------------------------------------- reverse sweep
        const double* sd = seeds + 4 * g;
        const float xb = (float)(w * (__ldg(sd) + 2.0 * __ldg(sd + 1) * (double)xs));
        const float yb = (float)(w * (__ldg(sd + 2) + 2.0 * __ldg(sd + 3) * (double)ys));
        f3 Pgb, dgb, PSb, dSb;
        float dg6[6], fg[6];
        det_bwd(rec + F, q, xb, yb, Pgb, dgb, dg6);
        grating_bwd(rec + j, q, nsign, Pgb, dgb, PSb, dSb, fg);
        const f3 dLb = scatter_bwd(rec + F + 2, q, al, be, PSb, dSb);
        // lens: the output position does not depend on theta; df from the direction
        acc[0] += (double)dotf(normalize_adj_f(q.dL, q.nu, dLb), q.h0);
#pragma unroll
        for (int k = 0; k < 6; ++k) acc[1 + k] += (double)dg6[k];
#pragma unroll
        for (int k = 0; k < 6; ++k) add_shared(sh + 6 * j + k, (double)fg[k]);
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
    } else {
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
cudaError_t launch32(const mgpu_adjoint_problem& P, const Posed32* rec, const double* seeds,
                     double* moments, double* grad, size_t smem, cudaStream_t s) {
    cudaError_t e;
    if (smem > 48 * 1024) {
        e = cudaFuncSetAttribute(adjoint32_kernel<mode>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess) return e;
    }
    int dev = 0, sms = 0, per_sm = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, adjoint32_kernel<mode>,
                                                           kThreads, smem)) != cudaSuccess)
        return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    // every block flushes its shared sums once: few blocks when the sums are large
    if (mode == MGPU_ADJ_BACKWARD && per_sm > 2) per_sm = 2;
    int64_t blocks = (P.n + kThreads - 1) / kThreads;
    const int64_t cap = (int64_t)sms * per_sm;
    if (blocks > cap) blocks = cap;
    adjoint32_kernel<mode><<<(unsigned)blocks, kThreads, smem, s>>>(P, rec, seeds, moments, grad);
    return cudaGetLastError();
}

}  // namespace

// FORWARD / BACKWARD of mgpu_pose_adjoint in FP32-local precision, flat
// detectors; prob->rot holds at least (n_facets + 3) 192-byte posed records
cudaError_t mgpu_pose_adjoint_fp32local(const mgpu_adjoint_problem& P, const double* theta,
                                        int mode, const double* seeds, double* moments,
                                        double* grad, cudaStream_t s) {
    const int F = P.n_facets;
    Posed32* rec = reinterpret_cast<Posed32*>(P.rot);
    pose_prep32_kernel<<<(F + 3 + 127) / 128, 128, 0, s>>>(P, theta, rec);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || P.n == 0) return e;
    if (mode == MGPU_ADJ_FORWARD)
        return launch32<MGPU_ADJ_FORWARD>(P, rec, seeds, moments, grad,
                                          sizeof(double) * 5 * (size_t)P.n_groups, s);
    return launch32<MGPU_ADJ_BACKWARD>(P, rec, seeds, moments, grad,
                                       sizeof(double) * (6 * (size_t)F + 7), s);
}
