// Device helpers shared by the raytrace kernels (sm_103a).
//
// Float64 helpers restate the MARXS numpy arithmetic element by element so
// that the FP64 kernels agree with the reference to rounding level:
//   norm_vector            marxs/math/utils.py:150-164
//   angle_between          marxs/math/utils.py:180-215 (numpy floor modulo)
//   axangle2mat (applied   marxs/math/rotations.py:50-87 with the transposed
//     as R^T v)              product einsum('...ij,...i->...j') of scatter.py:59,67
//   parallel_transport     marxs/math/polarization.py:90-170 (Jones = identity)
#pragma once
#include <stdint.h>
#include <math.h>
#include "../../include/marxs_gb300.h"

#define MGPU_FULL_MASK 0xffffffffu
#define kNaN __longlong_as_double(0x7ff8000000000000ll)

struct d3 {
    double x, y, z;
};

__device__ __forceinline__ d3 mk3(double x, double y, double z) { return d3{x, y, z}; }
__device__ __forceinline__ d3 operator+(d3 a, d3 b) { return d3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ d3 operator-(d3 a, d3 b) { return d3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ d3 operator*(double s, d3 a) { return d3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ double dot3(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ d3 cross3(d3 a, d3 b) {
    return d3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// v / sqrt(v.v), component-wise division as numpy does
__device__ __forceinline__ d3 normalize3(d3 v) {
    double n = sqrt(dot3(v, v));
    return d3{v.x / n, v.y / n, v.z / n};
}

__device__ __forceinline__ d3 load3(const mgpu_vec& v, int64_t i) {
    const double* p = v.ptr + i * v.stride;
    return d3{p[0], p[v.cstride], p[2 * v.cstride]};
}
__device__ __forceinline__ void store3(const mgpu_vec& v, int64_t i, d3 a) {
    double* p = v.ptr + i * v.stride;
    p[0] = a.x;
    p[v.cstride] = a.y;
    p[2 * v.cstride] = a.z;
}
__device__ __forceinline__ d3 arr3(const double* a) { return d3{a[0], a[1], a[2]}; }
__device__ __forceinline__ d3 ldg3(const double* a) { return d3{__ldg(a), __ldg(a + 1), __ldg(a + 2)}; }

__device__ __forceinline__ void store_col(const mgpu_col& c, int64_t i, double v) {
    if (c.ptr) c.ptr[i * c.stride] = v;
}

// numpy floor modulo for doubles (remainder with the sign of the divisor)
__device__ __forceinline__ double np_mod(double a, double b) {
    double m = fmod(a, b);
    if (m != 0.0) {
        if ((b < 0.0) != (m < 0.0)) m += b;
    } else {
        m = copysign(0.0, b);
    }
    return m;
}

// angle_between with borders already reduced on the host:
// b1 = (2pi + (border1 % 2pi)) % 2pi, b2 likewise
__device__ __forceinline__ bool angle_between_dev(double angle, double b1, double b2) {
    const double twopi = 2.0 * 3.141592653589793;
    double ang = np_mod(twopi + np_mod(angle, twopi), twopi);
    if (b1 < b2) return (b1 <= ang) && (ang <= b2);
    return (b1 <= ang) || (ang <= b2);
}

// R^T v where R = axangle2mat(axis, angle) (axis normalised inside)
__device__ __forceinline__ d3 rot_transpose_apply(d3 axis, double angle, d3 v) {
    double n = sqrt(dot3(axis, axis));
    double x = axis.x / n, y = axis.y / n, z = axis.z / n;
    double s, c;
    sincos(angle, &s, &c);
    double C = 1.0 - c;
    double xs = x * s, ys = y * s, zs = z * s;
    double xC = x * C, yC = y * C, zC = z * C;
    double xyC = x * yC, yzC = y * zC, zxC = z * xC;
    double m00 = x * xC + c, m01 = xyC - zs, m02 = zxC + ys;
    double m10 = xyC + zs, m11 = y * yC + c, m12 = yzC - xs;
    double m20 = zxC - ys, m21 = yzC + xs, m22 = z * zC + c;
    return d3{m00 * v.x + m10 * v.y + m20 * v.z,
              m01 * v.x + m11 * v.y + m21 * v.z,
              m02 * v.x + m12 * v.y + m22 * v.z};
}

// parallel_transport(dir_old, dir_new, pol) with Jones = identity and
// replace_nans=True: identity where |dir1 x dir2| <= 1e-8 (np.isclose)
__device__ __forceinline__ d3 parallel_transport_dev(d3 d_old, d3 d_new, d3 pol) {
    d3 a = normalize3(d_old);
    d3 b = normalize3(d_new);
    d3 s = cross3(a, b);
    double sn = sqrt(dot3(s, s));
    if (sn <= 1e-8) return pol;
    s = d3{s.x / sn, s.y / sn, s.z / sn};
    d3 pin = cross3(a, s);
    d3 pout = cross3(b, s);
    double ks = dot3(s, pol), kp = dot3(pin, pol), kd = dot3(a, pol);
    return d3{s.x * ks + pout.x * kp + b.x * kd,
              s.y * ks + pout.y * kp + b.y * kd,
              s.z * ks + pout.z * kp + b.z * kd};
}

// FinitePlane.intersect (math/geometry.py:211-261) for one photon
struct PlaneHit {
    bool hit;
    double k;
    d3 ip;
    double ly, lz;
};

__device__ __forceinline__ PlaneHit plane_intersect(d3 c, d3 ex, d3 ey, d3 ez, double hy,
                                                    double hz, d3 pos, d3 dir) {
    PlaneHit r;
    double kn = dot3(c - pos, ex);
    double kd = dot3(dir, ex);
    r.k = kn / kd;
    // pos + k * dir with the product rounded on its own, as numpy evaluates it
    r.ip = d3{__dadd_rn(pos.x, __dmul_rn(r.k, dir.x)), __dadd_rn(pos.y, __dmul_rn(r.k, dir.y)),
              __dadd_rn(pos.z, __dmul_rn(r.k, dir.z))};
    d3 v = r.ip - c;
    r.ly = dot3(v, ey);
    r.lz = dot3(v, ez);
    r.hit = (kd != 0.0) && (r.k >= 0.0) && (fabs(r.ly) <= hy) && (fabs(r.lz) <= hz);
    return r;
}


struct CylHit {
    bool hit;
    double phi, zl;   // local phi and z (z already scaled by the pose's z zoom)
    d3 ip;            // global intersection point
};

// Cylinder.intersect (math/geometry.py:470-564) for one photon.  cyl holds
// pos4d rows 0..2 (12), inverse rows 0..2 (12), zoom_z, R, and the two
// reduced phi_lim borders.
__device__ __forceinline__ CylHit cylinder_intersect_dev(const double* cyl, d3 p, d3 d) {
    const double* M = cyl;
    const double* Mi = cyl + 12;
    double zoomz = cyl[24], b1 = cyl[26], b2 = cyl[27];
    d3 xyz{Mi[0] * p.x + Mi[1] * p.y + Mi[2] * p.z + Mi[3],
           Mi[4] * p.x + Mi[5] * p.y + Mi[6] * p.z + Mi[7],
           Mi[8] * p.x + Mi[9] * p.y + Mi[10] * p.z + Mi[11]};
    d3 r{Mi[0] * d.x + Mi[1] * d.y + Mi[2] * d.z,
         Mi[4] * d.x + Mi[5] * d.y + Mi[6] * d.z,
         Mi[8] * d.x + Mi[9] * d.y + Mi[10] * d.z};
    double c = (xyz.x * xyz.x + xyz.y * xyz.y) - 1.0;
    double b = 2.0 * (xyz.x * r.x + xyz.y * r.y);
    double a = r.x * r.x + r.y * r.y;
    double ur = b * b - 4.0 * a * c;
    CylHit out;
    out.hit = false;
    out.phi = out.zl = 0.0;
    out.ip = d3{0.0, 0.0, 0.0};
    if (!(ur >= 0.0)) return out;
    double sq = sqrt(ur);
    double den = 2.0 * a;
    double a1 = (-b + sq) / den;
    double a2 = (-b - sq) / den;
    double phi1 = atan2(xyz.y + a1 * r.y, xyz.x + a1 * r.x);
    double phi2 = atan2(xyz.y + a2 * r.y, xyz.x + a2 * r.x);
    double z1 = xyz.z + a1 * r.z;
    double z2 = xyz.z + a2 * r.z;
    bool h1 = (a1 >= 0.0) && (fabs(z1) <= 1.0) && angle_between_dev(phi1, b1, b2);
    bool h2 = (a2 >= 0.0) && (fabs(z2) <= 1.0) && angle_between_dev(phi2, b1, b2);
    if (h1 && h2) {
        if (a2 < a1) h1 = false;
        else h2 = false;
    }
    double t;
    if (h1) {
        out.phi = phi1;
        out.zl = z1;
        t = a1;
    } else if (h2) {
        out.phi = phi2;
        out.zl = z2;
        t = a2;
    } else {
        return out;
    }
    out.hit = true;
    d3 lp{__dadd_rn(xyz.x, __dmul_rn(t, r.x)), __dadd_rn(xyz.y, __dmul_rn(t, r.y)),
          __dadd_rn(xyz.z, __dmul_rn(t, r.z))};
    out.ip = d3{M[0] * lp.x + M[1] * lp.y + M[2] * lp.z + M[3],
                M[4] * lp.x + M[5] * lp.y + M[6] * lp.z + M[7],
                M[8] * lp.x + M[9] * lp.y + M[10] * lp.z + M[11]};
    out.zl = out.zl * zoomz;
    return out;
}

// ---------------------------------------------------------------------------
// Philox4x32-10 counter-based generator (Salmon et al., SC'11): 10 rounds of
// the Philox S-box with the published multipliers and Weyl key increments.
// ---------------------------------------------------------------------------
struct u4 {
    uint32_t x, y, z, w;
};

__device__ __forceinline__ u4 philox4x32_10(u4 ctr, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(M0, ctr.x), lo0 = M0 * ctr.x;
        uint32_t hi1 = __umulhi(M1, ctr.z), lo1 = M1 * ctr.z;
        ctr = u4{hi1 ^ ctr.y ^ k0, lo1, hi0 ^ ctr.w ^ k1, lo0};
        k0 += W0;
        k1 += W1;
    }
    return ctr;
}

// two 53-bit uniforms in [0, 1) for (seed, photon row, stage, draw pair)
__device__ __forceinline__ void philox_uniform2(uint64_t seed, uint64_t row, uint32_t stage,
                                                uint32_t draw, double* u0, double* u1) {
    u4 c{(uint32_t)row, (uint32_t)(row >> 32), stage, draw};
    u4 r = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    uint64_t a = ((uint64_t)r.x << 21) ^ (uint64_t)(r.y >> 11);
    uint64_t b = ((uint64_t)r.z << 21) ^ (uint64_t)(r.w >> 11);
    a &= (1ull << 53) - 1;
    b &= (1ull << 53) - 1;
    *u0 = (double)a * (1.0 / 9007199254740992.0);
    *u1 = (double)b * (1.0 / 9007199254740992.0);
}

// two standard normals by the Box-Muller transform
__device__ __forceinline__ void philox_normal2(uint64_t seed, uint64_t row, uint32_t stage,
                                               uint32_t draw, double* n0, double* n1) {
    double u0, u1;
    philox_uniform2(seed, row, stage, draw, &u0, &u1);
    double r = sqrt(-2.0 * log(1.0 - u0));   // 1-u0 in (0, 1]
    double s, c;
    sincospi(2.0 * u1, &s, &c);
    *n0 = r * c;
    *n1 = r * s;
}

// ---------------------------------------------------------------------------
// Degree-1 tensor spline as scipy's RectBivariateSpline(kx=1, ky=1).ev
// evaluates it (FITPACK fpbisp + fpbspl): the argument is clamped to
// [t[1], t[n-2]] (a NaN stays NaN), the interval l is the first one with
// arg < t[l+1], capped at n-3, the weights are f (t[l+1] - arg) and
// f (arg - t[l]) with f = 1 / (t[l+1] - t[l]), and the value is
// sum over the 2x2 coefficients of (c * hx) * hy, x-major, added to 0 in that
// order.  Multiplies and adds are issued unfused so the result is the one
// the float64 reference computes.
struct Spline1W {
    int base;
    double hx0, hx1, hy0, hy1;
};

__device__ __forceinline__ void spline1_axis(const double* t, int n, double a, int& l, double& h0,
                                             double& h1) {
    double arg = a;
    if (arg < t[1]) arg = t[1];
    if (arg > t[n - 2]) arg = t[n - 2];
    // first j in [2, n-2] with t[j] > arg (n-1 when none); l = j - 1, at most n - 3
    int lo = 2, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (t[mid] > arg) hi = mid;
        else lo = mid + 1;
    }
    l = lo - 1;
    if (l > n - 3) l = n - 3;
    const double f = 1.0 / (t[l + 1] - t[l]);
    h0 = __dmul_rn(f, t[l + 1] - arg);
    h1 = __dmul_rn(f, arg - t[l]);
}

__device__ __forceinline__ Spline1W spline1_weights(const mgpu_spline1& S, double x, double y) {
    Spline1W w;
    int lx, ly;
    spline1_axis(S.tx, S.nx, x, lx, w.hx0, w.hx1);
    spline1_axis(S.ty, S.ny, y, ly, w.hy0, w.hy1);
    w.base = (lx - 1) * (S.ny - 2) + (ly - 1);
    return w;
}

__device__ __forceinline__ double spline1_value(const mgpu_spline1& S, int s, const Spline1W& w) {
    const int nky1 = S.ny - 2;
    const double* c = S.c + (size_t)s * (size_t)(S.nx - 2) * (size_t)nky1 + w.base;
    double sp = 0.0;
    sp = __dadd_rn(sp, __dmul_rn(__dmul_rn(c[0], w.hx0), w.hy0));
    sp = __dadd_rn(sp, __dmul_rn(__dmul_rn(c[1], w.hx0), w.hy1));
    sp = __dadd_rn(sp, __dmul_rn(__dmul_rn(c[nky1], w.hx1), w.hy0));
    sp = __dadd_rn(sp, __dmul_rn(__dmul_rn(c[nky1 + 1], w.hx1), w.hy1));
    return sp;
}

// spline surface 0 at (x, y)
__device__ __forceinline__ double spline1_at(const mgpu_spline1& S, double x, double y) {
    return spline1_value(S, 0, spline1_weights(S, x, y));
}

// h c in keV nm, the factor of astropy's spectral() keV -> nm conversion
#define MGPU_HC_KEV_NM 1.2398419843320026

// InterpolateEfficiencyTable.__call__ (missions/mitsnl/catgrating.py:101-144):
// each order's spline at (wavelength nm, blaze rad); total = their sum in
// order; the chosen index is the first whose running sum / total exceeds u
// (numpy argmax: index 0 when none does); the probability factor is total.
__device__ __forceinline__ int select_order_spline(const mgpu_selector& sel, double energy,
                                                   double blaze, double u, double* prob) {
    const double wave = MGPU_HC_KEV_NM / energy;
    const Spline1W w = spline1_weights(sel.spline, wave, blaze);
    double total = 0.0;
    for (int k = 0; k < sel.n_orders; ++k) total = __dadd_rn(total, spline1_value(sel.spline, k, w));
    double cum = 0.0;
    int pick = -1;
    for (int k = 0; k < sel.n_orders && pick < 0; ++k) {
        cum = __dadd_rn(cum, spline1_value(sel.spline, k, w));
        if (cum / total > u) pick = k;
    }
    *prob = total;
    return sel.orders[pick < 0 ? 0 : pick];
}

// np.interp / scipy interp1d (linear, equal results): largest j <= n - 2
// with x[j] <= v, slope (y[j+1] - y[j]) / (x[j+1] - x[j]),
// slope * (v - x[j]) + y[j]; the last knot maps to y[n-1]; outside the
// table interp1d raises (status bit, NaN)
__device__ __forceinline__ double np_interp(const double* x, const double* y, int n, double v, uint32_t* status) {
    if (!(v >= x[0] && v <= x[n - 1])) {
        atomicOr(status, MGPU_STATUS_TABLE_RANGE);
        return kNaN;
    }
    if (v == x[n - 1]) return y[n - 1];
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (x[mid] <= v) lo = mid;
        else hi = mid;
    }
    double slope = (y[lo + 1] - y[lo]) / (x[lo + 1] - x[lo]);
    return __dadd_rn(__dmul_rn(slope, v - x[lo]), y[lo]);
}
