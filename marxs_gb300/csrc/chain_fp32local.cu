// Fused element-chain kernel, FP32-local precision mode.
//
// Same stage semantics as the float64 kernel (chain_fp64.cu, which follows
// OpticalElement.process_photons, optics/base.py:149-211), with the
// arithmetic split by what each quantity needs:
//   * photon positions are float-float (hi + lo) in the global frame, so a
//     ray is re-centred on each element exactly (pos - centre) and the
//     element's own arithmetic runs in float32 on small local numbers: the
//     intersection's local offset is formed inside FMAs, where the large
//     parts of (pos - centre) and k dir cancel exactly, and the parameter k
//     is refined once against the element so the stored position lies on it
//     (the float32 solve alone leaves it ~1e-7 k off along the ray);
//   * directions, polarization, probability and local coordinates are
//     float32 (the lean fixed chains keep the probability in float64: it
//     only meets the efficiency table's total there, one float64 multiply
//     instead of two conversions); the grating term m * lambda / d is
//     formed in float-float;
//   * the cylinder hit is solved in float32 around the tabulated reference
//     point at the nearest angle k/1024 (global float-float point, radial
//     and tangential unit vectors): one Newton step on the small offset from
//     that point, and det_phi = k/1024 + a small float32 residual angle, so
//     det_phi keeps ~1e-11 rad;
//   * order selection is exact: a 53-bit draw U against integer thresholds
//     ceil(cdf * 2^53); the nearest energy row by integer keys against the
//     rows' float64 midpoints (made on the host);
//   * interpolated tables (efficiency splines, lens reflectivity, the L1
//     support transmission) and the CAT stack layers run in float32 /
//     float-float from host-made float constants.
// The float64 positions are converted on the integer pipe (mgpu_bits.cuh),
// the other inputs by the FP64 pipe's conversion instructions (this split
// measured faster than either pipe alone), the outputs on the integer pipe
// with one float64 add per float-float value; in Philox mode no other float64
// arithmetic runs, except the float64 scan of an energy table whose rows
// are not increasing.
//
// The kernel is issue-bound (one photon per thread), and instruction fetch
// is a large part of it: each fixed
// stage sequence gets its own kernel with the stage kinds and constants
// compiled in, and the plain ones ("lean") compile only the common element
// configuration (no lens reflectivity table; one sorted, guided efficiency
// table per grating array; no host-evaluated columns), which took the CAT
// chain from 90 to 55 KB of code and 6 % of its time; rarely run code
// (large-angle sines, the reflection form of the polarization transport)
// stays out of line.  Other configurations of the same stage sequences run
// the fixed chains compiled with every path; other sequences the generic
// stage loop.
// Photon i of a column is addressed with 32-bit offsets (launches of at
// most 2^30 photons).
#include <cuda_runtime.h>
#include <utility>
#include "mgpu_ff.cuh"

// branch hints: cold paths (misses, status flags, the brute-force scan) are
// laid out away from the hot instruction stream
#define MGPU_LIKELY(x) __builtin_expect(!!(x), 1)
#define MGPU_UNLIKELY(x) __builtin_expect(!!(x), 0)

namespace {

// block size and the minimum resident blocks per SM the register
// allocation is bounded for (compile-time; see the launch below): 4 blocks
// of 256 (64 registers) for the fixed plain chains, 3 (80 registers) for
// the generic and the CAT-stack chains, which spill at 64
#ifndef MGPU_FP32L_THREADS
#define MGPU_FP32L_THREADS 256
#endif
#ifndef MGPU_FP32L_MIN_BLOCKS
#define MGPU_FP32L_MIN_BLOCKS 4
#endif
#ifndef MGPU_FP32L_MIN_BLOCKS_WIDE
#define MGPU_FP32L_MIN_BLOCKS_WIDE 3
#endif
// grid cap in blocks of 256 threads per SM (0: one block per 256 photons)
#ifndef MGPU_FP32L_GRID_PER_SM
#define MGPU_FP32L_GRID_PER_SM 0
#endif
constexpr int kThreads = MGPU_FP32L_THREADS;
constexpr int kMinBlocks = MGPU_FP32L_MIN_BLOCKS;
constexpr int kMinBlocksWide = MGPU_FP32L_MIN_BLOCKS_WIDE;
constexpr int kGridPerSm = MGPU_FP32L_GRID_PER_SM;

struct PhotonL {
    ff3 pos;
    f3 dir, pol;
    ff energy;
    double energy_d;
    float prob;
    double prob_d;   // lean fixed chains: the probability in float64
    int row0;      // energy row of the first facet stage's selector (-1: not found yet)
};

__device__ __forceinline__ ff3 ldff3(const float* hi, const float* lo) {
    return ff3{ff{hi[0], lo[0]}, ff{hi[1], lo[1]}, ff{hi[2], lo[2]}};
}

// float64 -> float-float: hi = nearest float, lo = the exact residual d - hi
// (exact in float64) rounded to float
__device__ __forceinline__ ff d2ff_hw(double d) {
    const float h = __double2float_rn(d);
    return ff{h, __double2float_rn(d - (double)h)};
}

// element i of a column of stride s (elements).  The launcher keeps
// i < 2^30 and |s| * sizeof(T) < 2^31, so the address is one 32 x 32 ->
// 64-bit multiply-add onto the base pointer.
template <class T>
__device__ __forceinline__ T* at(T* p, int i, int64_t s) {
    return (T*)((uintptr_t)p + (uintptr_t)((int64_t)i * (int64_t)(int)(s * (int64_t)sizeof(T))));
}

// photon columns are written once and not read again by the kernel: stored
// evict-first (st.global.cs) so they do not displace the facet records,
// candidate lists and order tables in L1/L2 (measured 0.6 % faster than
// plain stores on the CAT chain; streaming loads of the inputs gained less)
template <class T>
__device__ __forceinline__ void put(T* p, T v) {
    __stcs(p, v);
}

template <bool kAll = false>
__device__ __forceinline__ void storef(const mgpu_col& c, int i, float v) {
    if (kAll || c.ptr) put(at(c.ptr, i, c.stride), f2d_bits(v));
}
// the same for values that are finite by construction (hit coordinates,
// pixels, angles): no infinity / NaN cases in the conversion
// kAll (the fixed chains): the launcher checked that the column exists,
// so the store needs no test (the tests' uniform branches measured 2.8 % of
// the CAT chain: they split the stages' straight-line code)
template <bool kAll = false>
__device__ __forceinline__ void store_hit(const mgpu_col& c, int i, float v) {
    if (kAll || c.ptr) put(at(c.ptr, i, c.stride), f2d_fin_bits(v));
}
template <bool kAll = false>
__device__ __forceinline__ void stored(const mgpu_col& c, int i, double v) {
    if (kAll || c.ptr) put(at(c.ptr, i, c.stride), v);
}

__device__ __forceinline__ void store_id(const mgpu_stage& st, int i, int64_t v) {
    if ((st.first_writer >> 17) & 1) put(at((long long*)st.id_out, i, st.id_stride), (long long)v);
    else put(at((int*)st.id_out, i, st.id_stride), (int)v);
}

// 3-vector columns: component c of photon i at ptr + c * cstride, stride s
__device__ __forceinline__ d3 load3i(const mgpu_vec& v, int i) {
    return d3{*at(v.ptr, i, v.stride), *at(v.ptr + v.cstride, i, v.stride),
              *at(v.ptr + 2 * v.cstride, i, v.stride)};
}
__device__ __forceinline__ void store3i(const mgpu_vec& v, int i, d3 a) {
    put(at(v.ptr, i, v.stride), a.x);
    put(at(v.ptr + v.cstride, i, v.stride), a.y);
    put(at(v.ptr + 2 * v.cstride, i, v.stride), a.z);
}

__device__ __forceinline__ void write_miss_defaults(const mgpu_stage& st, int i, int nout) {
#pragma unroll 1
    for (int k = 0; k < nout; ++k)
        if ((st.first_writer >> k) & 1) stored(st.out[k], i, kNaN);
    if (st.id_out && ((st.first_writer >> 16) & 1)) store_id(st, i, -1);
}

// ------------------------------------------------------------ flat planes
struct HitL {
    bool hit;
    float k;
    ff3 ip;      // intersection point, global (float-float)
    f3 v;        // intersection point - element centre
    f3 r0;       // ray start - element centre
    float ly, lz;
};

// FinitePlane.intersect in the element frame.  The ray start is re-centred
// once on the element (pos - c as an unnormalised pair s + e, exact to
// ~2^-46); the parameter k comes from a float32 solve, and the local offset
// v = (s + k dir) + e is formed inside FMAs, where the large parts of s and
// k dir cancel exactly, so v carries only its own rounding (~2^-24 |v|)
// plus an offset along the ray from the error of k, which one refinement
// against the plane removes.  The global point is c + v in float-float.
__device__ __forceinline__ HitL plane_hit_l(ff3 c, f3 n, f3 ey, f3 ez, float hy, float hz,
                                            const ff3& pos, f3 dir) {
    HitL h;
    f3 s, e;
    ff3_rel(pos, c, s, e);
    const float kd = dotf(dir, n);
    float k = -(dotf(s, n) + dotf(e, n)) / kd;
    f3 v{fmaf(k, dir.x, s.x) + e.x, fmaf(k, dir.y, s.y) + e.y, fmaf(k, dir.z, s.z) + e.z};
    const float dk = -dotf(v, n) / kd;
    if (MGPU_LIKELY(isfinite(dk))) {
        k += dk;
        v = f3{fmaf(dk, dir.x, v.x), fmaf(dk, dir.y, v.y), fmaf(dk, dir.z, v.z)};
    }
    h.k = k;
    h.v = v;
    h.r0 = s + e;
    h.ip = ff3{ff_add_f(c.x, v.x), ff_add_f(c.y, v.y), ff_add_f(c.z, v.z)};
    h.ly = dotf(v, ey);
    h.lz = dotf(v, ez);
    h.hit = (kd != 0.0f) && (k >= 0.0f) && (fabsf(h.ly) <= hy) && (fabsf(h.lz) <= hz);
    return h;
}

__device__ __forceinline__ HitL flat_hit(const mgpu_flat32* F, const ff3& pos, f3 dir) {
    return plane_hit_l(ldff3(F->c_hi, F->c_lo), ldf3(F->ex), ldf3(F->ey), ldf3(F->ez), F->hy, F->hz,
                       pos, dir);
}

// the plane of an FP32-local facet record, from its first five float4 rows
struct FacetPlane {
    ff3 c;
    f3 n, ey, ez;
    float hy, hz;
};
__device__ __forceinline__ const float4* facet_rows(const mgpu_facet32* fc) {
    return reinterpret_cast<const float4*>(fc);
}
__device__ __forceinline__ ff3 facet_centre(const mgpu_facet32* fc) {
    const float4 A = __ldg(facet_rows(fc)), B = __ldg(facet_rows(fc) + 1);
    return ff3{ff{A.x, B.x}, ff{A.y, B.y}, ff{A.z, B.z}};
}
__device__ __forceinline__ FacetPlane facet_plane(const mgpu_facet32* fc) {
    const float4* r = facet_rows(fc);
    const float4 A = __ldg(r), B = __ldg(r + 1), E = __ldg(r + 2), D = __ldg(r + 3);
    const float G = __ldg(reinterpret_cast<const float*>(r + 4));
    FacetPlane P;
    P.c = ff3{ff{A.x, B.x}, ff{A.y, B.y}, ff{A.z, B.z}};
    P.hy = A.w;
    P.hz = B.w;
    P.n = f3{E.x, E.y, E.z};
    P.ey = f3{E.w, D.x, D.y};
    P.ez = f3{D.z, D.w, G};
    return P;
}

__device__ __forceinline__ HitL facet_hit(const mgpu_facet32* fc, const ff3& pos, f3 dir) {
    const FacetPlane P = facet_plane(fc);
    return plane_hit_l(P.c, P.n, P.ey, P.ez, P.hy, P.hz, pos, dir);
}

// parallel_transport (polarization.py:90-170) in float32 for a turn of the
// direction from a to b (any lengths), given ax = a x b: the rotation about
// a x b that takes a to b maps the frame (s, a x s, a) of the reference onto
// (s, b x s, b).  Below 90 degrees in the Rodrigues form
//   pol cos t + w x pol + w (w . pol) / (1 + cos t),  w = a x b / (|a| |b|),
// beyond it through the frame, where 1 + cos t loses its precision;
// |a x b| <= 1e-8 |a| |b| leaves pol unchanged.  The frame form (turns of
// 90 degrees or more: reflections) is out of line, away from the hot code.
__device__ __noinline__ f3 transport_frame_f(f3 a, f3 b, f3 ax, f3 pol, float n0, float n1, float ss) {
    const f3 s = rsqrtf(ss) * ax;
    const f3 an = rsqrtf(n0) * a, bn = rsqrtf(n1) * b;
    const f3 pin = crossf(an, s), pout = crossf(bn, s);
    const float ks = dotf(s, pol), kp = dotf(pin, pol), kd = dotf(an, pol);
    return f3{s.x * ks + pout.x * kp + bn.x * kd, s.y * ks + pout.y * kp + bn.y * kd,
              s.z * ks + pout.z * kp + bn.z * kd};
}
__device__ __forceinline__ f3 transport_axis_f(f3 a, f3 b, f3 ax, f3 pol) {
    const float n0 = dotf(a, a), n1 = dotf(b, b);
    const float ss = dotf(ax, ax);
    if (MGPU_UNLIKELY(!(ss > 1e-16f * n0 * n1))) return pol;
    const float r = rsqrtf(n0 * n1);
    const float c = dotf(a, b) * r;
    if (MGPU_LIKELY(c > 0.0f)) {
        const f3 w = r * ax;
        const f3 wp = crossf(w, pol);
        const float t = __fdividef(dotf(w, pol), 1.0f + c);
        return f3{fmaf(c, pol.x, fmaf(w.x, t, wp.x)), fmaf(c, pol.y, fmaf(w.y, t, wp.y)),
                  fmaf(c, pol.z, fmaf(w.z, t, wp.z))};
    }
    return transport_frame_f(a, b, ax, pol, n0, n1, ss);
}

__device__ __forceinline__ f3 transport_f(f3 d_old, f3 d_new, f3 pol) {
    return transport_axis_f(d_old, d_new, crossf(d_old, d_new), pol);
}

// the same for d_new = d_old + delta where the change delta is known
// directly: the axis d_old x delta keeps full relative precision even when
// the two directions are nearly parallel (a float32 cross product of the
// two unit vectors would be dominated by rounding there)
__device__ __forceinline__ f3 transport_delta_f(f3 d_old, f3 delta, f3 pol) {
    return transport_axis_f(d_old, d_old + delta, crossf(d_old, delta), pol);
}

// change of v under R^T v for R = axangle2mat(axis, angle):
// -sin(a) (k x v) + (1 - cos a) k x (k x v), with 1 - cos a = 2 sin^2(a/2)
// so small angles keep full relative precision
// sin for the small scatter angles (|a| < 1e-2: odd polynomial, error below
// a^7/5040 relative), the library sine otherwise, out of line: its
// argument reduction would add ~1.5 KB of rarely run code to each of the
// four inlined rotations (instruction-cache pressure measured 1 % of the
// CAT chain's time)
__device__ __noinline__ float sin_large(float a) { return sinf(a); }
__device__ __forceinline__ float sin_small(float a) {
    if (MGPU_LIKELY(fabsf(a) < 1e-2f)) {
        float a2 = a * a;
        return a * (1.0f - a2 * (1.0f / 6.0f) * (1.0f - a2 * (1.0f / 20.0f)));
    }
    return sin_large(a);
}

__device__ __forceinline__ f3 rot_transpose_delta_f(f3 axis, float a, f3 v) {
    f3 k = normf(axis);
    float s = sin_small(a);
    float h = sin_small(0.5f * a);
    float C = 2.0f * h * h;
    f3 kv = crossf(k, v);
    f3 kkv = crossf(k, kv);
    return f3{-s * kv.x + C * kkv.x, -s * kv.y + C * kkv.y, -s * kv.z + C * kkv.z};
}

// 53-bit uniform as an integer and as float, from the Philox stream the
// float64 kernel uses (same counters, so both modes draw the same u)
__device__ __forceinline__ void philox_u53(uint64_t seed, uint64_t row, uint32_t stage,
                                           uint64_t* U0, uint64_t* U1) {
    u4 c{(uint32_t)row, (uint32_t)(row >> 32), stage, 0u};
    u4 r = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    *U0 = (((uint64_t)r.x << 21) ^ (uint64_t)(r.y >> 11)) & ((1ull << 53) - 1);
    *U1 = (((uint64_t)r.z << 21) ^ (uint64_t)(r.w >> 11)) & ((1ull << 53) - 1);
}

// the same with a draw index (the float64 kernel's philox_uniform2 counters)
__device__ __forceinline__ void philox_u53_draw(uint64_t seed, uint64_t row, uint32_t stage,
                                                uint32_t draw, uint64_t* U0, uint64_t* U1) {
    u4 c{(uint32_t)row, (uint32_t)(row >> 32), stage, draw};
    u4 r = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    *U0 = (((uint64_t)r.x << 21) ^ (uint64_t)(r.y >> 11)) & ((1ull << 53) - 1);
    *U1 = (((uint64_t)r.z << 21) ^ (uint64_t)(r.w >> 11)) & ((1ull << 53) - 1);
}

__device__ __forceinline__ float u53_to_f(uint64_t U) {
    return (float)(uint32_t)(U >> 29) * (1.0f / 16777216.0f);
}

// ------------------------------------------------------------ splines
// Degree-1 spline (the FITPACK evaluation of spline1_at, mgpu_device.cuh)
// in float32: the knots as float-float pairs (tx_ff, ty_ff), the argument
// as float-float, so the interval and the offsets from its knots match the
// float64 evaluation to ~2^-44 relative; the weights and the 2x2
// coefficient sum in float32 (coefficients from the float32 copy).
__device__ __forceinline__ ff knot_ff(const float* t2, int j) {
    return ff{__ldg(t2 + 2 * j), __ldg(t2 + 2 * j + 1)};
}

__device__ __forceinline__ bool ff_gt(ff a, ff b) {
    return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo);
}

__device__ __forceinline__ void spline1_axis_f(const float* t2, int n, ff a, int& l, float& h0,
                                               float& h1) {
    ff arg = a;
    if (!isnan(a.hi)) {
        const ff tb = knot_ff(t2, 1), te = knot_ff(t2, n - 2);
        if (ff_gt(tb, a)) arg = tb;
        else if (ff_gt(a, te)) arg = te;
    }
    int lo = 2, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (ff_gt(knot_ff(t2, mid), arg)) hi = mid;
        else lo = mid + 1;
    }
    l = lo - 1;
    if (l > n - 3) l = n - 3;
    const ff t0 = knot_ff(t2, l), t1 = knot_ff(t2, l + 1);
    const float w = ff_f(ff_sub(t1, t0));
    if (w > 0.0f) {
        const float inv = 1.0f / w;
        h0 = ff_f(ff_sub(t1, arg)) * inv;
        h1 = ff_f(ff_sub(arg, t0)) * inv;
    } else {   // knots closer than float-float resolution
        h0 = 1.0f;
        h1 = 0.0f;
    }
}

struct Spline1Wf {
    int base;
    float hx0, hx1, hy0, hy1;
};

__device__ __forceinline__ Spline1Wf spline1_weights_f(const mgpu_spline1& S, ff x, ff y) {
    Spline1Wf w;
    int lx, ly;
    spline1_axis_f(S.tx_ff, S.nx, x, lx, w.hx0, w.hx1);
    spline1_axis_f(S.ty_ff, S.ny, y, ly, w.hy0, w.hy1);
    w.base = (lx - 1) * (S.ny - 2) + (ly - 1);
    return w;
}

__device__ __forceinline__ float spline1_value_f(const mgpu_spline1& S, int s, const Spline1Wf& w) {
    const int nky1 = S.ny - 2;
    const float* c = S.c32 + (size_t)s * (size_t)(S.nx - 2) * (size_t)nky1 + w.base;
    return fmaf(__ldg(c) * w.hx0, w.hy0,
                fmaf(__ldg(c + 1) * w.hx0, w.hy1,
                     fmaf(__ldg(c + nky1) * w.hx1, w.hy0, __ldg(c + nky1 + 1) * w.hx1 * w.hy1)));
}

// energy2wave (marxs/__init__.py:14) in nm keV as a float-float constant,
// and in mm keV as a float
constexpr float kHcNmHi = (float)MGPU_HC_KEV_NM;
constexpr float kHcNmLo = (float)(MGPU_HC_KEV_NM - (double)kHcNmHi);
constexpr float kHcMm = (float)(MGPU_HC_KEV_NM * 1e-6);
// energy2wave of the grating equation (marxs/__init__.py:14), mm keV, as float-float
constexpr double kE2w = 1.2398419292004202e-06;
constexpr float kE2wHi = (float)kE2w;
constexpr float kE2wLo = (float)(kE2w - (double)kE2wHi);

// InterpolateEfficiencyTable.__call__ (missions/mitsnl/catgrating.py:101-144)
// in float32: the order whose running sum / total first exceeds u (index 0
// when none does); the probability factor is the total
__device__ __forceinline__ int select_order_spline_f(const mgpu_selector& sel, ff energy,
                                                     float blaze, float u, float* prob) {
    const ff wave = ff_div(ff{kHcNmHi, kHcNmLo}, energy);
    const Spline1Wf w = spline1_weights_f(sel.spline, wave, ff{blaze, 0.0f});
    // the total from the summed surface (the last one of the float copy)
    const float total = spline1_value_f(sel.spline, sel.n_orders, w);
    float cum = 0.0f;
    int pick = -1;
    for (int k = 0; k < sel.n_orders && pick < 0; ++k) {
        cum += spline1_value_f(sel.spline, k, w);
        if (cum / total > u) pick = k;
    }
    *prob = total;
    return sel.orders[pick < 0 ? 0 : pick];
}

// ------------------------------------------------------------------ stages
// kLean (the plain fixed chains): the lens has no reflectivity table
template <bool kLean, bool kAll>
__device__ bool stage_lens_l(const mgpu_stage& st, PhotonL& ph, int i, uint32_t* status) {
    // PerfectLens.specific_process_photons, optics/mirror.py:53-82
    const mgpu_flat32* F = reinterpret_cast<const mgpu_flat32*>(st.aux32);
    HitL h = flat_hit(F, ph.pos, ph.dir);
    if (MGPU_UNLIKELY(!h.hit)) {
        write_miss_defaults(st, i, 2);
        return false;
    }
    // focus - interpos = (centre - interpos) - d_off e_z + f norm(dir)
    f3 v = (F->p[0] * normf(ph.dir) - F->p[1] * ldf3(F->ez)) - h.v;
    f3 nd = normf(v);
    if (!kLean && st.spline.n_surf > 0) {
        // probability *= reflectivity_interpolator(E, angle / 4) ** 2 (mirror.py:73-79);
        // the angle from atan2(|a x b|, a . b), accurate for small deflections
        f3 od = normf(ph.dir);
        f3 cr = crossf(od, nd);
        float angle = atan2f(sqrtf(dotf(cr, cr)), fabsf(dotf(od, nd)));
        const Spline1Wf w = spline1_weights_f(st.spline, ph.energy, ff{0.25f * angle, 0.0f});
        float r = spline1_value_f(st.spline, 0, w);
        r = r * r;
        if (MGPU_UNLIKELY(!(r >= 0.0f && r <= 1.0f))) atomicOr(status, MGPU_STATUS_PROB_RANGE);
        ph.prob = ph.prob * r;
    }
    ph.pol = transport_f(ph.dir, nd, ph.pol);
    ph.dir = nd;
    store_hit<kAll>(st.out[0], i, h.ly);
    store_hit<kAll>(st.out[1], i, h.lz);
    ph.pos = h.ip;
    return true;
}

// kAll: every column of the stage exists (fixed chains; checked at launch);
// kLean: both widths are nonzero (checked at launch)
template <bool kAll, bool kLean>
__device__ bool stage_scatter_l(const mgpu_stage& st, PhotonL& ph, int i, int rng,
                                uint64_t seed, uint64_t row_base, int sidx, uint32_t* status) {
    // RadialMirrorScatter.specific_process_photons, optics/scatter.py:49-77
    const mgpu_flat32* F = reinterpret_cast<const mgpu_flat32*>(st.aux32);
    HitL h = flat_hit(F, ph.pos, ph.dir);
    if (MGPU_UNLIKELY(!h.hit)) {
        write_miss_defaults(st, i, 4);
        return false;
    }
    float sig_in = F->p[0], sig_perp = F->p[1];
    float a_in = 0.0f, a_perp = 0.0f;
    double a_in_d = 0.0, a_perp_d = 0.0;
    bool have_d = false;
    if (rng == MGPU_RNG_PREDRAWN) {
        if ((sig_in != 0.0f && st.draw[0] == nullptr) || (sig_perp != 0.0f && st.draw[1] == nullptr)) {
            atomicOr(status, MGPU_STATUS_BAD_STAGE);
            return false;
        }
        if (sig_in != 0.0f) a_in_d = *at(st.draw[0], i, st.draw_stride);
        if (sig_perp != 0.0f) a_perp_d = *at(st.draw[1], i, st.draw_stride);
        a_in = d2f_bits(a_in_d);
        a_perp = d2f_bits(a_perp_d);
        have_d = true;
    } else {
        uint64_t U0, U1;
        philox_u53(seed, row_base + (uint64_t)i, (uint32_t)sidx, &U0, &U1);
        // 1 - u0 formed exactly from the 53-bit integer keeps the normal's
        // tail identical to the float64 path's draw
        float one_minus_u0 = (float)((1ull << 53) - U0) * 1.1102230246251565e-16f;
        float u1 = u53_to_f(U1);
        float r = sqrtf(-2.0f * __logf(one_minus_u0));
        float sn, cs;
        sincospif(2.0f * u1, &sn, &cs);
        a_in = sig_in * (r * cs);
        a_perp = sig_perp * (r * sn);
    }
    const f3 radial = h.r0;   // previous position - centre
    f3 perpplane = crossf(ph.dir, radial);
    f3 delta{0.0f, 0.0f, 0.0f};
    if (kLean || sig_in != 0.0f) delta = rot_transpose_delta_f(perpplane, a_in, ph.dir);
    if (kLean || sig_perp != 0.0f) delta = delta + rot_transpose_delta_f(radial, a_perp, ph.dir + delta);
    ph.pol = transport_delta_f(ph.dir, delta, ph.pol);
    ph.dir = ph.dir + delta;
    store_hit<kAll>(st.out[0], i, h.ly);
    store_hit<kAll>(st.out[1], i, h.lz);
    if (have_d) {
        stored<kAll>(st.out[2], i, a_in_d);
        stored<kAll>(st.out[3], i, a_perp_d);
    } else {
        store_hit<kAll>(st.out[2], i, a_in);
        store_hit<kAll>(st.out[3], i, a_perp);
    }
    ph.pos = h.ip;
    return true;
}

template <bool kAll>
__device__ bool stage_flatdet_l(const mgpu_stage& st, PhotonL& ph, int i) {
    // FlatDetector.specific_process_photons, optics/detector.py:72-75
    const mgpu_flat32* F = reinterpret_cast<const mgpu_flat32*>(st.aux32);
    HitL h = flat_hit(F, ph.pos, ph.dir);
    if (MGPU_UNLIKELY(!h.hit)) {
        write_miss_defaults(st, i, 4);
        return false;
    }
    store_hit<kAll>(st.out[0], i, h.ly);
    store_hit<kAll>(st.out[1], i, h.lz);
    store_hit<kAll>(st.out[2], i, h.ly * F->p[3] + F->p[1]);
    store_hit<kAll>(st.out[3], i, h.lz * F->p[3] + F->p[2]);
    if (st.id_out) store_id(st, i, st.id_num);
    ph.pos = h.ip;
    return true;
}

// phi_lim test of a point (x, y) of the cylinder's (e1, e2) plane against
// the borders as unit vectors w1, w2 (angle_between, math/utils.py:180-215,
// as half-plane tests: the arc from w1 counter-clockwise to w2 is the
// intersection of two half-planes when it spans at most pi, their union
// otherwise)
__device__ __forceinline__ bool in_arc(const mgpu_cyl32* K, float x, float y) {
    const bool s1 = K->w1[0] * y - K->w1[1] * x >= 0.0f;     // w1 x p >= 0
    const bool s2 = x * K->w2[1] - y * K->w2[0] >= 0.0f;     // p x w2 >= 0
    return K->arc == 2 || (K->arc == 0 ? (s1 && s2) : (s1 || s2));
}

// angle of (x, y) to within 8.3e-5 rad: octant reduction and an odd
// least-squares polynomial of atan on [0, 1] (fitted here, 4 terms).  It
// only picks the tabulated reference point of the cylinder solve, where a
// neighbouring one serves as well
__device__ __forceinline__ float angle_coarse(float y, float x) {
    const float ax = fabsf(x), ay = fabsf(y);
    const float r = __fdividef(fminf(ax, ay), fmaxf(ax, ay));
    const float r2 = r * r;
    float a = r * fmaf(fmaf(fmaf(-0.038997583f, r2, 0.14628096f), r2, -0.32118174f), r2, 0.99921447f);
    if (ay > ax) a = 1.5707964f - a;
    if (x < 0.0f) a = 3.1415927f - a;
    return copysignf(a, y);
}

template <bool kAll>
__device__ bool stage_cyldet_l(const mgpu_stage& st, PhotonL& ph, int i) {
    // Cylinder.intersect (math/geometry.py:470-564) + CircularDetector
    // (optics/detector.py:115-118) for a circular tube
    const mgpu_cyl32* K = reinterpret_cast<const mgpu_cyl32*>(st.aux32);
    const f3 e1 = ldf3(K->e1), e2 = ldf3(K->e2), ax = ldf3(K->a);
    const float R = K->R;
    // approximate root in float32 from q = pos - c (error ~1e-3 mm from the
    // cancellation in c at |q_perp| ~ R; the Newton step below removes it)
    f3 qs, qe;
    ff3_rel(ph.pos, ldff3(K->c_hi, K->c_lo), qs, qe);
    const f3 qf = qs + qe;
    const float q1 = dotf(qf, e1), q2 = dotf(qf, e2), q3 = dotf(qf, ax);
    const f3 d = ph.dir;
    const float d1 = dotf(d, e1), d2 = dotf(d, e2), d3 = dotf(d, ax);
    const float a = d1 * d1 + d2 * d2;
    const float b = q1 * d1 + q2 * d2;                              // half of the linear term
    const float c = (q1 - R) * (q1 + R) + q2 * q2;
    const float disc = b * b - a * c;
    bool hit = false;
    float t = 0.0f;
    if (MGPU_LIKELY(disc >= 0.0f && a > 0.0f)) {
        const float sq = sqrtf(disc);
        const float qq = -(b + copysignf(sq, b));
        const float tA = qq / a, tB = c / qq;
        const float a1 = (b < 0.0f) ? tA : tB;     // (-b + sq) / a
        const float a2 = (b < 0.0f) ? tB : tA;     // (-b - sq) / a
        bool h1 = (a1 >= 0.0f) && (fabsf(q3 + a1 * d3) <= K->Rz) &&
                  in_arc(K, q1 + a1 * d1, q2 + a1 * d2);
        bool h2 = (a2 >= 0.0f) && (fabsf(q3 + a2 * d3) <= K->Rz) &&
                  in_arc(K, q1 + a2 * d1, q2 + a2 * d2);
        if (h1 && h2) {
            if (a2 < a1) h1 = false;
            else h2 = false;
        }
        hit = h1 || h2;
        t = h1 ? a1 : a2;
    }
    if (MGPU_UNLIKELY(!hit)) {
        write_miss_defaults(st, i, 4);
        return false;
    }
    // reference point P_k = c + R u_k on the cylinder at the angle k/1024
    // nearest the approximate hit; table row: (P_k hi, u.x), (P_k lo, u.y),
    // (tangent t_k, u.z), P_k global
    int kk = __float2int_rn(angle_coarse(q2 + t * d2, q1 + t * d1) * 1024.0f);
    const int idx = min(max(kk - K->k0, 0), K->nk - 1);
    kk = idx + K->k0;
    const float4* tb = reinterpret_cast<const float4*>(st.table) + 3 * idx;
    const float4 T0 = __ldg(tb), T1 = __ldg(tb + 1), T2 = __ldg(tb + 2);
    const ff3 P{ff{T0.x, T1.x}, ff{T0.y, T1.y}, ff{T0.z, T1.z}};
    const f3 u{T0.w, T1.w, T2.w}, tg{T2.x, T2.y, T2.z};
    // w = pos + t d - P_k, a few mm: the large parts cancel inside the FMAs
    f3 ws, we;
    ff3_rel(ph.pos, P, ws, we);
    f3 w{fmaf(t, d.x, ws.x) + we.x, fmaf(t, d.y, ws.y) + we.y, fmaf(t, d.z, ws.z) + we.z};
    float wu = dotf(w, u), wt = dotf(w, tg), wa = dotf(w, ax);
    // one Newton step along the ray on |R u_k + w_perp|^2 = R^2:
    // g = wu (2R + wu) + wt^2, g' = 2 ((R + wu) d.u + wt d.t)
    const float du = dotf(d, u), dtg = dotf(d, tg);
    const float g = fmaf(wu, 2.0f * R + wu, wt * wt);
    const float dt = -g / (2.0f * fmaf(R + wu, du, wt * dtg));
    if (MGPU_LIKELY(isfinite(dt))) {
        w = f3{fmaf(dt, d.x, w.x), fmaf(dt, d.y, w.y), fmaf(dt, d.z, w.z)};
        wu = fmaf(dt, du, wu);
        wt = fmaf(dt, dtg, wt);
        wa = fmaf(dt, d3, wa);
    }
    // det_phi = k/1024 + atan(wt / (R + wu)); |ratio| < 6e-4 (5.8e-4 with
    // the coarse angle's error), so two terms of the series (next term
    // r^5/5 < 2e-17)
    const float r = wt / (R + wu);
    const float psi = fmaf(-(1.0f / 3.0f) * r * r, r, r);
    const ff phi = fast_two_sum((float)kk * (1.0f / 1024.0f), psi);
    stored<kAll>(st.out[0], i, f2d_fin_bits(phi.hi) + f2d_fin_bits(phi.lo));
    store_hit<kAll>(st.out[1], i, wa);                // P_k - c is perpendicular to the axis
    const ff px = ff_add_f(ff_mul(phi, ff{K->rpix_hi, K->rpix_lo}), K->cp0);
    stored<kAll>(st.out[2], i, f2d_fin_bits(px.hi) + f2d_fin_bits(px.lo));
    store_hit<kAll>(st.out[3], i, wa * K->inv_pix + K->cp1);
    if (st.id_out) store_id(st, i, st.id_num);
    ph.pos = ff3{ff_add_f(P.x, w.x), ff_add_f(P.y, w.y), ff_add_f(P.z, w.z)};
    return true;
}

// exact order selection (see the header comment): the energy row of the
// table for photon energy e (float64; ef its float32 value)
// kLean: the rows are sorted and carry their midpoints (checked at launch)
template <bool kLean = false>
__device__ __forceinline__ int energy_row(const mgpu_selector& sel, double e, float ef) {
    int row = 0;
    if (kLean || sel.by_energy) {
        const int n = sel.n_rows;
        if (kLean || sel.sorted) {
            // largest j with E_j <= e (positive doubles order as integers)
            long long key = __double_as_longlong(e);
            const double e0 = sel.energy[0], e1 = sel.energy[n - 1];
            if (!(key >= __double_as_longlong(e0))) {
                row = 0;
            } else {
                // guess from a uniform grid, then step to the largest j with E_j <= e
                const float g = (kLean || sel.e_mid) ? (ef - sel.e0_f) * sel.e_scale_f
                                          : __fdividef((float)(e - e0), (float)(e1 - e0)) *
                                                (float)(n - 1);
                int lo = min(max((int)g, 0), n - 1);
                while (lo + 1 < n && __double_as_longlong(sel.energy[lo + 1]) <= key) ++lo;
                while (lo > 0 && __double_as_longlong(sel.energy[lo]) > key) --lo;
                row = lo;
                if (row + 1 < n) {
                    // the nearer row: past the midpoint (integer keys), or |E - e| in float64
                    if (kLean || sel.e_mid) {
                        if (key > __double_as_longlong(sel.e_mid[row])) row = row + 1;
                    } else {
                        double d0 = fabs(sel.energy[row] - e), d1 = fabs(sel.energy[row + 1] - e);
                        if (d1 < d0) row = row + 1;
                    }
                }
            }
        } else {
            double best = fabs(sel.energy[0] - e);
            for (int j = 1; j < n; ++j) {
                double dd = fabs(sel.energy[j] - e);
                if (dd < best) {
                    best = dd;
                    row = j;
                }
            }
        }
    }
    return row;
}

// the order for the draw U (53 bits) in table row `row`; *prob the row's
// total (in float64 into *prob_d instead, when given).  kLean: the selector
// has its guide table (checked at launch)
template <bool kLean = false>
__device__ __forceinline__ int select_order_row(const mgpu_selector& sel, int row, uint64_t U,
                                                float* prob, uint32_t* status, double* prob_d = nullptr) {
    const uint64_t* th = sel.thresholds + (int64_t)row * sel.n_orders;
    int k = 0;
    if (kLean || sel.guide) {
        // start at the first order of the draw's 1/64 bin, then step
        k = __ldg(sel.guide + row * 64 + (int)(U >> 47));
        while (k < sel.n_orders && !(U < th[k])) ++k;
    } else if (sel.sorted) {
        int hi = sel.n_orders;
        while (k < hi) {
            int mid = (k + hi) >> 1;
            if (U < th[mid]) hi = mid;
            else k = mid + 1;
        }
    } else {
        while (k < sel.n_orders && !(U < th[k])) ++k;
    }
    if (MGPU_UNLIKELY(k == sel.n_orders)) {
        atomicOr(status, MGPU_STATUS_ORDER_EMPTY);
        k = sel.n_orders - 1;
    }
    double tot = sel.total[row];
    if (prob_d) *prob_d = tot;
    else *prob = d2f_bits(tot);
    if (MGPU_UNLIKELY(tot < 0.0 || tot > 1.0)) atomicOr(status, MGPU_STATUS_PROB_RANGE);
    return sel.orders[k];
}

__device__ __forceinline__ int select_order_l(const mgpu_selector& sel, double e, float ef,
                                              uint64_t U, float* prob, uint32_t* status) {
    return select_order_row(sel, energy_row(sel, e, ef), U, prob, status);
}

// photons the grid cannot bound (slope beyond the grid's limit): the whole
// warp scans all facets for each of them, one photon at a time, with a warp
// min-reduction on (k, facet).  (Inlined: an out-of-line call spills at 64
// registers and measured slower.)
__device__ __forceinline__ int brute_force_nearest(const mgpu_stage& st, ff3 pos, f3 dir, unsigned bm) {
    const int lane = threadIdx.x & 31;
    int mine = -1;
    while (bm) {
        int src = __ffs(bm) - 1;
        bm &= bm - 1;
        ff3 p;
        p.x = ff{__shfl_sync(MGPU_FULL_MASK, pos.x.hi, src), __shfl_sync(MGPU_FULL_MASK, pos.x.lo, src)};
        p.y = ff{__shfl_sync(MGPU_FULL_MASK, pos.y.hi, src), __shfl_sync(MGPU_FULL_MASK, pos.y.lo, src)};
        p.z = ff{__shfl_sync(MGPU_FULL_MASK, pos.z.hi, src), __shfl_sync(MGPU_FULL_MASK, pos.z.lo, src)};
        f3 d{__shfl_sync(MGPU_FULL_MASK, dir.x, src), __shfl_sync(MGPU_FULL_MASK, dir.y, src),
             __shfl_sync(MGPU_FULL_MASK, dir.z, src)};
        float bk = 0.0f;
        int bf = -1;
        for (int q = lane; q < st.n_facets; q += 32) {
            HitL hq = facet_hit(st.facets32 + q, p, d);
            if (hq.hit && (bf < 0 || hq.k < bk)) {
                bf = q;
                bk = hq.k;
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            float ok = __shfl_xor_sync(MGPU_FULL_MASK, bk, off);
            int of = __shfl_xor_sync(MGPU_FULL_MASK, bf, off);
            bool take = (of >= 0) && (bf < 0 || ok < bk || (ok == bk && of < bf));
            if (take) {
                bk = ok;
                bf = of;
            }
        }
        if (lane == src) mine = bf;
    }
    return mine;
}

// the candidate range [*s0, *s1) of the photon's grid cell in cell_items;
// *brute: the grid cannot bound the ray (slope beyond its limit, or no grid)
__device__ __forceinline__ void grid_cell_range(const mgpu_stage& st, const PhotonL& ph, bool valid,
                                                int* s0, int* s1, bool* brute) {
    const mgpu_grid32* G = reinterpret_cast<const mgpu_grid32*>(st.aux32);
    *s0 = *s1 = 0;
    *brute = false;
    if (!valid) return;
    if (MGPU_UNLIKELY(G == nullptr || st.grid.cell_start == nullptr)) {
        *brute = true;
        return;
    }
    f3 rs, re;
    ff3_rel(ph.pos, ldff3(G->o_hi, G->o_lo), rs, re);
    const f3 rel = rs + re;
    f3 n = ldf3(G->n), a = ldf3(G->a), b = ldf3(G->b);
    float dn = dotf(ph.dir, n), da = dotf(ph.dir, a), db = dotf(ph.dir, b);
    if (MGPU_UNLIKELY(!(fabsf(da) <= G->slope_max * fabsf(dn)) || !(fabsf(db) <= G->slope_max * fabsf(dn)) ||
                      dn == 0.0f)) {
        *brute = true;
        return;
    }
    const float rdn = 1.0f / dn;
    const float t0 = -dotf(rel, n) * rdn;
    float u = dotf(rel, a) + t0 * da;
    float v = dotf(rel, b) + t0 * db;
    // looked up where the ray meets the depth model of the facet surface
    const float* dq = G->depth;
    const float D = dq[0] + u * (dq[1] + dq[3] * u + dq[4] * v) + v * (dq[2] + dq[5] * v);
    u = fmaf(da * rdn, D, u);
    v = fmaf(db * rdn, D, v);
    float fu = floorf((u - G->u0) * G->inv_cell);
    float fv = floorf((v - G->v0) * G->inv_cell);
    if (MGPU_UNLIKELY(!(fu >= 0.0f && fu < (float)G->nu && fv >= 0.0f && fv < (float)G->nv))) return;
    int cell = (int)fu * G->nv + (int)fv;
    const mgpu_grid& g = st.grid;
    *s0 = __ldg(g.cell_start + cell);
    *s1 = min(__ldg(g.cell_start + cell + 1), g.capacity);
}

// nearest facet: every candidate of the photon's grid cell gets the full
// FP32-local plane test (re-centring, float32 solve, one refinement), the
// nearest hit (smallest k, then lowest index) keeps its local offset, so the
// winner needs no second test; its global point is c + v.  Photons the grid
// cannot bound take the warp's brute-force scan, whose winner then runs
// through the same candidate test (one code path for the hit record).
__device__ __forceinline__ int nearest_facet_l(const mgpu_stage& st, const PhotonL& ph, bool valid,
                                               HitL* best_hit) {
    int s0, s1;
    bool brute;
    grid_cell_range(st, ph, valid, &s0, &s1, &brute);
    const unsigned bm = __ballot_sync(MGPU_FULL_MASK, brute);
    int bf = -1;
    if (MGPU_UNLIKELY(bm != 0)) {
        bf = brute_force_nearest(st, ph.pos, ph.dir, bm);
        if (brute) {
            s0 = 0;
            s1 = bf >= 0 ? 1 : 0;
        }
    }
    int best = -1;
    best_hit->k = 0.0f;
    for (int q = s0; q < s1; ++q) {
        const int f = brute ? bf : __ldg(st.grid.cell_items + q);
        const HitL h = facet_hit(st.facets32 + f, ph.pos, ph.dir);
        if (h.hit && (best < 0 || h.k < best_hit->k || (h.k == best_hit->k && f < best))) {
            best = f;
            best_hit->k = h.k;
            best_hit->v = h.v;
            best_hit->ly = h.ly;
            best_hit->lz = h.lz;
        }
    }
    return best;
}

// order-preserving integer key of a float64 (all finite values and
// infinities; NaN sorts above +inf)
__device__ __forceinline__ uint64_t order_key(double x) {
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// np.interp (the L1 support transmission) with the interval found on the
// float64 table's integer keys and the interpolation in float32 from the
// float copies; outside the table: NaN and MGPU_STATUS_TABLE_RANGE, as the
// float64 np_interp
__device__ __forceinline__ float np_interp_f(const double* x, const float* x32, const float* y32,
                                             int n, double v, float vf, uint32_t* status) {
    const uint64_t kv = order_key(v);
    if (!(kv >= order_key(x[0]) && kv <= order_key(x[n - 1]))) {
        atomicOr(status, MGPU_STATUS_TABLE_RANGE);
        return __int_as_float(0x7fc00000);
    }
    if (kv == order_key(x[n - 1])) return y32[n - 1];
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (order_key(x[mid]) <= kv) lo = mid;
        else hi = mid;
    }
    const float w = x32[lo + 1] - x32[lo];
    if (!(w > 0.0f)) return y32[lo];
    return fmaf((y32[lo + 1] - y32[lo]) / w, vf - x32[lo], y32[lo]);
}

// CATL1L2Stack layers after the membrane (missions/mitsnl/catgrating.py):
// QualityFactor (:160-161), L1 (:196-207), L2Abs (:231-245), L2Diffraction
// (:263-268) through RandomGaussianScatter (optics/scatter.py:109-150), in
// FP32-local arithmetic: direction changes formed directly (the L1 grating
// as the membrane, the L2 turn as two small rotations), probabilities and
// the support transmission in float32 from host-made float constants, no
// float64 arithmetic.  ``support``: the support draw exceeded the open
// fraction.  Inlined into the stacked-chain kernels only (kStack), which
// then fit 80 registers without spills.
template <bool kAll>
__device__ __forceinline__ void cat_stack_layers_l(const mgpu_stage& st, const mgpu_catstack& K,
                                                int f, int m, float ly, float lz, uint64_t U1,
                                                bool support, float z_l2, float u_phi,
                                                PhotonL& ph, int i, uint32_t* status) {
    const mgpu_facet32* fc = st.facets32 + f;
    const f3 n = ldf3(fc->ex);
    // QualityFactor: factor ** (order ** 2)
    const float q = powf(K.qf32, (float)(m * m));
    if (MGPU_UNLIKELY(!(q >= 0.0f && q <= 1.0f))) atomicOr(status, MGPU_STATUS_PROB_RANGE);
    ph.prob *= q;
    // L1: a CAT grating with grooves at pi/2, or the support bars
    const float* lv = K.l1_vec32 + 6 * (int64_t)f;
    const f3 l1{__ldg(lv), __ldg(lv + 1), __ldg(lv + 2)};
    const f3 d1{__ldg(lv + 3), __ldg(lv + 4), __ldg(lv + 5)};
    const f3 p = normf(ph.dir);
    const float p_l = dotf(p, l1), p_d = dotf(p, d1), p_n = dotf(p, n);
    const float blaze1 = atan2f(fabsf(p_d), fabsf(p_n));       // = arccos|p_perp . n|
    float prob1;
    int m1 = select_order_l(st.selectors[K.l1_selector], ph.energy_d, ph.energy.hi, U1, &prob1,
                            status);
    if (support) {
        m1 = 0;
        prob1 = np_interp_f(K.l1_trans_e, K.l1_trans_e32, K.l1_trans_t32, K.l1_n_trans,
                            ph.energy_d, ph.energy.hi, status);
    } else if (m1 != 0) {
        const float sign = (p_d > 0.0f) ? 1.0f : ((p_d < 0.0f) ? -1.0f : 1.0f);
        // sign * m * lambda / d in float-float
        ff term = ff_div(ff{K.l1_wd_hi, K.l1_wd_lo}, ph.energy);
        term = ff_mul_f(term, sign * (float)m1);
        const float tf = ff_f(term);
        const float pd2 = ff_f(ff_add_f(term, p_d));
        const float p_n2 = sqrtf(1.0f - pd2 * pd2 - p_l * p_l);
        const float sgn_n = (p_n > 0.0f) ? 1.0f : ((p_n < 0.0f) ? -1.0f : 0.0f);
        const float dn_comp = sgn_n * (-tf * (2.0f * p_d + tf)) / (p_n2 + fabsf(p_n));
        const f3 delta = tf * d1 + dn_comp * n;
        ph.pol = transport_delta_f(p, delta, ph.pol);
        ph.dir = p + delta;
    }
    if (MGPU_UNLIKELY(!(prob1 >= 0.0f && prob1 <= 1.0f))) atomicOr(status, MGPU_STATUS_PROB_RANGE);
    ph.prob *= prob1;
    stored<kAll>(st.out[6], i, f2d_bits((float)m1));
    storef<kAll>(st.out[7], i, blaze1);
    // L2Abs: open fraction minus the shadow of the inclined hexagon walls;
    // sin(arccos |p . n|) = |p x n| (no cancellation near normal incidence)
    const f3 p3 = normf(ph.dir);
    const f3 pxn = crossf(p3, n);
    const float sin3 = fminf(sqrtf(dotf(pxn, pxn)), 1.0f);
    const float a2 = K.l2_open32 - K.l2_absorb32 * sin3;
    if (MGPU_UNLIKELY(!(a2 >= 0.0f && a2 <= 1.0f))) atomicOr(status, MGPU_STATUS_PROB_RANGE);
    ph.prob *= a2;
    // L2Diffraction: N(0,1) * sigma about dir x guess, then a uniform turn
    // about the direction, both as direction changes
    const f3 guess = (fabsf(p3.x) < 0.99999f) ? f3{1.0f, 0.0f, 0.0f} : f3{0.0f, 1.0f, 0.0f};
    const f3 perp = crossf(p3, guess);
    const float wave_mm = kHcMm / ph.energy.hi;
    const float sigma = (1.22f * 0.4f) * asinf(wave_mm * K.l2_inv_inner32);
    const float ang = z_l2 * sigma;
    const f3 dl1 = rot_transpose_delta_f(perp, ang, p3);
    const f3 dl2 = rot_transpose_delta_f(p3, u_phi * 6.283185307179586f, p3 + dl1);
    const f3 delta2 = dl1 + dl2;
    ph.pol = transport_delta_f(p3, delta2, ph.pol);
    ph.dir = p3 + delta2;
    storef<kAll>(st.out[8], i, ang);
    storef<kAll>(st.out[4], i, ly);
    storef<kAll>(st.out[5], i, lz);
}

// kStack: compiled with the CATL1L2Stack layers (launches whose chain has a
// stacked facet stage); plain facet chains leave them out entirely.
// kSel0: every facet uses the stage's first selector, read from the inline
// copy in the parameter bank.  kLean (the plain fixed chains): that
// selector is a sorted, guided efficiency table and no column is evaluated
// on the host
template <bool kStack, bool kSel0, bool kLean>
__device__ bool stage_gratings_l(const mgpu_stage& st, PhotonL& ph, int i, bool valid,
                                 int rng, uint64_t seed, uint64_t row_base, int sidx,
                                 uint32_t* status) {
    HitL h;
    int f = nearest_facet_l(st, ph, valid, &h);
    if (!valid) return false;
    if (MGPU_UNLIKELY(f < 0)) {
        write_miss_defaults(st, i, kStack ? MGPU_MAX_OUT : 4);
        return false;
    }
    {
        const ff3 c = facet_centre(st.facets32 + f);
        h.ip = ff3{ff_add_f(c.x, h.v.x), ff_add_f(c.y, h.v.y), ff_add_f(c.z, h.v.z)};
    }
    // FlatGrating.diffract_photons (grating.py:233-266) in the facet frame;
    // rows (ex, ey.x), (ez.z, l), (dneg, wd_hi), (wd_lo, id, selector, flags)
    const mgpu_facet32* fc = st.facets32 + f;
    const float4* fr = facet_rows(fc);
    const float4 R2 = __ldg(fr + 2), R4 = __ldg(fr + 4), R5 = __ldg(fr + 5), R6 = __ldg(fr + 6);
    f3 l{R4.y, R4.z, R4.w}, dn{R5.x, R5.y, R5.z}, n{R2.x, R2.y, R2.z};
    f3 p = normf(ph.dir);
    float p_l = dotf(p, l), p_d = dotf(p, dn), p_n = dotf(p, n);
    float blaze = atan2f(fabsf(p_d), fabsf(p_n));      // = arccos|p_perp . n|
    // NonParallelCATGrating.blaze_angle_modifier (catgrating.py:324-333)
    float blaze_s = (kStack && st.stack)
                        ? blaze + (st.stack->blaze_center32 + h.ly * st.stack->d_blaze32)
                        : blaze;
    // a custom blaze_angle_modifier, evaluated on the host (grating.py:255)
    if (!kLean && st.blaze_add.ptr) {
        blaze_s += d2f_bits(*at(st.blaze_add.ptr, i, st.blaze_add.stride));
        blaze = blaze_s;
    }
    uint64_t U, U1 = 0;
    double u_pre = 0.0;
    if (rng == MGPU_RNG_PREDRAWN) {
        if (st.draw[0] == nullptr) {
            atomicOr(status, MGPU_STATUS_BAD_STAGE);
            return false;
        }
        u_pre = *at(st.draw[0], i, st.draw_stride);
        U = (uint64_t)(u_pre * 9007199254740992.0);
        if (kStack && st.draw[1]) U1 = (uint64_t)(*at(st.draw[1], i, st.draw_stride) * 9007199254740992.0);
    } else {
        philox_u53(seed, row_base + (uint64_t)i, (uint32_t)sidx, &U, &U1);
    }
    float selprob = 1.0f;
    double selprob_d = 1.0;
    const int flags = __float_as_int(R6.w);
    const mgpu_selector& sel = kSel0 ? st.sel0 : st.selectors[__float_as_int(R6.z)];
    int m;
    if (!kLean && sel.kind == MGPU_SEL_SPLINE) {
        // float32 evaluation of the interpolated table
        m = select_order_spline_f(sel, ph.energy, blaze_s, u53_to_f(U), &selprob);
        if (MGPU_UNLIKELY(!(selprob >= 0.0f && selprob <= 1.0f))) atomicOr(status, MGPU_STATUS_PROB_RANGE);
    } else {
        // fixed chains found the energy row at the start of the photon
        const int row = kSel0 ? ph.row0 : energy_row(sel, ph.energy_d, ph.energy.hi);
        if (kLean) m = select_order_row<kLean>(sel, row, U, &selprob, status, &selprob_d);
        else m = select_order_row<kLean>(sel, row, U, &selprob, status);
    }
    float sign;
    if (flags & 1) sign = (p_d > 0.0f) ? 1.0f : ((p_d < 0.0f) ? -1.0f : 1.0f);
    else sign = -1.0f;
    // sign * m * lambda / d in float-float
    ff wd{R5.w, R6.x};
    if (!kLean && st.grating_d.ptr) {
        // a position-dependent grating constant: energy2wave / d per photon
        const double v = *at(st.grating_d.ptr, i, st.grating_d.stride);
        if (!isnan(v)) wd = ff_div(ff{kE2wHi, kE2wLo}, d2ff_hw(v));
    }
    ff term = ff_div(wd, ph.energy);
    term = ff_mul_f(term, sign * (float)m);
    float tf = ff_f(term);
    float pd2 = ff_f(ff_add_f(term, p_d));
    float p_n2 = sqrtf(1.0f - pd2 * pd2 - p_l * p_l);
    float sgn_n = (p_n > 0.0f) ? 1.0f : ((p_n < 0.0f) ? -1.0f : 0.0f);
    // change of the unit direction: tf along d, and along n the difference
    // p_n2 - |p_n| = -tf (2 p_d + tf) / (p_n2 + |p_n|) (no cancellation);
    // a reflection grating flips the normal component instead
    float dn_comp;
    if (flags & 2) dn_comp = sgn_n * (-tf * (2.0f * p_d + tf)) / (p_n2 + fabsf(p_n));
    else dn_comp = -sgn_n * p_n2 - p_n;
    f3 delta = tf * dn + dn_comp * n;
    ph.pol = transport_delta_f(p, delta, ph.pol);
    ph.dir = p + delta;
    if (kLean) ph.prob_d *= selprob_d;
    else ph.prob *= selprob;
    store_hit<kSel0>(st.out[0], i, h.ly);
    store_hit<kSel0>(st.out[1], i, h.lz);
    stored<kSel0>(st.out[2], i, f2d_fin_bits((float)m));
    if (kStack && st.stack) storef<kSel0>(st.out[3], i, blaze_s);
    else if (kLean) store_hit<kSel0>(st.out[3], i, blaze);
    else storef<kSel0>(st.out[3], i, blaze);
    if (kLean || st.id_out) store_id(st, i, __float_as_int(R6.y));
    if (kStack && st.stack) {
        bool support;
        float u_phi, z;
        if (rng == MGPU_RNG_PREDRAWN) {
            if (!st.draw[1] || !st.draw[2] || !st.draw[3] || !st.draw[4]) {
                atomicOr(status, MGPU_STATUS_BAD_STAGE);
                return false;
            }
            support = *at(st.draw[2], i, st.draw_stride) > st.stack->l1_open;
            z = __double2float_rn(*at(st.draw[3], i, st.draw_stride));
            u_phi = __double2float_rn(*at(st.draw[4], i, st.draw_stride));
        } else {
            // the float64 kernel's counters: draw 1 (u_sup, u_phi), draw 2
            // (the normal, by Box-Muller in float32 from the same uniforms);
            // u_sup > l1_open decided exactly on the 53-bit integer
            const uint64_t row = row_base + (uint64_t)i;
            uint64_t A, B;
            philox_u53_draw(seed, row, (uint32_t)sidx, 1u, &A, &B);
            support = (int64_t)A > st.stack->l1_open_u53;
            u_phi = u53_to_f(B);
            philox_u53_draw(seed, row, (uint32_t)sidx, 2u, &A, &B);
            const float one_minus_u0 = (float)((1ull << 53) - A) * 1.1102230246251565e-16f;
            float sn, cs;
            sincospif(2.0f * u53_to_f(B), &sn, &cs);
            z = sqrtf(-2.0f * logf(one_minus_u0)) * cs;   // accurate log: small u
        }
        cat_stack_layers_l<kSel0>(st, *st.stack, f, m, h.ly, h.lz, U1, support, z, u_phi, ph, i,
                                  status);
    }
    ph.pos = h.ip;
    return true;
}

// Parallel of FlatDetectors (a CCD array): FlatDetector.specific_process_photons
// (optics/detector.py:72-75) on the nearest element the ray crosses; record
// row (ez.z, l) holds 1 / pixel size and the centre pixel
template <bool kAll, bool kLean>
__device__ bool stage_detarray_l(const mgpu_stage& st, PhotonL& ph, int i, bool valid) {
    HitL h;
    int f = nearest_facet_l(st, ph, valid, &h);
    if (!valid) return false;
    if (MGPU_UNLIKELY(f < 0)) {
        write_miss_defaults(st, i, 4);
        return false;
    }
    const mgpu_facet32* fc = st.facets32 + f;
    const ff3 c = facet_centre(fc);
    const float4 R4 = __ldg(facet_rows(fc) + 4), R6 = __ldg(facet_rows(fc) + 6);
    store_hit<kAll>(st.out[0], i, h.ly);
    store_hit<kAll>(st.out[1], i, h.lz);
    store_hit<kAll>(st.out[2], i, fmaf(h.ly, R4.y, R4.z));
    store_hit<kAll>(st.out[3], i, fmaf(h.lz, R4.y, R4.w));
    if (kLean || st.id_out) store_id(st, i, __float_as_int(R6.y));
    ph.pos = ff3{ff_add_f(c.x, h.v.x), ff_add_f(c.y, h.v.y), ff_add_f(c.z, h.v.z)};
    return true;
}

// one stage, kind known at compile time (KIND > 0) or read from the
// descriptor (KIND == 0, generic chains)
template <int KIND, bool kStack, bool kSel0, bool kPhilox, bool kLean>
__device__ __forceinline__ bool run_stage_l(const mgpu_stage& st, PhotonL& ph, int i,
                                            bool valid, const mgpu_chain& chain, int s) {
    // fixed chains run Philox only: the pre-drawn branches fold away
    const int rng = kPhilox ? MGPU_RNG_PHILOX : chain.rng;
    const int kind = KIND ? KIND : st.kind;
    switch (kind) {
    case MGPU_STAGE_GRATINGS:
        return stage_gratings_l<kStack, kSel0, kLean>(st, ph, i, valid, rng, chain.seed, chain.row_base,
                                        s, chain.status);
    case MGPU_STAGE_DETARRAY:
        return stage_detarray_l<kSel0, kLean>(st, ph, i, valid);
    case MGPU_STAGE_LENS:
        return valid && stage_lens_l<kLean, kSel0>(st, ph, i, chain.status);
    case MGPU_STAGE_SCATTER:
        return valid && stage_scatter_l<kSel0, kLean>(st, ph, i, rng, chain.seed, chain.row_base, s,
                                        chain.status);
    case MGPU_STAGE_FLATDET:
        return valid && stage_flatdet_l<kSel0>(st, ph, i);
    case MGPU_STAGE_CYLDET:
        return valid && stage_cyldet_l<kSel0>(st, ph, i);
    case MGPU_STAGE_SUPPORT:
        // catsupportbars (missions/mitsnl/catgrating.py:314-324)
        if (valid) {
            bool absorb = true;
            if (st.id_out)
                absorb = (((st.first_writer >> 17) & 1)
                              ? *at((const int64_t*)st.id_out, i, st.id_stride)
                              : (int64_t)*at((const int32_t*)st.id_out, i, st.id_stride)) < 0;
            if (absorb) {
                ph.prob = 0.0f;
                ph.prob_d = 0.0;     // the lean chains' float64 probability
            }
        }
        return false;
    default:
        if (valid) atomicOr(chain.status, MGPU_STATUS_BAD_STAGE);
        return false;
    }
}

// per-warp hit counts of a photon's stages (bit s of mask: stage s hit),
// added once at the end of the chain: one short loop instead of a vote and
// an atomic between every two stages (4 KB less code in the CAT chain)
// the same for a stage count known at compile time: the votes unrolled, one
// lane-0 block for the atomics
template <int N>
__device__ __forceinline__ void count_hits_fixed(uint32_t mask, unsigned* s_hits, int lane) {
    unsigned m[N];
#pragma unroll
    for (int s = 0; s < N; ++s) m[s] = __ballot_sync(MGPU_FULL_MASK, (mask >> s) & 1u);
    if (lane == 0) {
#pragma unroll
        for (int s = 0; s < N; ++s)
            if (m[s]) atomicAdd(&s_hits[s], (unsigned)__popc(m[s]));
    }
}

__device__ __forceinline__ void count_hits(uint32_t mask, unsigned* s_hits, int n_stages, int lane) {
#pragma unroll 1
    for (int s = 0; s < n_stages; ++s) {
        const unsigned m = __ballot_sync(MGPU_FULL_MASK, (mask >> s) & 1u);
        if (lane == 0 && m) atomicAdd(&s_hits[s], (unsigned)__popc(m));
    }
}

// generic chain: stage loop over the descriptors
struct GenericChain {
    static constexpr bool kFixed = false;
    static constexpr int kSearches = 2;
    template <bool kStack, bool kLean>
    __device__ static uint32_t run(const mgpu_chain& chain, PhotonL& ph, int i, bool valid) {
        static_assert(!kLean, "the generic loop serves every configuration");
        uint32_t mask = 0;
        for (int s = 0; s < chain.n_stages; ++s)
            mask |= (uint32_t)run_stage_l<0, kStack, false, false, false>(chain.stages[s], ph, i, valid,
                                                                       chain, s)
                    << s;
        return mask;
    }
};

// fixed chain: stage kinds and descriptor offsets known at compile time, so
// the per-stage constants are read straight from the parameter bank
template <int... K>
struct FixedChain {
    static constexpr bool kFixed = true;
    // facet-table searches (grating arrays, CCD arrays) in the chain
    static constexpr int kSearches =
        (0 + ... + (K == MGPU_STAGE_GRATINGS || K == MGPU_STAGE_DETARRAY ? 1 : 0));
    static constexpr int kStages = (int)sizeof...(K);
    template <int KIND, int S, bool kStack, bool kLean>
    __device__ static uint32_t step(const mgpu_chain& chain, PhotonL& ph, int i, bool valid) {
        return (uint32_t)run_stage_l<KIND, kStack, true, true, kLean>(chain.stages[S], ph, i, valid,
                                                                     chain, S)
               << S;
    }
    template <bool kStack, bool kLean, int... S>
    __device__ static uint32_t run_seq(const mgpu_chain& chain, PhotonL& ph, int i, bool valid,
                                       std::integer_sequence<int, S...>) {
        uint32_t mask = 0;
        ((mask |= step<K, S, kStack, kLean>(chain, ph, i, valid)), ...);
        return mask;
    }
    // the facet stage (at most one) whose selector's energy row is found
    // at the start, so its table loads overlap the stages before it
    static constexpr int kGratings = []() {
        const int kinds[] = {K...};
        for (int s = 0; s < (int)sizeof...(K); ++s)
            if (kinds[s] == MGPU_STAGE_GRATINGS) return s;
        return -1;
    }();
    static_assert((0 + ... + (K == MGPU_STAGE_GRATINGS ? 1 : 0)) <= 1,
                  "fixed chains hold at most one grating array");
    // kLean: compiled for the common element configuration only (lean_ok)
    template <bool kStack, bool kLean>
    __device__ static uint32_t run(const mgpu_chain& chain, PhotonL& ph, int i, bool valid) {
        static_assert(!(kLean && kStack), "the stacked chains are not lean");
        if constexpr (kGratings >= 0) {
            const mgpu_selector& sel = chain.stages[kGratings].sel0;
            if (kLean) ph.row0 = energy_row<true>(sel, ph.energy_d, ph.energy.hi);
            else if (sel.kind != MGPU_SEL_SPLINE) ph.row0 = energy_row(sel, ph.energy_d, ph.energy.hi);
        }
        return run_seq<kStack, kLean>(chain, ph, i, valid,
                                      std::make_integer_sequence<int, sizeof...(K)>{});
    }
    // the stage kinds match, every facet stage reads its first selector, and
    // the draws come from Philox (the pre-drawn code is compiled out)
    static bool matches(const mgpu_chain& chain) {
        const int kinds[] = {K...};
        if (chain.n_stages != (int)sizeof...(K) || chain.rng != MGPU_RNG_PHILOX) return false;
        for (int s = 0; s < chain.n_stages; ++s) {
            if (chain.stages[s].kind != kinds[s]) return false;
            if (kinds[s] == MGPU_STAGE_GRATINGS && !chain.stages[s].facet_sel0) return false;
        }
        return true;
    }
};

// the configuration the plain fixed chains are compiled for (kLean): lenses
// without a reflectivity table; scatter surfaces with both widths nonzero;
// facet arrays with an id column;
// grating arrays whose facets all use one efficiency table with increasing
// energy rows, row midpoints and a guide table, with no column evaluated on
// the host
// every column the stages write exists (what the fixed chains store to
// without a pointer test): 2 for a lens, 9 for a stacked facet array, none
// for the support bars, 4 otherwise
bool cols_ok(const mgpu_chain& chain) {
    for (int s = 0; s < chain.n_stages; ++s) {
        const mgpu_stage& st = chain.stages[s];
        const int nout = (st.kind == MGPU_STAGE_LENS) ? 2
                         : (st.kind == MGPU_STAGE_SUPPORT) ? 0
                         : (st.kind == MGPU_STAGE_GRATINGS && st.stack) ? 9 : 4;
        for (int k = 0; k < nout; ++k)
            if (st.out[k].ptr == nullptr) return false;
    }
    return true;
}

bool lean_ok(const mgpu_chain& chain) {
    for (int s = 0; s < chain.n_stages; ++s) {
        const mgpu_stage& st = chain.stages[s];
        if (st.kind == MGPU_STAGE_LENS && st.spline.n_surf > 0) return false;
        if (st.kind == MGPU_STAGE_SCATTER && (st.p[0] == 0.0 || st.p[1] == 0.0)) return false;
        if ((st.kind == MGPU_STAGE_GRATINGS || st.kind == MGPU_STAGE_DETARRAY) && !st.id_out)
            return false;
        if (st.kind == MGPU_STAGE_GRATINGS) {
            const mgpu_selector& q = st.sel0;
            if (!st.facet_sel0 || st.stack || st.grating_d.ptr || st.blaze_add.ptr ||
                q.kind != MGPU_SEL_CDF || !q.by_energy || !q.sorted || !q.guide || !q.e_mid ||
                q.n_rows < 1)
                return false;
        }
    }
    return true;
}

template <class Chain, bool kStack, bool kLean>
// fixed plain chains with one facet search: 4 blocks of 256 per SM (64
// registers, no spills; the stage constants come from the parameter bank),
// measured 6 % faster than 3 blocks (80 registers) on the CAT chain at 1e8
// photons; 5 blocks (48 registers) spill and measured 4 % slower, 128-thread
// blocks at 56 registers (36 warps, small spills) 5 % slower.  The others
// keep 3 blocks (at 64 registers they spill), which measured 4 % faster
// than the unconstrained allocation (100 registers, 2 blocks); a capped
// (persistent) grid measured no faster.  One photon per thread.
__global__ void __launch_bounds__(kThreads, (Chain::kFixed && !kStack && Chain::kSearches <= 1)
                                                ? kMinBlocks : kMinBlocksWide)
chain_fp32local_kernel(const __grid_constant__ mgpu_chain chain, const __grid_constant__ mgpu_photons io) {
    constexpr bool kLeanChain = kLean;
    __shared__ unsigned int s_hits[MGPU_MAX_STAGES];
    if (threadIdx.x < MGPU_MAX_STAGES) s_hits[threadIdx.x] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int n = (int)io.n;                      // < 2^30 per launch
    const int warp_id = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int n_warps = (int)((gridDim.x * blockDim.x) >> 5);
    for (int base = warp_id * 32; base < n; base += n_warps * 32) {
        const int i = base + lane;
        const bool valid = i < n;
        PhotonL ph;
        if (valid) {
            d3 p = load3i(io.pos, i), d = load3i(io.dir, i), q = load3i(io.pol, i);
            // positions on the integer pipe, the rest on the FP64 pipe's
            // conversions: measured 1.2 % faster than all of them on either
            ph.pos = ff3{d2ff_bits(p.x), d2ff_bits(p.y), d2ff_bits(p.z)};
            ph.dir = f3{__double2float_rn(d.x), __double2float_rn(d.y), __double2float_rn(d.z)};
            ph.pol = f3{__double2float_rn(q.x), __double2float_rn(q.y), __double2float_rn(q.z)};
            ph.energy_d = *at(io.energy.ptr, i, io.energy.stride);
            ph.energy = d2ff_hw(ph.energy_d);
            if (kLeanChain) ph.prob_d = *at(io.prob.ptr, i, io.prob.stride);
            else ph.prob = __double2float_rn(*at(io.prob.ptr, i, io.prob.stride));
            ph.row0 = -1;
        } else {
            ph.pos = ff3{ff{0.f, 0.f}, ff{0.f, 0.f}, ff{0.f, 0.f}};
            ph.dir = ph.pol = f3{0.f, 0.f, 0.f};
            ph.energy = ff{1.f, 0.f};
            ph.energy_d = 1.0;
            ph.prob = 0.f;
            ph.prob_d = 0.0;
            ph.row0 = -1;
        }
        if (valid && (chain.flags & MGPU_FLAG_CHECK_W)) {
            if (*at(io.pos.ptr + 3 * io.pos.cstride, i, io.pos.stride) != 1.0 ||
                *at(io.dir.ptr + 3 * io.dir.cstride, i, io.dir.stride) != 0.0 ||
                *at(io.pol.ptr + 3 * io.pol.cstride, i, io.pol.stride) != 0.0)
                atomicOr(chain.status, MGPU_STATUS_BAD_W);
        }
        const uint32_t hits = Chain::template run<kStack, kLean>(chain, ph, i, valid);
        if (valid) {
            store3i(io.pos_out, i, d3{ff2d(ph.pos.x), ff2d(ph.pos.y), ff2d(ph.pos.z)});
            // state outputs on the FP64 pipe's conversions, stage columns on
            // the integer pipe: the split measured fastest (0.6 % against
            // all on the integer pipe, which the columns keep)
            store3i(io.dir_out, i, d3{(double)ph.dir.x, (double)ph.dir.y, (double)ph.dir.z});
            store3i(io.pol_out, i, d3{(double)ph.pol.x, (double)ph.pol.y, (double)ph.pol.z});
            put(at(io.prob_out.ptr, i, io.prob_out.stride), kLeanChain ? ph.prob_d : (double)ph.prob);
        }
        if constexpr (Chain::kFixed) count_hits_fixed<Chain::kStages>(hits, s_hits, lane);
        else count_hits(hits, s_hits, chain.n_stages, lane);
    }
    __syncthreads();
    if (threadIdx.x < chain.n_stages && s_hits[threadIdx.x])
        atomicAdd(chain.hits + threadIdx.x, (unsigned long long)s_hits[threadIdx.x]);
}

// the chains of the standard instruments: lens, scatter, gratings, cylinder
// or flat detector; lens, scatter, flat detector
using ChainCat = FixedChain<MGPU_STAGE_LENS, MGPU_STAGE_SCATTER, MGPU_STAGE_GRATINGS, MGPU_STAGE_CYLDET>;
using ChainSpec = FixedChain<MGPU_STAGE_LENS, MGPU_STAGE_SCATTER, MGPU_STAGE_GRATINGS, MGPU_STAGE_FLATDET>;
using ChainTel = FixedChain<MGPU_STAGE_LENS, MGPU_STAGE_SCATTER, MGPU_STAGE_FLATDET>;
// the grating array followed by a CCD camera (a Parallel of FlatDetectors)
using ChainCcd = FixedChain<MGPU_STAGE_LENS, MGPU_STAGE_SCATTER, MGPU_STAGE_GRATINGS,
                            MGPU_STAGE_DETARRAY>;
// the CAT array followed by its support structure (catsupportbars)
using ChainCatBars = FixedChain<MGPU_STAGE_LENS, MGPU_STAGE_SCATTER, MGPU_STAGE_GRATINGS,
                                MGPU_STAGE_SUPPORT, MGPU_STAGE_CYLDET>;

}  // namespace

namespace {

// the kernel addresses photon i of a column with a 32-bit byte offset
// (i * stride * 8), so launches cover at most 2^30 photons and strides stay
// below 2^28 elements
constexpr int64_t kMaxLaunch = 1ll << 30;
bool stride_ok(int64_t s) { return s > -(1ll << 28) && s < (1ll << 28); }
bool col_ok(const mgpu_col& c) { return c.ptr == nullptr || stride_ok(c.stride); }
bool vec_ok(const mgpu_vec& v) { return stride_ok(v.stride); }

template <class T>
T* advanced(T* p, int64_t off, int64_t stride, int64_t size) {
    return p ? (T*)((char*)p + off * stride * size) : p;
}

// the descriptors of photon rows [off, ...): every column pointer moved
// to row off, the Philox row counter with them
void advance_rows(mgpu_chain& c, mgpu_photons& io, int64_t off) {
    for (mgpu_vec* v : {&io.pos, &io.dir, &io.pol, &io.pos_out, &io.dir_out, &io.pol_out})
        v->ptr = advanced(v->ptr, off, v->stride, 8);
    for (mgpu_col* k : {&io.energy, &io.prob, &io.prob_out}) k->ptr = advanced(k->ptr, off, k->stride, 8);
    c.row_base += (uint64_t)off;
    for (int s = 0; s < c.n_stages; ++s) {
        mgpu_stage& st = c.stages[s];
        for (int k = 0; k < MGPU_MAX_OUT; ++k) st.out[k].ptr = advanced(st.out[k].ptr, off, st.out[k].stride, 8);
        st.id_out = advanced((char*)st.id_out, off, st.id_stride, ((st.first_writer >> 17) & 1) ? 8 : 4);
        for (int k = 0; k < MGPU_MAX_DRAWS; ++k) st.draw[k] = advanced(st.draw[k], off, st.draw_stride, 8);
        st.grating_d.ptr = advanced(st.grating_d.ptr, off, st.grating_d.stride, 8);
        st.blaze_add.ptr = advanced(st.blaze_add.ptr, off, st.blaze_add.stride, 8);
    }
}

// the fixed (plain) chain kernel of the chain's stage sequence, lean or
// not; false when no fixed chain matches
template <bool kLean>
bool launch_fixed(const mgpu_chain& chain, const mgpu_photons& io, unsigned gb, cudaStream_t stream) {
    if (ChainCat::matches(chain))
        chain_fp32local_kernel<ChainCat, false, kLean><<<gb, kThreads, 0, stream>>>(chain, io);
    else if (ChainSpec::matches(chain))
        chain_fp32local_kernel<ChainSpec, false, kLean><<<gb, kThreads, 0, stream>>>(chain, io);
    else if (ChainCcd::matches(chain))
        chain_fp32local_kernel<ChainCcd, false, kLean><<<gb, kThreads, 0, stream>>>(chain, io);
    else if (ChainTel::matches(chain))
        chain_fp32local_kernel<ChainTel, false, kLean><<<gb, kThreads, 0, stream>>>(chain, io);
    else if (ChainCatBars::matches(chain))
        chain_fp32local_kernel<ChainCatBars, false, kLean><<<gb, kThreads, 0, stream>>>(chain, io);
    else
        return false;
    return true;
}

cudaError_t launch_rows(const mgpu_chain& chain, const mgpu_photons& io, cudaStream_t stream,
                        int sm_count) {
    int64_t warps = (io.n + 31) / 32;
    int64_t blocks = (warps * 32 + kThreads - 1) / kThreads;
    if (kGridPerSm > 0) {
        const int64_t cap = (int64_t)sm_count * kGridPerSm * 256 / kThreads;
        if (blocks > cap) blocks = cap;
    }
    bool stacked = false;
    for (int s = 0; s < chain.n_stages; ++s) stacked = stacked || chain.stages[s].stack != nullptr;
    const unsigned gb = (unsigned)blocks;
    if (chain.flags & MGPU_FLAG_GENERIC) {
        if (stacked)
            chain_fp32local_kernel<GenericChain, true, false><<<gb, kThreads, 0, stream>>>(chain, io);
        else
            chain_fp32local_kernel<GenericChain, false, false><<<gb, kThreads, 0, stream>>>(chain, io);
    } else if (!cols_ok(chain)) {
        // a column the stages write is missing: the generic loop tests each
        if (stacked)
            chain_fp32local_kernel<GenericChain, true, false><<<gb, kThreads, 0, stream>>>(chain, io);
        else
            chain_fp32local_kernel<GenericChain, false, false><<<gb, kThreads, 0, stream>>>(chain, io);
    } else if (stacked) {
        if (ChainCatBars::matches(chain))
            chain_fp32local_kernel<ChainCatBars, true, false><<<gb, kThreads, 0, stream>>>(chain, io);
        else
            chain_fp32local_kernel<GenericChain, true, false><<<gb, kThreads, 0, stream>>>(chain, io);
    } else if (lean_ok(chain)) {
        if (!launch_fixed<true>(chain, io, gb, stream))
            chain_fp32local_kernel<GenericChain, false, false><<<gb, kThreads, 0, stream>>>(chain, io);
    } else if (!launch_fixed<false>(chain, io, gb, stream)) {
        chain_fp32local_kernel<GenericChain, false, false><<<gb, kThreads, 0, stream>>>(chain, io);
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t mgpu_launch_chain_fp32local(const mgpu_chain& chain, const mgpu_photons& io,
                                        cudaStream_t stream, int sm_count) {
    if (io.n <= 0) return cudaSuccess;
    if (!vec_ok(io.pos) || !vec_ok(io.dir) || !vec_ok(io.pol) || !vec_ok(io.pos_out) ||
        !vec_ok(io.dir_out) || !vec_ok(io.pol_out) || !col_ok(io.energy) || !col_ok(io.prob) ||
        !col_ok(io.prob_out))
        return cudaErrorInvalidValue;
    for (int s = 0; s < chain.n_stages; ++s) {
        const mgpu_stage& st = chain.stages[s];
        if (st.aux_size <= 0 && st.kind != MGPU_STAGE_SUPPORT) return cudaErrorInvalidValue;
        if ((st.kind == MGPU_STAGE_GRATINGS || st.kind == MGPU_STAGE_DETARRAY) &&
            (st.facets32 == nullptr || ((uintptr_t)st.facets32 & 15u) != 0))
            return cudaErrorInvalidValue;
        if (st.kind == MGPU_STAGE_CYLDET && (st.table == nullptr || ((uintptr_t)st.table & 15u) != 0))
            return cudaErrorInvalidValue;
        if (st.kind == MGPU_STAGE_LENS && st.spline.n_surf > 0 &&
            (st.spline.tx_ff == nullptr || st.spline.ty_ff == nullptr || st.spline.c32 == nullptr))
            return cudaErrorInvalidValue;
        for (int k = 0; k < MGPU_MAX_OUT; ++k)
            if (!col_ok(st.out[k])) return cudaErrorInvalidValue;
        if ((st.id_out && !stride_ok(st.id_stride)) || !stride_ok(st.draw_stride) ||
            !col_ok(st.grating_d) || !col_ok(st.blaze_add))
            return cudaErrorInvalidValue;
    }
    const int64_t max_launch = (chain.flags & MGPU_FLAG_SPLIT_4K) ? 4096 : kMaxLaunch;
    if (io.n <= max_launch) return launch_rows(chain, io, stream, sm_count);
    for (int64_t off = 0; off < io.n; off += max_launch) {
        mgpu_chain c = chain;
        mgpu_photons part = io;
        advance_rows(c, part, off);
        part.n = (io.n - off < max_launch) ? io.n - off : max_launch;
        const cudaError_t e = launch_rows(c, part, stream, sm_count);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}
