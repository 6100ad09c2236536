// Float32 / float-float helpers for the FP32-local kernel (sm_103a).
//
// On GB300 every float64 operation -- including float64<->float32
// conversion -- issues on the FP64 pipe (about 2 per clock per SM, against
// ~128 FP32 FMAs).  The FP32-local kernel therefore
//   * converts float64 inputs/outputs with integer bit manipulation (INT
//     pipe) instead of F2F instructions,
//   * carries positions as float-float pairs (hi + lo, ~48-bit mantissa)
//     built from error-free transformations (Dekker/Knuth TwoSum, FMA-based
//     TwoProd), so that re-centring a ray on an element far from the origin
//     loses nothing,
//   * keeps directions, polarization and per-element local arithmetic in
//     float32.
#pragma once
#include <stdint.h>
#include "mgpu_device.cuh"

struct ff {
    float hi, lo;
};
struct f3 {
    float x, y, z;
};
struct ff3 {
    ff x, y, z;
};

__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return f3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ float dotf(f3 a, f3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }
__device__ __forceinline__ f3 crossf(f3 a, f3 b) {
    return f3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ f3 normf(f3 v) {
    float r = rsqrtf(dotf(v, v));
    return f3{v.x * r, v.y * r, v.z * r};
}
__device__ __forceinline__ f3 ldf3(const float* p) { return f3{p[0], p[1], p[2]}; }

// ---------------------------------------------------------------- float-float
__device__ __forceinline__ ff two_sum(float a, float b) {
    float s = a + b;
    float bb = s - a;
    float e = (a - (s - bb)) + (b - bb);
    return ff{s, e};
}
__device__ __forceinline__ ff fast_two_sum(float a, float b) {   // |a| >= |b|
    float s = a + b;
    return ff{s, b - (s - a)};
}
__device__ __forceinline__ ff two_prod(float a, float b) {
    float p = a * b;
    return ff{p, fmaf(a, b, -p)};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = two_sum(a.hi, b.hi);
    ff t = two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ ff ff_add_f(ff a, float b) {
    ff s = two_sum(a.hi, b);
    s.lo += a.lo;
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
    ff p = two_prod(a.hi, b);
    p.lo = fmaf(a.lo, b, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    ff p = two_prod(a.hi, b.hi);
    p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
    return fast_two_sum(p.hi, p.lo);
}
// a / b: q1 = a.hi / b.hi, then the remainder a - q1 b formed with FMAs,
// (a.hi - q1 b.hi) rounded once (|.| a few ulp of a.hi, so its rounding is
// ~2^-47 |a|) plus (a.lo - q1 b.lo), and q2 = remainder / b.hi: ~2^-44
// relative, in 8 operations instead of the 30 of a float-float subtraction
__device__ __forceinline__ ff ff_div(ff a, ff b) {
    const float rb = __fdividef(1.0f, b.hi);
    const float q1 = a.hi * rb;
    const float r = fmaf(-q1, b.hi, a.hi) + fmaf(-q1, b.lo, a.lo);
    return fast_two_sum(q1, r * rb);
}
__device__ __forceinline__ float ff_f(ff a) { return a.hi + a.lo; }

// a - b as an unnormalised pair s + e: s = a.hi - b.hi rounded, e its exact
// rounding error (TwoSum) plus the low words; |e| is a few ulp of s, so
// s + e carries a - b to ~2^-46 relative.  The cheap entry to an element's
// frame: 8 flops instead of the 20 of ff_sub.
__device__ __forceinline__ void ff_rel(ff a, ff b, float& s, float& e) {
    s = a.hi - b.hi;
    const float bb = s - a.hi;
    e = ((a.hi - (s - bb)) + (-b.hi - bb)) + (a.lo - b.lo);
}
__device__ __forceinline__ void ff3_rel(const ff3& a, const ff3& b, f3& s, f3& e) {
    ff_rel(a.x, b.x, s.x, e.x);
    ff_rel(a.y, b.y, s.y, e.y);
    ff_rel(a.z, b.z, s.z, e.z);
}

__device__ __forceinline__ ff3 ff3_add_f3(ff3 a, f3 b) {
    return ff3{ff_add_f(a.x, b.x), ff_add_f(a.y, b.y), ff_add_f(a.z, b.z)};
}
__device__ __forceinline__ ff3 ff3_sub(ff3 a, ff3 b) {
    return ff3{ff_sub(a.x, b.x), ff_sub(a.y, b.y), ff_sub(a.z, b.z)};
}
__device__ __forceinline__ f3 ff3_f(ff3 a) { return f3{ff_f(a.x), ff_f(a.y), ff_f(a.z)}; }
// a + k * d with the products formed exactly
__device__ __forceinline__ ff3 ff3_axpy(ff3 a, float k, f3 d) {
    return ff3{ff_add(a.x, two_prod(k, d.x)), ff_add(a.y, two_prod(k, d.y)),
               ff_add(a.z, two_prod(k, d.z))};
}
__device__ __forceinline__ ff ff_dot_f(ff3 a, f3 b) {
    ff s = ff_mul_f(a.x, b.x);
    s = ff_add(s, ff_mul_f(a.y, b.y));
    return ff_add(s, ff_mul_f(a.z, b.z));
}
__device__ __forceinline__ ff ff_dot(ff3 a, ff3 b) {
    ff s = ff_mul(a.x, b.x);
    s = ff_add(s, ff_mul(a.y, b.y));
    return ff_add(s, ff_mul(a.z, b.z));
}

// ---------------------------------------------------------- bit conversions
#include "mgpu_bits.cuh"

__device__ __forceinline__ ff d2ff_bits(double d) {
    ff r;
    d2ff_bits_pair(d, &r.hi, &r.lo);
    return r;
}

// float-float -> float64: one FP64 add of two exact conversions
__device__ __forceinline__ double ff2d(ff a) { return f2d_bits(a.hi) + f2d_bits(a.lo); }
