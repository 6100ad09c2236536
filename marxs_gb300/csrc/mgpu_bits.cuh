// Float64 <-> float32 conversions on the integer pipe (host and device).
//
// GB300 issues F2F conversions on its FP64 pipe (~2 per clock per SM); these
// bit-level versions use shifts, adds and compares instead.  They are
// __host__ __device__ so the CPU test suite checks them against exact casts.
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define MGPU_HD __host__ __device__ __forceinline__
#else
#define MGPU_HD inline
#endif

MGPU_HD uint32_t mgpu_dhi(double d) {
#if defined(__CUDA_ARCH__)
    return (uint32_t)__double2hiint(d);
#else
    uint64_t b;
    memcpy(&b, &d, 8);
    return (uint32_t)(b >> 32);
#endif
}
MGPU_HD uint32_t mgpu_dlo(double d) {
#if defined(__CUDA_ARCH__)
    return (uint32_t)__double2loint(d);
#else
    uint64_t b;
    memcpy(&b, &d, 8);
    return (uint32_t)b;
#endif
}
MGPU_HD double mgpu_mkd(uint32_t hi, uint32_t lo) {
#if defined(__CUDA_ARCH__)
    return __hiloint2double((int)hi, (int)lo);
#else
    uint64_t b = ((uint64_t)hi << 32) | lo;
    double d;
    memcpy(&d, &b, 8);
    return d;
#endif
}
MGPU_HD float mgpu_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}
MGPU_HD uint32_t mgpu_f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

// float64 -> float32, round to nearest even.  Magnitudes below 2^-126 flush
// to signed zero; beyond the float range -> inf; NaN stays NaN.
MGPU_HD float d2f_bits(double d) {
    uint32_t hi = mgpu_dhi(d), lo = mgpu_dlo(d);
    uint32_t sign = hi & 0x80000000u;
    uint32_t e = (hi >> 20) & 0x7ffu;
    uint32_t m = (hi << 3) | (lo >> 29);                 // low 9 exponent bits + 23 mantissa bits
    uint32_t r = (m - 0xC0000000u) & 0x7fffffffu;        // exponent - 896 (mod 2^9), 8 bits kept
    uint32_t rem = lo & 0x1fffffffu;
    r += (rem > 0x10000000u) | ((rem == 0x10000000u) & (r & 1u));
    uint32_t bits;
    if (e >= 897u && e <= 1150u) bits = r;
    else if (e < 897u) bits = 0u;
    else if (e == 0x7ffu && (((hi & 0xfffffu) | lo) != 0u)) bits = 0x7fc00000u;
    else bits = 0x7f800000u;
    return mgpu_u2f(bits | sign);
}

// float32 -> float64, exact (denormal floats -> 0)
MGPU_HD double f2d_bits(float f) {
    uint32_t b = mgpu_f2u(f);
    uint32_t sign = b & 0x80000000u, mag = b & 0x7fffffffu;
    uint32_t hi, lo;
    if (mag >= 0x00800000u && mag < 0x7f800000u) {
        hi = (mag >> 3) + 0x38000000u;
        lo = b << 29;
    } else if (mag >= 0x7f800000u) {
        hi = 0x7ff00000u | (mag >> 3);
        lo = b << 29;
    } else {
        hi = 0u;
        lo = 0u;
    }
    return mgpu_mkd(hi | sign, lo);
}

// float32 -> float64 for finite values, exact (denormal floats -> signed
// zero); infinities and NaN are not handled (callers pass hit coordinates
// and angles only)
MGPU_HD double f2d_fin_bits(float f) {
    uint32_t b = mgpu_f2u(f);
    uint32_t mag = b & 0x7fffffffu;
    uint32_t hi = (mag >> 3) + 0x38000000u, lo = b << 29;
    if (mag < 0x00800000u) hi = lo = 0u;
    return mgpu_mkd(hi | (b & 0x80000000u), lo);
}

// float64 -> (hi, lo) float32 pair: hi = d2f_bits(d), lo = d - hi rounded
// to float32 (exact residual of the 53-bit mantissa, scaled).  Values below
// 2^-74 or outside the float range get lo = 0.
MGPU_HD void d2ff_bits_pair(double d, float* out_hi, float* out_lo) {
    float hi = d2f_bits(d);
    uint32_t dhi = mgpu_dhi(d), dlo = mgpu_dlo(d);
    uint32_t e = (dhi >> 20) & 0x7ffu;
    *out_hi = hi;
    if (e < 949u || e > 1150u) {
        *out_lo = 0.0f;
        return;
    }
    int32_t rem = (int32_t)(dlo & 0x1fffffffu);
    uint32_t trunc = (((dhi << 3) | (dlo >> 29)) - 0xC0000000u) & 0x7fffffffu;
    uint32_t mag_f = mgpu_f2u(hi) & 0x7fffffffu;
    if (mag_f != trunc) rem -= 0x20000000;               // hi was rounded up
    float scale = mgpu_u2f((e - 948u) << 23);             // 2^(e - 1075)
    float lo = (float)rem * scale;
    if (dhi & 0x80000000u) lo = -lo;
    *out_lo = lo;
}
