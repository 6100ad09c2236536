// Host-side check of the integer-pipe float64<->float32 conversions used by
// the FP32-local kernel (marxs_gb300/csrc/mgpu_bits.cuh) against exact casts.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <random>
#include "../../marxs_gb300/csrc/mgpu_bits.cuh"

static uint32_t fbits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static uint64_t dbits(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }

int main() {
    std::mt19937_64 rng(1234);
    long fail_d2f = 0, fail_f2d = 0, fail_ff = 0, n = 0;
    auto check_d = [&](double d) {
        ++n;
        float ref = (float)d;
        float got = d2f_bits(d);
        bool in_range = std::fabs(d) >= 1.1754943508222875e-38 || d == 0.0 || std::isnan(d);
        if (std::isnan(ref)) { if (!std::isnan(got)) ++fail_d2f; }
        else if (in_range && fbits(ref) != fbits(got)) {
            if (fail_d2f < 5) printf("d2f %.17g: ref %08x got %08x\n", d, fbits(ref), fbits(got));
            ++fail_d2f;
        }
        float hi, lo;
        d2ff_bits_pair(d, &hi, &lo);
        double a = std::fabs(d);
        if (a >= 1e-20 && a < 1e38) {
            double err = std::fabs(((double)hi + (double)lo) - d);
            if (fbits(hi) != fbits(ref) || err > std::ldexp(a, -46)) {
                if (fail_ff < 5) printf("ff %.17g: hi %.9g lo %.9g err %g\n", d, hi, lo, err);
                ++fail_ff;
            }
        }
    };
    // random bit patterns over the float-representable exponent range
    for (int i = 0; i < 2000000; ++i) {
        uint64_t m = rng() & ((1ull << 52) - 1);
        uint64_t e = 897 + rng() % (1150 - 897 + 1);
        uint64_t s = rng() & 1;
        uint64_t b = (s << 63) | (e << 52) | m;
        double d; memcpy(&d, &b, 8);
        check_d(d);
    }
    // exact halfway cases and their neighbours
    for (int i = 0; i < 200000; ++i) {
        uint64_t m = (rng() & ((1ull << 52) - 1)) & ~((1ull << 29) - 1);
        uint64_t e = 900 + rng() % 240;
        uint64_t b = (e << 52) | m | (1ull << 28);
        double d; memcpy(&d, &b, 8);
        check_d(d);
        check_d(std::nextafter(d, 0.0));
        check_d(std::nextafter(d, 1e300));
    }
    double specials[] = {0.0, -0.0, 1.0, -1.0, 10000.0, 12000.0, 5900.0, 0.024, 1e-8, 2.0,
                         1.2398419292004202e-06, 3.4028234663852886e38, -3.4028234663852886e38,
                         INFINITY, -INFINITY, NAN, 1e300, -1e300};
    for (double d : specials) check_d(d);
    if (!std::isinf(d2f_bits(1e300)) || !std::isnan(d2f_bits(NAN))) ++fail_d2f;
    // float -> double over normal floats
    for (int i = 0; i < 2000000; ++i) {
        uint32_t u = (uint32_t)rng();
        float f; memcpy(&f, &u, 4);
        if (!(std::fabs(f) >= 1.17549435e-38f) || std::isinf(f) || std::isnan(f)) continue;
        if (dbits((double)f) != dbits(f2d_bits(f)) || dbits((double)f) != dbits(f2d_fin_bits(f))) {
            if (fail_f2d < 5) printf("f2d %.9g\n", f);
            ++fail_f2d;
        }
    }
    if (f2d_bits(0.0f) != 0.0 || !std::isinf(f2d_bits(INFINITY)) || !std::isnan(f2d_bits(NAN)))
        ++fail_f2d;
    // the finite-only conversion: signed zeros and denormals -> signed zero
    if (dbits(f2d_fin_bits(0.0f)) != dbits(0.0) || dbits(f2d_fin_bits(-0.0f)) != dbits(-0.0) ||
        dbits(f2d_fin_bits(1e-40f)) != dbits(0.0) || dbits(f2d_fin_bits(-1e-40f)) != dbits(-0.0))
        ++fail_f2d;
    printf("checked %ld doubles: d2f failures %ld, ff failures %ld, f2d failures %ld\n", n,
           fail_d2f, fail_ff, fail_f2d);
    return (fail_d2f || fail_ff || fail_f2d) ? 1 : 0;
}
