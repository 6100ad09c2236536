// Per-order statistics of a photon list: the reductions behind
// resolvingpower_from_photonlist / effectivearea_from_photonlist /
// CaptureResAeff (marxs/analysis/gratings.py:215-270, 333-363, 470-501) and
// astropy.stats.sigma_clipped_stats (median centre, population std, sigma 3,
// maxiters 5), for event columns that live on the device.
//
// Layout in HBM.  Two streaming passes over the photon columns group the
// finite values of every requested order into one contiguous segment per
// order (a stable counting sort: per 2048-photon tile, per-group counts,
// a column scan over tiles, then a scatter with ranks from warp match
// masks).  The clipping then touches only the segments: each round is one
// fused pass (count, shifted sums for mean and variance, and the first
// radix level of the median) and up to five more radix levels (11 bits
// each) of an exact selection of the middle order statistic(s).  Rounds
// stop per group as the reference loop does (no value removed, or
// maxiters reached).
//
// The FP64 pipe of this GPU runs at a small fraction of its integer and
// FP32 rate, so the streaming passes use no float64 arithmetic where an
// integer does the same job: orders are matched and filters tested on bit
// patterns, bounds are compared as order-preserving 64-bit keys, and the
// effective-area sums are exact 128-bit fixed-point integers (2^-64
// units).  What remains in float64 is the shifted sum and sum of squares,
// three operations per value and round.
//
// Determinism: integer sums are exact, so their atomics may run in any
// order; float sums are formed per tile in a fixed tree and summed over
// tiles in a fixed order.
#include <cuda_runtime.h>
#include <math.h>
#include "mgpu_device.cuh"
#include "mgpu_ff.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kTileIn = 2048;                  // photons per classify / scatter tile
constexpr int kPerLane = kTileIn / kThreads;   // 8: each warp owns 256 consecutive photons
constexpr int kTileSeg = 8192;                 // segment values per clipping-pass tile
constexpr int kSegPerThread = kTileSeg / kThreads;
constexpr int kRadixBits = 11;
constexpr int kBins = 1 << kRadixBits;
constexpr int kVBins = 8192;                   // value bins of the first level
constexpr int kHist = kVBins > 2 * kBins ? kVBins : 2 * kBins;   // per-group histogram words
constexpr int kLevels = 6;                     // ceil(64 / 11)
constexpr int kCenterSample = 31;              // values whose median centres the first clipping round's sums
constexpr int kG = MGPU_STATS_MAX_GROUPS;
constexpr uint64_t kSign = 0x8000000000000000ull;
constexpr uint64_t kExp = 0x7ff0000000000000ull;

struct GState {
    double mean, stdev, aeff, c;       // c: centre of the shifted sums
    int64_t n_cur, n_prev, n_finite;
    unsigned long long n_member;
    unsigned long long aeff_lo, aeff_hi;   // sum of probabilities, 128-bit two's complement, 2^-64 units
    unsigned long long kmin_inv, kmax;     // key range of the group's finite values (~min, max)
    uint64_t klo, khi;                 // current bounds as keys: kept iff klo <= key <= khi
    uint64_t pref[2];
    int64_t rank[2];
    unsigned long long n_cand;         // candidates of the median after the first digit
    unsigned long long cmin_inv, cmax; // key range of the candidates (~min, max)
    int32_t use_ff;                    // shifted sums in float-float (deviations of moderate size)
    float voff, vinv;                  // first level: value bin of x from d = x - c (value_bin)
    int32_t vb[2];                     // the value bins holding the two ranks
    int32_t pad_;
    uint32_t aeff_flags;               // 1: NaN or |p| >= 2^62, 2: +inf, 4: -inf
    int32_t pb;        // leading key bits known for both selections
    int32_t two;       // even count: the median averages ranks n/2-1 and n/2
    int32_t split;     // the two selections diverged: B has its own histogram
    int32_t active;    // the group is still clipping
    int32_t sel_done;  // both order statistics resolved
    int32_t final_;    // this round's statistics are the result
    int32_t round;
    int32_t bad;       // the selection lost its rank: the median is reported as NaN
};

struct Work {
    GState* gs;
    int32_t* cnt;        // [G][n_tin] finite members per tile
    int64_t* off;        // [G][n_tin] exclusive scan of cnt
    int64_t* seg_base;   // [G + 1]
    int64_t* tile_base;  // [G + 1]
    double* parts;       // [max_tseg][3]: count, sum of (x - c), sum of (x - c)^2
    uint32_t* hist;      // [G][kHist]: the value level, or two key-digit histograms
    double* seg;         // [n]
    uint64_t* cand;      // [n] keys of the median candidates, group g from seg_base[g]
    int64_t* ctile_base; // [G + 1] tiles of the candidate lists
    int64_t n_tin;
};

struct Layout {
    size_t gstate, cnt, off, seg_base, tile_base, parts, hist, seg, cand, ctile_base, total;
    int64_t n_tin, max_tseg;
};

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

Layout layout(int64_t n, int G) {
    Layout L;
    L.n_tin = (n + kTileIn - 1) / kTileIn;
    L.max_tseg = (n + kTileSeg - 1) / kTileSeg + G;
    size_t o = 0;
    L.gstate = o;    o = align256(o + sizeof(GState) * (size_t)G);
    L.cnt = o;       o = align256(o + 4 * (size_t)G * (size_t)L.n_tin);
    L.off = o;       o = align256(o + 8 * (size_t)G * (size_t)L.n_tin);
    L.seg_base = o;  o = align256(o + 8 * (size_t)(G + 1));
    L.tile_base = o; o = align256(o + 8 * (size_t)(G + 1));
    L.parts = o;     o = align256(o + 24 * (size_t)L.max_tseg);
    L.hist = o;      o = align256(o + 4 * (size_t)G * kHist);
    L.seg = o;       o = align256(o + 8 * (size_t)(n > 0 ? n : 1));
    L.cand = o;      o = align256(o + 8 * (size_t)(n > 0 ? n : 1));
    L.ctile_base = o; o = align256(o + 8 * (size_t)(G + 1));
    L.total = o;
    return L;
}

__device__ __forceinline__ uint64_t dbits(double x) { return (uint64_t)__double_as_longlong(x); }
// order-preserving map of non-NaN doubles onto unsigned keys
__device__ __forceinline__ uint64_t okey_bits(uint64_t b) { return (b >> 63) ? ~b : (b | kSign); }
__device__ __forceinline__ uint64_t okey(double x) { return okey_bits(dbits(x)); }
__device__ __forceinline__ double from_okey(uint64_t k) {
    const uint64_t b = (k >> 63) ? (k & ~kSign) : ~k;
    return __longlong_as_double((long long)b);
}
__device__ __forceinline__ bool finite_bits(uint64_t b) { return (b & kExp) != kExp; }
// 0 < p (+inf included, NaN excluded)
__device__ __forceinline__ bool positive_bits(uint64_t b) { return (int64_t)b > 0 && b <= kExp; }

struct U128 {
    unsigned long long lo, hi;
};

// v * 2^64 truncated toward zero as a 128-bit two's complement integer;
// false for non-finite v or |v| >= 2^62
__device__ __forceinline__ bool to_fixed(uint64_t b, U128& r) {
    const int ex = (int)((b >> 52) & 0x7ff);
    if (ex == 0x7ff) return false;
    unsigned long long m = b & 0xfffffffffffffull;
    int e = -1074;
    if (ex != 0) {
        m |= 1ull << 52;
        e = ex - 1075;
    }
    const int s = e + 64;  // fixed = m * 2^s
    unsigned long long lo = 0, hi = 0;
    if (m != 0) {
        if (s > 73) return false;
        if (s >= 64) {
            hi = m << (s - 64);
        } else if (s > 0) {
            lo = m << s;
            hi = m >> (64 - s);
        } else if (s > -64) {
            lo = m >> (-s);
        }
    }
    if (b >> 63) {
        lo = ~lo;
        hi = ~hi;
        lo += 1ull;
        if (lo == 0ull) hi += 1ull;
    }
    r.lo = lo;
    r.hi = hi;
    return true;
}

// 128-bit add through two 64-bit atomics (exact: integer addition commutes)
__device__ __forceinline__ void add128(unsigned long long* lo, unsigned long long* hi, U128 v) {
    const unsigned long long old = atomicAdd(lo, v.lo);
    const unsigned long long carry = (old + v.lo < old) ? 1ull : 0ull;
    if (v.hi + carry) atomicAdd(hi, v.hi + carry);
}

__device__ __forceinline__ double fixed_to_double(unsigned long long lo, unsigned long long hi) {
    const bool neg = (hi >> 63) != 0;
    if (neg) {
        lo = ~lo;
        hi = ~hi;
        lo += 1ull;
        if (lo == 0ull) hi += 1ull;
    }
    const double v = (double)hi + (double)lo * 0x1p-64;
    return neg ? -v : v;
}

// order keys of the requested groups: float64 bit patterns (-0.0 as 0.0)
// for a float column, the integer value for an integer column (valid bit
// clear for a non-integral order).  Orders that are integers in
// [-kLutHalf, kLutHalf] also go into a lookup table (first group wins);
// *s_all_lut says that every valid order is there, so a photon whose order
// is not a small integer matches no group.
constexpr int kLutHalf = 64;

struct OrderLut {
    int16_t g[2 * kLutHalf + 1];
    int all;
};

__device__ void load_orders(const mgpu_stats_problem& P, uint64_t* s_key, uint64_t* s_valid,
                            OrderLut* lut) {
    for (int k = threadIdx.x; k < 2 * kLutHalf + 1; k += blockDim.x) lut->g[k] = -1;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t valid = 0;
        int all = 1;
        for (int k = 0; k < P.n_groups; ++k) {
            const double o = P.orders[k];
            uint64_t key = 0;
            bool ok = true;
            if (P.order_type == MGPU_ORDER_F64) {
                key = dbits(o);
                if (key == kSign) key = 0;
                ok = !isnan(o);
            } else if (P.order_type != MGPU_ORDER_NONE) {
                ok = (o == floor(o)) && fabs(o) < 9.0e18;
                key = ok ? (uint64_t)(long long)o : 0;
            }
            s_key[k] = key;
            if (ok) {
                valid |= 1ull << k;
                if (o == floor(o) && fabs(o) <= (double)kLutHalf) {
                    const int idx = (int)o + kLutHalf;
                    if (lut->g[idx] < 0) lut->g[idx] = (int16_t)k;
                } else {
                    all = 0;
                }
            }
        }
        *s_valid = valid;
        lut->all = all;
    }
    __syncthreads();
}

// a float64 as an integer in [-kLutHalf, kLutHalf] (integer operations):
// false when it is not such an integer
__device__ __forceinline__ bool small_int_bits(uint64_t b, int* v) {
    const uint64_t mag = b & ~kSign;
    if (mag == 0) {
        *v = 0;
        return true;
    }
    const int e = (int)(mag >> 52) - 1023;
    if (e < 0 || e > 6) return false;
    const uint64_t m = (mag & 0xfffffffffffffull) | (1ull << 52);
    const int sh = 52 - e;
    if (m & ((1ull << sh) - 1ull)) return false;
    int x = (int)(m >> sh);
    if (x > kLutHalf) return false;
    *v = (b >> 63) ? -x : x;
    return true;
}

__device__ __forceinline__ uint64_t order_key(const mgpu_stats_problem& P, int64_t i) {
    switch (P.order_type) {
        case MGPU_ORDER_F64: {
            const uint64_t b = dbits(((const double*)P.order)[i * P.order_stride]);
            return b == kSign ? 0 : b;
        }
        case MGPU_ORDER_I32: return (uint64_t)(int64_t)((const int32_t*)P.order)[i * P.order_stride];
        case MGPU_ORDER_I64: return (uint64_t)((const int64_t*)P.order)[i * P.order_stride];
        default: return 0;
    }
}

struct Photon {
    int g;        // group, -1 = none
    bool member;  // counted in n_member
    bool seg;     // finite member: enters the clipping
    bool aeff;    // counted in aeff_sum
    uint64_t vb, pb;
};

__device__ __forceinline__ Photon classify(const mgpu_stats_problem& P, int64_t i,
                                           const uint64_t* s_key, uint64_t valid,
                                           const OrderLut* lut) {
    Photon ph{-1, false, false, false, 0ull, 0ull};
    if (i >= P.n) return ph;
    int g = -1;
    if (P.order_type == MGPU_ORDER_NONE) {
        g = 0;
    } else {
        const uint64_t key = order_key(P, i);
        int v;
        bool small;
        if (P.order_type == MGPU_ORDER_F64) {
            small = small_int_bits(key, &v);
        } else {
            const int64_t iv = (int64_t)key;
            small = iv >= -kLutHalf && iv <= kLutHalf;
            v = (int)iv;
        }
        // a small integer can only equal an order in the table
        if (small) {
            g = lut->g[v + kLutHalf];
        } else if (!lut->all) {
            for (int k = P.n_groups - 1; k >= 0; --k)
                if (((valid >> k) & 1ull) && s_key[k] == key) g = k;
        }
    }
    if (g < 0) return ph;
    ph.g = g;
    ph.vb = dbits(P.value.ptr[i * P.value.stride]);
    ph.pb = P.prob.ptr ? dbits(P.prob.ptr[i * P.prob.stride]) : 0x3ff0000000000000ull;
    const bool fin = finite_bits(ph.vb);
    ph.member = (P.flags & MGPU_STATS_RES_FILTER) ? (fin && positive_bits(ph.pb)) : true;
    ph.seg = ph.member && fin;
    ph.aeff = P.aeff_mask ? (P.aeff_mask[i] != 0) : true;
    return ph;
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---------------------------------------------------------------- grouping
// Per tile: finite members per group (-> cnt).  Per group (block
// accumulators, then global atomics): members, the key range of the finite
// members and the fixed-point probability sum.
__global__ void __launch_bounds__(kThreads)
classify_kernel(const __grid_constant__ mgpu_stats_problem P, Work W) {
    __shared__ uint64_t s_key[kG];
    __shared__ uint64_t s_valid;
    __shared__ OrderLut s_lut;
    __shared__ int32_t tcnt[kG];
    __shared__ unsigned long long s_mem[kG], s_lo[kG], s_hi[kG], s_kmin_inv[kG], s_kmax[kG];
    __shared__ uint32_t s_flags[kG];
    const int G = P.n_groups;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = threadIdx.x; k < kG; k += kThreads) {
        tcnt[k] = 0;
        s_mem[k] = s_lo[k] = s_hi[k] = s_kmin_inv[k] = s_kmax[k] = 0ull;
        s_flags[k] = 0u;
    }
    load_orders(P, s_key, &s_valid, &s_lut);
    const uint64_t valid = s_valid;
    for (int64_t t = blockIdx.x; t < W.n_tin; t += gridDim.x) {
        const int64_t base = t * kTileIn + (int64_t)w * (kPerLane * 32);
        for (int k = 0; k < kPerLane; ++k) {
            const Photon ph = classify(P, base + k * 32 + lane, s_key, valid, &s_lut);
            const unsigned sp = __match_any_sync(MGPU_FULL_MASK, ph.seg ? ph.g : -1);
            if (ph.seg && lane == __ffs(sp) - 1) atomicAdd(&tcnt[ph.g], __popc(sp));
            const unsigned mp = __match_any_sync(MGPU_FULL_MASK, ph.member ? ph.g : -1);
            if (ph.member && lane == __ffs(mp) - 1)
                atomicAdd(&s_mem[ph.g], (unsigned long long)__popc(mp));
            if (ph.seg) {
                const uint64_t key = okey_bits(ph.vb);
                atomicMax(&s_kmin_inv[ph.g], (unsigned long long)~key);
                atomicMax(&s_kmax[ph.g], (unsigned long long)key);
            }
            if (ph.g >= 0 && ph.aeff) {
                U128 v;
                if (to_fixed(ph.pb, v)) {
                    if (v.lo | v.hi) add128(&s_lo[ph.g], &s_hi[ph.g], v);
                } else {
                    const uint32_t f = ((ph.pb & ~kSign) > kExp) ? 1u           // NaN
                                       : ((ph.pb & ~kSign) == kExp) ? ((ph.pb >> 63) ? 4u : 2u)
                                                                    : 1u;       // too large
                    atomicOr(&s_flags[ph.g], f);
                }
            }
        }
        __syncthreads();
        for (int g = threadIdx.x; g < G; g += kThreads) {
            W.cnt[(int64_t)g * W.n_tin + t] = tcnt[g];
            tcnt[g] = 0;
        }
        __syncthreads();
    }
    for (int g = threadIdx.x; g < G; g += kThreads) {
        GState& s = W.gs[g];
        if (s_mem[g]) atomicAdd(&s.n_member, s_mem[g]);
        if (s_lo[g] | s_hi[g]) add128(&s.aeff_lo, &s.aeff_hi, U128{s_lo[g], s_hi[g]});
        if (s_flags[g]) atomicOr(&s.aeff_flags, s_flags[g]);
        if (s_kmin_inv[g]) atomicMax(&s.kmin_inv, s_kmin_inv[g]);
        if (s_kmax[g]) atomicMax(&s.kmax, s_kmax[g]);
    }
}

// one block per group: exclusive scan of the group's tile counts
__global__ void __launch_bounds__(kThreads)
scan_kernel(Work W) {
    __shared__ int64_t tsum[kThreads];
    const int g = blockIdx.x;
    const int64_t n = W.n_tin;
    const int64_t per = (n + kThreads - 1) / kThreads;
    const int64_t a = threadIdx.x * per, b = min(n, a + per);
    const int32_t* c = W.cnt + (int64_t)g * n;
    int64_t s = 0;
    for (int64_t t = a; t < b; ++t) s += c[t];
    tsum[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t run = 0;
        for (int k = 0; k < kThreads; ++k) {
            const int64_t v = tsum[k];
            tsum[k] = run;
            run += v;
        }
        W.gs[g].n_finite = run;
    }
    __syncthreads();
    int64_t run = tsum[threadIdx.x];
    int64_t* o = W.off + (int64_t)g * n;
    for (int64_t t = a; t < b; ++t) {
        o[t] = run;
        run += c[t];
    }
}

__device__ void write_result(const mgpu_stats_problem& P, const GState& s, int g, double mean,
                             double med, double sd, int64_t n_clip) {
    double* r = P.result + (int64_t)g * MGPU_STATS_NRES;
    r[MGPU_STATS_MEAN] = mean;
    r[MGPU_STATS_MEDIAN] = med;
    r[MGPU_STATS_STD] = sd;
    r[MGPU_STATS_N_CLIP] = (double)n_clip;
    r[MGPU_STATS_N_MEMBER] = (double)s.n_member;
    r[MGPU_STATS_AEFF] = s.aeff;
    r[MGPU_STATS_N_FINITE] = (double)s.n_finite;
    r[MGPU_STATS_ROUNDS] = (double)s.round;
}

// int32 -> float32 by bit construction (truncated toward zero); the
// hardware conversion issues on the FP64 pipe of this GPU
__device__ __forceinline__ float i2f_int(int32_t v) {
    if (v == 0) return 0.0f;
    const uint32_t sign = v < 0 ? 0x80000000u : 0u;
    const uint32_t m = v < 0 ? (uint32_t)(-(int64_t)v) : (uint32_t)v;
    const int e = 31 - __clz(m);
    const uint32_t mant = e > 23 ? (m >> (e - 23)) : (m << (23 - e));
    return __uint_as_float(sign | ((uint32_t)(e + 127) << 23) | (mant & 0x7fffffu));
}

// float64 -> float-float on the integer pipe: hi = d rounded to float32,
// lo = the rest truncated to float32 (2^-47 relative); d finite with
// 2^-74 <= |d| < 2^127 (smaller magnitudes give lo = 0)
__device__ __forceinline__ ff d2ff_int(double d) {
    const float hi = d2f_bits(d);
    const uint32_t dhi = mgpu_dhi(d), dlo = mgpu_dlo(d);
    const uint32_t e = (dhi >> 20) & 0x7ffu;
    if (e < 949u || e > 1150u) return ff{hi, 0.0f};
    int32_t rem = (int32_t)(dlo & 0x1fffffffu);
    const uint32_t trunc = (((dhi << 3) | (dlo >> 29)) - 0xC0000000u) & 0x7fffffffu;
    if ((mgpu_f2u(hi) & 0x7fffffffu) != trunc) rem -= 0x20000000;   // hi was rounded up
    float lo = i2f_int(rem) * __uint_as_float((e - 948u) << 23);      // 2^(e - 1075)
    if (dhi & 0x80000000u) lo = -lo;
    return ff{hi, lo};
}

// Shifted sums in float-float: d = x - c is formed in float64 (exact for
// x within a factor two of c), split into float-float (2^-48 relative) and
// summed on the float32 pipes.  Used when the kept deviations |x - c| <= D
// satisfy D = 0 or 2^-60 <= D <= 2^60: the float32 parts neither overflow
// nor drop deviations that matter next to D.
__device__ void choose_sums(GState& s) {
    const double a = fabs(from_okey(s.klo) - s.c), b = fabs(from_okey(s.khi) - s.c);
    const double D = a > b ? a : b;
    s.use_ff = (D == 0.0 || (D >= 0x1p-60 && D <= 0x1p60)) ? 1 : 0;
}

// First level of the median selection, in the value domain: bins linear
// in x over [vlo, vhi] (kVBins - 2 inner bins; bin 0 and kVBins - 1 also take
// what lies below and above).  The bin is formed in float32 from the
// float64 deviation d = x - c, a monotone map of x, so the kept values of
// a bin interval are a contiguous run of the sorted values.
__device__ void set_value_bins(GState& s, double vlo, double vhi) {
    const double range = vhi - vlo;
    const double inv = (double)(kVBins - 2) / range;
    const bool ok = isfinite(vlo) && isfinite(vhi) && range > 0.0 && isfinite(inv) &&
                    inv < 1e37;
    s.voff = ok ? __double2float_rn(vlo - s.c) : 0.0f;
    s.vinv = ok ? __double2float_rn(inv) : 0.0f;
}

__device__ __forceinline__ int value_bin(double d, float voff, float vinv) {
    if (vinv == 0.0f) return 1;
    const float t = (d2f_bits(d) - voff) * vinv;
    if (!(t >= 0.0f)) return 0;
    if (t >= (float)(kVBins - 2)) return kVBins - 1;
    return (int)t + 1;
}

// the selection state at the start of a round: the value level comes first
__device__ void start_selection(GState& s) {
    s.pref[0] = s.pref[1] = 0ull;
    s.pb = 0;
    s.split = 0;
    s.sel_done = 0;
}

// segment bases, tile bases, effective areas and the round-0 state of every group
__global__ void setup_kernel(const __grid_constant__ mgpu_stats_problem P, Work W) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int G = P.n_groups;
    int64_t run = 0, trun = 0;
    for (int g = 0; g < G; ++g) {
        GState& s = W.gs[g];
        W.seg_base[g] = run;
        W.tile_base[g] = trun;
        run += s.n_finite;
        trun += (s.n_finite + kTileSeg - 1) / kTileSeg;
        const uint32_t f = s.aeff_flags;
        s.aeff = (f & 1u) || ((f & 6u) == 6u) ? kNaN
                 : (f & 2u) ? INFINITY : (f & 4u) ? -INFINITY : fixed_to_double(s.aeff_lo, s.aeff_hi);
        s.klo = ~s.kmin_inv;
        s.khi = s.kmax;
        start_selection(s);
        s.n_prev = -1;
        s.round = 0;
        s.final_ = 0;
        s.bad = 0;
        s.active = (s.n_finite > 0 && !(P.flags & MGPU_STATS_AEFF_ONLY)) ? 1 : 0;
        if (!s.active) write_result(P, s, g, kNaN, kNaN, kNaN, 0);
    }
    W.seg_base[G] = run;
    W.tile_base[G] = trun;
}

// stable scatter of the finite members into their group's segment
__global__ void __launch_bounds__(kThreads)
scatter_kernel(const __grid_constant__ mgpu_stats_problem P, Work W) {
    __shared__ uint64_t s_key[kG];
    __shared__ uint64_t s_valid;
    __shared__ OrderLut s_lut;
    __shared__ int32_t wcnt[kWarps][kG];
    __shared__ int64_t wbase[kWarps][kG];
    const int G = P.n_groups;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = threadIdx.x; k < kWarps * kG; k += kThreads) (&wcnt[0][0])[k] = 0;
    load_orders(P, s_key, &s_valid, &s_lut);
    const uint64_t valid = s_valid;
    for (int64_t t = blockIdx.x; t < W.n_tin; t += gridDim.x) {
        const int64_t base = t * kTileIn + (int64_t)w * (kPerLane * 32);
        int gk[kPerLane];
        uint64_t vk[kPerLane];
        unsigned pk[kPerLane];
#pragma unroll
        for (int k = 0; k < kPerLane; ++k) {
            const Photon ph = classify(P, base + k * 32 + lane, s_key, valid, &s_lut);
            gk[k] = ph.seg ? ph.g : -1;
            vk[k] = ph.vb;
            pk[k] = __match_any_sync(MGPU_FULL_MASK, gk[k]);
            if (gk[k] >= 0 && lane == __ffs(pk[k]) - 1) wcnt[w][gk[k]] += __popc(pk[k]);
            __syncwarp();
        }
        __syncthreads();
        for (int g = threadIdx.x; g < G; g += kThreads) {
            int64_t run = W.seg_base[g] + W.off[(int64_t)g * W.n_tin + t];
#pragma unroll
            for (int ww = 0; ww < kWarps; ++ww) {
                wbase[ww][g] = run;
                run += wcnt[ww][g];
                wcnt[ww][g] = 0;
            }
        }
        __syncthreads();
        const unsigned lt = lanemask_lt();
#pragma unroll
        for (int k = 0; k < kPerLane; ++k) {
            const int g = gk[k];
            if (g >= 0)
                W.seg[wbase[w][g] + __popc(pk[k] & lt)] = __longlong_as_double((long long)vk[k]);
            __syncwarp();
            if (g >= 0 && lane == __ffs(pk[k]) - 1) wbase[w][g] += __popc(pk[k]);
            __syncwarp();
        }
        __syncthreads();
    }
}

// the first clipping round's centre: the median of the group's first values (a robust
// guess of the mean keeps the shifted sums well conditioned)
__global__ void center_kernel(Work W) {
    if (threadIdx.x != 0) return;
    GState& s = W.gs[blockIdx.x];
    if (!s.active) return;
    const int m = (int)min((int64_t)kCenterSample, s.n_finite);
    double v[kCenterSample];
    const double* seg = W.seg + W.seg_base[blockIdx.x];
    for (int j = 0; j < m; ++j) {
        const double x = seg[j];
        int k = j;
        while (k > 0 && v[k - 1] > x) {
            v[k] = v[k - 1];
            --k;
        }
        v[k] = x;
    }
    s.c = v[m / 2];
    choose_sums(s);
    // the first clipping round's value bins: the sample median -/+ 4 interquartile ranges,
    // or the group's whole range when the sample has no spread
    const double w = 4.0 * (v[(3 * m) / 4] - v[m / 4]);
    if (w > 0.0 && isfinite(w)) set_value_bins(s, s.c - w, s.c + w);
    else set_value_bins(s, from_okey(s.klo), from_okey(s.khi));
}

// ---------------------------------------------------------------- clipping
__device__ __forceinline__ bool seg_tile(const Work& W, int G, int64_t t, int& g, int64_t& a,
                                         int64_t& b) {
    if (t >= W.tile_base[G]) return false;
    // the last group whose first tile is at or before t (groups without
    // tiles share their base with the next group and are passed over)
    int lo = 0;
    for (int k = 1; k < G; ++k)
        if (W.tile_base[k] <= t) lo = k;
    g = lo;
    a = W.seg_base[g] + (t - W.tile_base[g]) * kTileSeg;
    b = min(W.seg_base[g + 1], a + kTileSeg);
    return true;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(MGPU_FULL_MASK, v, o);
    return v;
}

// The kept values of one tile: count, shifted sums (float-float when kFF)
// and the first-digit histogram (when sel).  The caller branches on the
// group's mode outside the loop, so each loop carries one kind of sum.
template <bool kFF>
__device__ __forceinline__ void stats_loop(const Work& W, int64_t a, int64_t b, uint64_t klo,
                                           uint64_t khi, double c, bool sel, float voff,
                                           float vinv, uint32_t* h, long long& cnt, double& s1,
                                           double& s2) {
    const int lane = threadIdx.x & 31;
    ff f1{0.0f, 0.0f}, f2{0.0f, 0.0f};
#pragma unroll 4
    for (int k = 0; k < kSegPerThread; ++k) {
        const int64_t i = a + (int64_t)k * kThreads + threadIdx.x;
        int bin = -1;
        if (i < b) {
            const double x = W.seg[i];
            const uint64_t key = okey(x);
            if (key >= klo && key <= khi) {
                ++cnt;
                const double d = x - c;
                if (kFF) {
                    const ff df = d2ff_int(d);
                    f1 = ff_add(f1, df);
                    f2 = ff_add(f2, ff_mul(df, df));
                } else {
                    s1 += d;
                    s2 = fma(d, d, s2);
                }
                if (sel) bin = value_bin(d, voff, vinv);
            }
        }
        if (sel) {
            const unsigned act = __ballot_sync(MGPU_FULL_MASK, bin >= 0);
            if (bin >= 0) {
                const unsigned peers = __match_any_sync(act, bin);
                if (lane == __ffs(peers) - 1) atomicAdd(h + bin, (uint32_t)__popc(peers));
            }
        }
    }
    if (kFF) {
        s1 = ff2d(f1);
        s2 = ff2d(f2);
    }
}

// One pass per clipping round over a tile of kept values: the count and the
// shifted sums (for the mean and the variance) and the histogram of the
// first radix digit of the kept values that carry each selection's prefix.
__global__ void __launch_bounds__(kThreads)
round_pass(Work W, int G) {
    __shared__ uint32_t h[1][kVBins];
    __shared__ double s_s1[kWarps], s_s2[kWarps];
    __shared__ long long s_cnt[kWarps];
    int g;
    int64_t a, b;
    if (!seg_tile(W, G, blockIdx.x, g, a, b)) return;
    const GState& s = W.gs[g];
    if (!s.active) return;
    const bool sel = !s.sel_done;
    if (sel) {
        for (int k = threadIdx.x; k < kVBins; k += kThreads) h[0][k] = 0u;
        __syncthreads();
    }
    long long cnt = 0;
    double s1 = 0.0, s2 = 0.0;
    if (s.use_ff)
        stats_loop<true>(W, a, b, s.klo, s.khi, s.c, sel, s.voff, s.vinv, &h[0][0], cnt, s1, s2);
    else
        stats_loop<false>(W, a, b, s.klo, s.khi, s.c, sel, s.voff, s.vinv, &h[0][0], cnt, s1,
                          s2);
    const int lane = threadIdx.x & 31;
    if (sel) {
        __syncthreads();
        uint32_t* gh = W.hist + (int64_t)g * kHist;
        for (int k = threadIdx.x; k < kVBins; k += kThreads) {
            const uint32_t v = (&h[0][0])[k];
            if (v) atomicAdd(gh + k, v);
        }
    }
    cnt = warp_sum(cnt);
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    if (lane == 0) {
        s_cnt[threadIdx.x >> 5] = cnt;
        s_s1[threadIdx.x >> 5] = s1;
        s_s2[threadIdx.x >> 5] = s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < kWarps; ++k) {
            cnt += s_cnt[k];
            s1 += s_s1[k];
            s2 += s_s2[k];
        }
        double* p = W.parts + 3 * (int64_t)blockIdx.x;
        p[0] = (double)cnt;
        p[1] = s1;
        p[2] = s2;
    }
}

// After the first digit: copy the keys of the kept values that still carry
// either selection's prefix into the group's candidate list (order does not
// matter to a selection; one atomic per warp).
__global__ void __launch_bounds__(kThreads)
compact_pass(Work W, int G) {
    int g;
    int64_t a, b;
    if (!seg_tile(W, G, blockIdx.x, g, a, b)) return;
    GState& s = W.gs[g];
    if (!s.active || s.sel_done) return;
    const int b0 = s.vb[0], b1 = s.vb[1];
    const double c = s.c;
    const float voff = s.voff, vinv = s.vinv;
    const uint64_t klo = s.klo, khi = s.khi;
    uint64_t* out = W.cand + W.seg_base[g];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __shared__ unsigned long long s_base[kWarps];
    // count (one bit per value of this thread), one atomic per tile, write
    uint32_t mine = 0;
    unsigned total = 0;
    unsigned long long kmn_inv = 0ull, kmx = 0ull;
#pragma unroll 8
    for (int k = 0; k < kSegPerThread; ++k) {
        const int64_t i = a + (int64_t)k * kThreads + threadIdx.x;
        bool want = false;
        if (i < b) {
            const double x = W.seg[i];
            const uint64_t key = okey(x);
            if (key >= klo && key <= khi) {
                const int vb = value_bin(x - c, voff, vinv);
                want = vb >= b0 && vb <= b1;
                if (want) {
                    kmn_inv = max(kmn_inv, (unsigned long long)~key);
                    kmx = max(kmx, (unsigned long long)key);
                }
            }
        }
        mine |= (want ? 1u : 0u) << k;
        total += __popc(__ballot_sync(MGPU_FULL_MASK, want));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        kmn_inv = max(kmn_inv, __shfl_xor_sync(MGPU_FULL_MASK, kmn_inv, o));
        kmx = max(kmx, __shfl_xor_sync(MGPU_FULL_MASK, kmx, o));
    }
    if (lane == 0) {
        s_base[w] = total;
        if (kmx) {
            atomicMax(&s.cmin_inv, kmn_inv);
            atomicMax(&s.cmax, kmx);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long run = 0;
        for (int k = 0; k < kWarps; ++k) {
            const unsigned long long c = s_base[k];
            s_base[k] = run;
            run += c;
        }
        const unsigned long long base = run ? atomicAdd(&s.n_cand, run) : 0ull;
        for (int k = 0; k < kWarps; ++k) s_base[k] += base;
    }
    __syncthreads();
    unsigned long long pos = s_base[w];
    const unsigned lt = lanemask_lt();
    for (int k = 0; k < kSegPerThread; ++k) {
        const bool want = (mine >> k) & 1u;
        const unsigned m = __ballot_sync(MGPU_FULL_MASK, want);
        if (want) {
            const int64_t i = a + (int64_t)k * kThreads + threadIdx.x;
            out[pos + __popc(m & lt)] = okey(W.seg[i]);
        }
        pos += __popc(m);
    }
}

// Groups whose candidate list is short: one block runs every remaining
// digit (shared-memory histogram with warp-aggregated updates, block-wide
// rank search) and leaves the group resolved, with no launch per digit;
// longer lists go through cand_pass + radix_step.  Runs after cand_setup
// (the prefix already spans the candidates' common bits).
constexpr int64_t kSmallCand = 3072;      // keys staged in shared memory (24 KB)

__device__ void find_rank(const uint32_t* hist, int64_t r, int64_t* s_tot, int* out_bin,
                          int64_t* out_below);

__global__ void __launch_bounds__(kThreads)
select_small(Work W) {
    __shared__ uint32_t h[2][kBins];
    __shared__ uint64_t keys[kSmallCand];
    __shared__ int64_t s_tot[kThreads];
    __shared__ int s_bin;
    __shared__ int64_t s_below;
    GState& s = W.gs[blockIdx.x];
    if (!s.active || s.sel_done) return;
    const int64_t nc = (int64_t)s.n_cand;
    if (nc > kSmallCand) return;
    {
        const uint64_t* src = W.cand + W.seg_base[blockIdx.x];
        for (int64_t j = threadIdx.x; j < nc; j += kThreads) keys[j] = src[j];
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    for (int level = 0; level < kLevels; ++level) {
        if (s.sel_done) break;                     // uniform: read after the barrier below
        const int pb = s.pb;
        const int width = min(kRadixBits, 64 - pb);
        const int shift = 64 - pb - width;
        const uint64_t dmask = (1ull << width) - 1ull;
        const uint64_t pa = pb ? (s.pref[0] >> (64 - pb)) : 0ull;
        const uint64_t pbv = pb ? (s.pref[1] >> (64 - pb)) : 0ull;
        const bool split = s.split != 0;
        for (int k = threadIdx.x; k < 2 * kBins; k += kThreads) (&h[0][0])[k] = 0u;
        __syncthreads();
        for (int64_t j0 = 0; j0 < nc; j0 += kThreads) {
            const int64_t j = j0 + threadIdx.x;
            int bin = -1;
            if (j < nc) {
                const uint64_t key = keys[j];
                const uint64_t top = pb ? (key >> (64 - pb)) : 0ull;
                const int digit = (int)((key >> shift) & dmask);
                if (top == pa) bin = digit;
                else if (split && top == pbv) bin = kBins + digit;
            }
            const unsigned act = __ballot_sync(MGPU_FULL_MASK, bin >= 0);
            if (bin >= 0) {
                const unsigned peers = __match_any_sync(act, bin);
                if (lane == __ffs(peers) - 1) atomicAdd(&(&h[0][0])[bin], (uint32_t)__popc(peers));
            }
        }
        __syncthreads();
        int bins[2] = {0, 0};
        bool lost = false;
        for (int q = 0; q < (s.two ? 2 : 1); ++q) {
            find_rank(&h[(split && q == 1) ? 1 : 0][0], s.rank[q], s_tot, &s_bin, &s_below);
            bins[q] = s_bin;
            lost = lost || s_bin < 0;
            if (threadIdx.x == 0 && s_bin >= 0) {
                s.rank[q] -= s_below;
                s.pref[q] |= (uint64_t)s_bin << shift;
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            if (lost) {
                s.bad = 1;
                s.pb = 64;
                s.sel_done = 1;
            } else {
                if (!s.two) {
                    s.pref[1] = s.pref[0];
                    s.rank[1] = s.rank[0];
                } else if (!split && bins[0] != bins[1]) {
                    s.split = 1;
                }
                s.pb = pb + width;
                s.sel_done = s.pb >= 64 ? 1 : 0;
            }
        }
        __syncthreads();
    }
}

// tiles of the candidate lists (one thread); before them, every key bit
// the candidates share is known: the prefix jumps to their common prefix
// (one selection, or two not yet split), so the next digits split the
// candidates' actual spread
__global__ void cand_setup(Work W, int G) {
    if (threadIdx.x != 0) return;
    int64_t run = 0;
    for (int g = 0; g < G; ++g) {
        W.ctile_base[g] = run;
        GState& s = W.gs[g];
        if (s.active && !s.sel_done) {
            if (s.n_cand == 0) {
                s.bad = 1;          // cannot happen for a consistent state
                s.pb = 64;
                s.sel_done = 1;
            } else {
                const uint64_t mn = ~s.cmin_inv, mx = s.cmax;
                const int cp = (mn == mx) ? 64 : __clzll((long long)(mn ^ mx));
                const uint64_t mask = cp == 0 ? 0ull : (cp == 64 ? ~0ull : (~0ull << (64 - cp)));
                s.pref[0] = s.pref[1] = mn & mask;
                s.pb = cp;
                s.split = 0;
                s.sel_done = cp == 64 ? 1 : 0;
            }
        }
        if (s.active && !s.sel_done && (int64_t)s.n_cand > kSmallCand)
            run += ((int64_t)s.n_cand + kTileSeg - 1) / kTileSeg;
    }
    W.ctile_base[G] = run;
}

// later digits over the candidate lists: a persistent grid walks the
// candidate tiles of every group
__global__ void __launch_bounds__(kThreads)
cand_pass(Work W, int G) {
    __shared__ uint32_t h[2][kBins];
    const int64_t total = W.ctile_base[G];
    const int lane = threadIdx.x & 31;
    for (int64_t t = blockIdx.x; t < total; t += gridDim.x) {
        int g = 0;
        for (int k = 1; k < G; ++k)
            if (W.ctile_base[k] <= t) g = k;
        const GState& s = W.gs[g];
        if (!s.active || s.sel_done || (int64_t)s.n_cand <= kSmallCand) continue;
        const int pb = s.pb;
        const int width = min(kRadixBits, 64 - pb);
        const int shift = 64 - pb - width;
        const uint64_t dmask = (1ull << width) - 1ull;
        const uint64_t pa = pb ? (s.pref[0] >> (64 - pb)) : 0ull;
        const uint64_t pbv = pb ? (s.pref[1] >> (64 - pb)) : 0ull;
        const bool split = s.split != 0;
        const int64_t a = W.seg_base[g] + (t - W.ctile_base[g]) * kTileSeg;
        const int64_t b = min(W.seg_base[g] + (int64_t)s.n_cand, a + kTileSeg);
        for (int k = threadIdx.x; k < 2 * kBins; k += kThreads) (&h[0][0])[k] = 0u;
        __syncthreads();
#pragma unroll 4
        for (int k = 0; k < kSegPerThread; ++k) {
            const int64_t i = a + (int64_t)k * kThreads + threadIdx.x;
            int bin = -1;
            if (i < b) {
                const uint64_t key = W.cand[i];
                const uint64_t top = pb ? (key >> (64 - pb)) : 0ull;
                const int digit = (int)((key >> shift) & dmask);
                if (top == pa) bin = digit;
                else if (split && top == pbv) bin = kBins + digit;
            }
            const unsigned act = __ballot_sync(MGPU_FULL_MASK, bin >= 0);
            if (bin >= 0) {
                const unsigned peers = __match_any_sync(act, bin);
                if (lane == __ffs(peers) - 1) atomicAdd(&(&h[0][0])[bin], (uint32_t)__popc(peers));
            }
        }
        __syncthreads();
        uint32_t* gh = W.hist + (int64_t)g * kHist;
        for (int k = threadIdx.x; k < (split ? 2 : 1) * kBins; k += kThreads) {
            const uint32_t v = (&h[0][0])[k];
            if (v) atomicAdd(gh + k, v);
        }
        __syncthreads();
    }
}

// block-wide search of the bin holding rank r in an NB-bin histogram: returns
// (bin, count of values in lower bins) through shared memory; bin -1 if the
// histogram holds fewer than r + 1 values
template <int NB>
__device__ void find_rank_n(const uint32_t* hist, int64_t r, int64_t* s_tot, int* out_bin,
                            int64_t* out_below) {
    constexpr int per = NB / kThreads;
    if (threadIdx.x == 0) *out_bin = -1;
    int64_t loc = 0;
    uint32_t v[per];
#pragma unroll
    for (int k = 0; k < per; ++k) {
        v[k] = hist[threadIdx.x * per + k];
        loc += v[k];
    }
    s_tot[threadIdx.x] = loc;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t run = 0;
        for (int k = 0; k < kThreads; ++k) {
            const int64_t t = s_tot[k];
            s_tot[k] = run;
            run += t;
        }
    }
    __syncthreads();
    int64_t below = s_tot[threadIdx.x];
#pragma unroll
    for (int k = 0; k < per; ++k) {
        if (below <= r && r < below + (int64_t)v[k]) {
            *out_bin = threadIdx.x * per + k;
            *out_below = below;
        }
        below += v[k];
    }
    __syncthreads();
}

__device__ void find_rank(const uint32_t* hist, int64_t r, int64_t* s_tot, int* out_bin,
                          int64_t* out_below) {
    find_rank_n<kBins>(hist, r, s_tot, out_bin, out_below);
}

// one block per group: (kStats) count, mean and std of the kept values and
// the ranks of the median; then one radix level of both selections
template <bool kStats>
__global__ void __launch_bounds__(kThreads)
radix_step(const __grid_constant__ mgpu_stats_problem P, Work W) {
    __shared__ int64_t s_tot[kThreads];
    __shared__ double s_s1[kThreads], s_s2[kThreads];
    __shared__ long long s_cnt[kThreads];
    __shared__ int s_bin;
    __shared__ int64_t s_below;
    const int g = blockIdx.x;
    GState& s = W.gs[g];
    if (!s.active) return;
    if (kStats) {
        const int64_t t0 = W.tile_base[g], t1 = W.tile_base[g + 1];
        double s1 = 0.0, s2 = 0.0;
        long long c = 0;
        for (int64_t t = t0 + threadIdx.x; t < t1; t += kThreads) {
            const double* p = W.parts + 3 * t;
            c += (long long)p[0];
            s1 += p[1];
            s2 += p[2];
        }
        s_cnt[threadIdx.x] = c;
        s_s1[threadIdx.x] = s1;
        s_s2[threadIdx.x] = s2;
        for (int st = kThreads / 2; st > 0; st >>= 1) {
            __syncthreads();
            if (threadIdx.x < st) {
                s_cnt[threadIdx.x] += s_cnt[threadIdx.x + st];
                s_s1[threadIdx.x] += s_s1[threadIdx.x + st];
                s_s2[threadIdx.x] += s_s2[threadIdx.x + st];
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const int64_t n = s_cnt[0];
            s.n_cur = n;
            s.final_ = (s.round > 0 && n == s.n_prev) || s.round >= P.maxiters;
            if (n == 0) {
                // nothing left inside the bounds: the statistics of an empty set
                write_result(P, s, g, kNaN, kNaN, kNaN, 0);
                s.active = 0;
            } else {
                const double m1 = s_s1[0] / (double)n;
                s.mean = s.c + m1;
                const double var = s_s2[0] / (double)n - m1 * m1;
                s.stdev = sqrt(var > 0.0 ? var : 0.0);
                s.two = (n % 2 == 0) ? 1 : 0;
                s.rank[1] = n / 2;
                s.rank[0] = s.two ? n / 2 - 1 : n / 2;
                s.n_cand = 0ull;
                s.cmin_inv = 0ull;
                s.cmax = 0ull;
            }
        }
        __syncthreads();
        if (!s.active) return;
        // the value level: the bins of both ranks, ranks counted from the
        // first of them (the candidates are the kept values of bins
        // vb[0]..vb[1]); the key digits follow on the candidates
        uint32_t* gh = W.hist + (int64_t)g * kHist;
        int vbs[2] = {0, 0};
        int64_t below0 = 0;
        bool lost = false;
        for (int q = 0; q < (s.two ? 2 : 1); ++q) {
            find_rank_n<kVBins>(gh, s.rank[q], s_tot, &s_bin, &s_below);
            vbs[q] = s_bin;
            if (q == 0) below0 = s_below;
            lost = lost || s_bin < 0;
            __syncthreads();       // every thread has read s_bin before the next search
        }
        if (threadIdx.x == 0) {
            if (lost) {
                s.bad = 1;
                s.pb = 64;
                s.sel_done = 1;
            } else {
                s.vb[0] = vbs[0];
                s.vb[1] = s.two ? vbs[1] : vbs[0];
                s.rank[0] -= below0;
                s.rank[1] = s.two ? s.rank[1] - below0 : s.rank[0];
            }
        }
        for (int k = threadIdx.x; k < kHist; k += kThreads) gh[k] = 0u;
        return;
    }
    if (s.sel_done) return;
    const int pb = s.pb;
    const int width = min(kRadixBits, 64 - pb);
    const int shift = 64 - pb - width;
    uint32_t* gh = W.hist + (int64_t)g * kHist;
    const bool split = s.split != 0;
    int bins[2] = {0, 0};
    bool lost = false;
    for (int q = 0; q < (s.two ? 2 : 1); ++q) {
        const uint32_t* src = gh + ((split && q == 1) ? kBins : 0);
        find_rank(src, s.rank[q], s_tot, &s_bin, &s_below);
        bins[q] = s_bin;
        lost = lost || s_bin < 0;
        if (threadIdx.x == 0 && s_bin >= 0) {
            s.rank[q] -= s_below;
            s.pref[q] |= (uint64_t)s_bin << shift;
        }
        __syncthreads();
    }
    if (lost) {
        // the histogram does not hold the rank (cannot happen for a
        // consistent state): report NaN rather than a wrong median
        if (threadIdx.x == 0) {
            s.bad = 1;
            s.pb = 64;
            s.sel_done = 1;
        }
    } else if (threadIdx.x == 0) {
        if (!s.two) {
            s.pref[1] = s.pref[0];
            s.rank[1] = s.rank[0];
        } else if (!split && bins[0] != bins[1]) {
            s.split = 1;
        }
        s.pb = pb + width;
        s.sel_done = s.pb >= 64 ? 1 : 0;
    }
    for (int k = threadIdx.x; k < 2 * kBins; k += kThreads) gh[k] = 0u;
}

// median and next bounds (or the result) of every active group
__global__ void finalize_round(const __grid_constant__ mgpu_stats_problem P, Work W) {
    const int g = threadIdx.x;
    if (g >= P.n_groups) return;
    GState& s = W.gs[g];
    if (!s.active) return;
    const double a = from_okey(s.pref[0]);
    const double med = s.bad ? kNaN : (s.two ? (a + from_okey(s.pref[1])) / 2.0 : a);
    if (s.final_) {
        write_result(P, s, g, s.mean, med, s.stdev, s.n_cur);
        s.active = 0;
        return;
    }
    const double lo = med - s.stdev * P.sigma;
    const double hi = med + s.stdev * P.sigma;
    if (isnan(lo) || isnan(hi)) {
        s.klo = ~0ull;   // nothing is kept
        s.khi = 0ull;
    } else {
        // -0.0 and 0.0 compare equal: the lower bound takes the smaller key
        // of the two, the upper bound the larger
        s.klo = okey(lo == 0.0 ? -0.0 : lo);
        s.khi = okey(hi == 0.0 ? 0.0 : hi);
    }
    start_selection(s);
    s.c = isnan(med) ? 0.0 : med;
    choose_sums(s);
    set_value_bins(s, lo, hi);
    s.n_prev = s.n_cur;
    s.round += 1;
}

}  // namespace

extern "C" int64_t mgpu_order_stats_workspace(int64_t n, int32_t n_groups) {
    if (n < 0 || n_groups < 1 || n_groups > MGPU_STATS_MAX_GROUPS) return -1;
    return (int64_t)layout(n, n_groups).total;
}

extern "C" int mgpu_order_stats(const mgpu_stats_problem* prob, void* stream) {
    if (prob == nullptr) return (int)cudaErrorInvalidValue;
    const mgpu_stats_problem& P = *prob;
    const int G = P.n_groups;
    if (P.n < 0 || G < 1 || G > MGPU_STATS_MAX_GROUPS || P.maxiters < 1 || !P.result ||
        !P.work || (P.n > 0 && !P.value.ptr))
        return (int)cudaErrorInvalidValue;
    if (P.order_type != MGPU_ORDER_NONE && P.order_type != MGPU_ORDER_F64 &&
        P.order_type != MGPU_ORDER_I32 && P.order_type != MGPU_ORDER_I64)
        return (int)cudaErrorInvalidValue;
    if (P.order_type != MGPU_ORDER_NONE && P.n > 0 && !P.order) return (int)cudaErrorInvalidValue;
    if (((uintptr_t)P.work & 255u) != 0) return (int)cudaErrorInvalidValue;
    const Layout L = layout(P.n, G);
    if (P.work_bytes < (int64_t)L.total) return (int)cudaErrorInvalidValue;
    char* base = (char*)P.work;
    Work W;
    W.gs = (GState*)(base + L.gstate);
    W.cnt = (int32_t*)(base + L.cnt);
    W.off = (int64_t*)(base + L.off);
    W.seg_base = (int64_t*)(base + L.seg_base);
    W.tile_base = (int64_t*)(base + L.tile_base);
    W.parts = (double*)(base + L.parts);
    W.hist = (uint32_t*)(base + L.hist);
    W.seg = (double*)(base + L.seg);
    W.cand = (uint64_t*)(base + L.cand);
    W.ctile_base = (int64_t*)(base + L.ctile_base);
    W.n_tin = L.n_tin;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e;
    int dev = 0, sms = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return (int)e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return (int)e;
    if ((e = cudaMemsetAsync(W.gs, 0, sizeof(GState) * (size_t)G, st)) != cudaSuccess) return (int)e;
    if ((e = cudaMemsetAsync(W.hist, 0, 4 * (size_t)G * kHist, st)) != cudaSuccess) return (int)e;
    const int64_t cap = (int64_t)sms * 8;
    const int cls_blocks = (int)(L.n_tin < cap ? L.n_tin : cap);
    if (cls_blocks > 0) classify_kernel<<<cls_blocks, kThreads, 0, st>>>(P, W);
    scan_kernel<<<G, kThreads, 0, st>>>(W);
    setup_kernel<<<1, 32, 0, st>>>(P, W);
    if ((P.flags & MGPU_STATS_AEFF_ONLY) || P.n == 0) return (int)cudaGetLastError();
    scatter_kernel<<<cls_blocks, kThreads, 0, st>>>(P, W);
    center_kernel<<<G, 32, 0, st>>>(W);
    const unsigned tiles = (unsigned)L.max_tseg;
    const unsigned persistent = (unsigned)(sms * 4);
    for (int r = 0; r <= P.maxiters; ++r) {
        round_pass<<<tiles, kThreads, 0, st>>>(W, G);
        radix_step<true><<<G, kThreads, 0, st>>>(P, W);
        compact_pass<<<tiles, kThreads, 0, st>>>(W, G);
        cand_setup<<<1, 32, 0, st>>>(W, G);
        select_small<<<G, kThreads, 0, st>>>(W);
        for (int lvl = 1; lvl < kLevels; ++lvl) {
            cand_pass<<<persistent, kThreads, 0, st>>>(W, G);
            radix_step<false><<<G, kThreads, 0, st>>>(P, W);
        }
        finalize_round<<<1, kG, 0, st>>>(P, W);
    }
    return (int)cudaGetLastError();
}
