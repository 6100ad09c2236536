// Fused element-chain kernel, float64 parity mode.
//
// One thread carries one photon through every stage of the chain with its
// state (pos, dir, polarization, energy, probability) in registers: the
// photon list is read once and written once per call, which is what makes
// the chain HBM-bound rather than bound by per-element passes as in MARXS
// (one full-N numpy pass per element, simulator.py:42-49).
//
// Stage semantics follow OpticalElement.process_photons (optics/base.py:
// 149-211): for hits, element columns are written, probability is
// multiplied (factor checked to lie in [0, 1]), local coordinates and the id
// are written and pos <- interpos; misses keep their state, and a column the
// stage creates receives NaN (or -1 for ids) for them.
//
// A grating stage (a Parallel of FlatGrating/CATGrating, simulator.py:
// 206-441) chooses, per photon, the nearest facet the ray crosses: a
// uniform grid in the array's mean plane yields candidate facets; photons
// whose slope exceeds the grid's bound are resolved by the whole warp
// scanning all facets with a warp min-reduction on (k, facet index).
#include <cuda_runtime.h>
#include "mgpu_device.cuh"

namespace {

constexpr int kThreads = 256;
// grid cap in blocks per SM (0: one block per 256 photons)
#ifndef MGPU_FP64_GRID_PER_SM
#define MGPU_FP64_GRID_PER_SM 0
#endif
constexpr int kGridPerSm = MGPU_FP64_GRID_PER_SM;
constexpr double kEnergy2Wave = 1.2398419292004202e-06;   // marxs/__init__.py:14

__device__ __forceinline__ PlaneHit plane_intersect_frame(const double* f, d3 pos, d3 dir) {
    return plane_intersect(arr3(f), arr3(f + 3), arr3(f + 6), arr3(f + 9), f[12], f[13], pos, dir);
}

__device__ __forceinline__ PlaneHit facet_intersect(const mgpu_facet* fc, d3 pos, d3 dir) {
    return plane_intersect(ldg3(fc->c), ldg3(fc->ex), ldg3(fc->ey), ldg3(fc->ez),
                           __ldg(&fc->hy), __ldg(&fc->hz), pos, dir);
}

// facet f of a facet stage: a flat facet, or a grating on a Cylinder
// surface (Cylinder.intersect, math/geometry.py:470-564; local coordinates
// (phi, z), k the ray parameter of the hit for the nearest-hit order)
__device__ __forceinline__ PlaneHit stage_facet_hit(const mgpu_stage& st, int f, d3 pos, d3 dir) {
    if (st.facet_cyl == nullptr) return facet_intersect(st.facets + f, pos, dir);
    const CylHit ch = cylinder_intersect_dev(st.facet_cyl + (int64_t)MGPU_FACET_CYL * f, pos, dir);
    PlaneHit h;
    h.hit = ch.hit;
    h.ip = ch.ip;
    h.ly = ch.phi;
    h.lz = ch.zl;
    h.k = dot3(ch.ip - pos, dir);
    return h;
}

// order selection: first order whose cumulative probability exceeds u, on
// the nearest-energy row for EfficiencyFile (grating.py:88-96) or the only
// row for OrderSelector (np.random.choice, grating.py:51-57)
__device__ __forceinline__ int select_order(const mgpu_selector& sel, double e, double u,
                                            double* prob, uint32_t* status) {
    int row = 0;
    if (sel.by_energy) {
        double best = fabs(sel.energy[0] - e);
        for (int j = 1; j < sel.n_rows; ++j) {
            double d = fabs(sel.energy[j] - e);
            if (d < best) {
                best = d;
                row = j;
            }
        }
    }
    const double* cdf = sel.cdf + (int64_t)row * sel.n_orders;
    int k = 0;
    while (k < sel.n_orders && !(cdf[k] > u)) ++k;
    if (k == sel.n_orders) {
        atomicOr(status, MGPU_STATUS_ORDER_EMPTY);
        k = sel.n_orders - 1;
    }
    *prob = sel.total[row];
    return sel.orders[k];
}

struct Photon {
    d3 pos, dir, pol;
    double energy, prob;
};

__device__ __forceinline__ void store_id(const mgpu_stage& st, int64_t i, int64_t v) {
    if ((st.first_writer >> 17) & 1) ((int64_t*)st.id_out)[i * st.id_stride] = v;
    else ((int32_t*)st.id_out)[i * st.id_stride] = (int32_t)v;
}

__device__ __forceinline__ void write_miss_defaults(const mgpu_stage& st, int64_t i, int nout) {
    for (int k = 0; k < nout; ++k)
        if ((st.first_writer >> k) & 1) store_col(st.out[k], i, kNaN);
    if (st.id_out && ((st.first_writer >> 16) & 1)) store_id(st, i, -1);
}

// catsupportbars (missions/mitsnl/catgrating.py:314-324): a photon that
// passed no facet is absorbed by the support structure
__device__ __forceinline__ bool support_absorbs(const mgpu_stage& st, int64_t i) {
    if (!st.id_out) return true;
    const int64_t v = ((st.first_writer >> 17) & 1) ? ((const int64_t*)st.id_out)[i * st.id_stride]
                                                    : ((const int32_t*)st.id_out)[i * st.id_stride];
    return v < 0;
}

__device__ __forceinline__ void check_prob(double f, uint32_t* status) {
    if (f < 0.0 || f > 1.0) atomicOr(status, MGPU_STATUS_PROB_RANGE);
}

// ------------------------------------------------------------------ stages
__device__ bool stage_lens(const mgpu_stage& st, Photon& ph, int64_t i, uint32_t* status) {
    // PerfectLens.specific_process_photons, optics/mirror.py:53-82
    PlaneHit h = plane_intersect_frame(st.frame, ph.pos, ph.dir);
    if (!h.hit) {
        write_miss_defaults(st, i, 2);
        return false;
    }
    d3 c = arr3(st.frame), ez = arr3(st.frame + 9);
    d3 popt = c - st.p[1] * ez;
    d3 focus = popt + st.p[0] * normalize3(ph.dir);
    d3 nd = normalize3(focus - h.ip);
    if (st.spline.n_surf > 0) {
        // probability *= reflectivity_interpolator(E, angle / 4) ** 2 (mirror.py:73-79)
        double angle = acos(fabs(dot3(nd, normalize3(ph.dir))));
        double r = spline1_at(st.spline, ph.energy, angle / 4.0);
        r = __dmul_rn(r, r);
        check_prob(r, status);
        ph.prob = ph.prob * r;
    }
    ph.pol = parallel_transport_dev(ph.dir, nd, ph.pol);
    ph.dir = nd;
    store_col(st.out[0], i, h.ly);
    store_col(st.out[1], i, h.lz);
    ph.pos = h.ip;
    return true;
}

__device__ bool stage_scatter(const mgpu_stage& st, Photon& ph, int64_t i, int rng,
                              uint64_t seed, uint64_t row_base, int sidx, uint32_t* status) {
    // RadialMirrorScatter.specific_process_photons, optics/scatter.py:49-77
    PlaneHit h = plane_intersect_frame(st.frame, ph.pos, ph.dir);
    if (!h.hit) {
        write_miss_defaults(st, i, 4);
        return false;
    }
    double sig_in = st.p[0], sig_perp = st.p[1];
    double a_in = 0.0, a_perp = 0.0;
    if (rng == MGPU_RNG_PREDRAWN) {
        if ((sig_in != 0.0 && st.draw[0] == nullptr) || (sig_perp != 0.0 && st.draw[1] == nullptr)) {
            atomicOr(status, MGPU_STATUS_BAD_STAGE);
            return false;
        }
        if (sig_in != 0.0) a_in = st.draw[0][i * st.draw_stride];
        if (sig_perp != 0.0) a_perp = st.draw[1][i * st.draw_stride];
    } else {
        double n0, n1;
        philox_normal2(seed, row_base + (uint64_t)i, (uint32_t)sidx, 0u, &n0, &n1);
        a_in = sig_in * n0;
        a_perp = sig_perp * n1;
    }
    d3 center = arr3(st.frame);
    d3 radial = ph.pos - center;                 // previous position (scatter.py:56)
    d3 perpplane = cross3(ph.dir, radial);
    d3 outdir = ph.dir;
    if (sig_in != 0.0) outdir = rot_transpose_apply(perpplane, a_in, outdir);
    if (sig_perp != 0.0) outdir = rot_transpose_apply(radial, a_perp, outdir);
    ph.pol = parallel_transport_dev(ph.dir, outdir, ph.pol);
    ph.dir = outdir;
    store_col(st.out[0], i, h.ly);
    store_col(st.out[1], i, h.lz);
    store_col(st.out[2], i, a_in);
    store_col(st.out[3], i, a_perp);
    ph.pos = h.ip;
    return true;
}

__device__ bool stage_flatdet(const mgpu_stage& st, Photon& ph, int64_t i) {
    // FlatDetector.specific_process_photons, optics/detector.py:72-75
    PlaneHit h = plane_intersect_frame(st.frame, ph.pos, ph.dir);
    if (!h.hit) {
        write_miss_defaults(st, i, 4);
        return false;
    }
    store_col(st.out[0], i, h.ly);
    store_col(st.out[1], i, h.lz);
    store_col(st.out[2], i, h.ly / st.p[0] + st.p[1]);
    store_col(st.out[3], i, h.lz / st.p[0] + st.p[2]);
    if (st.id_out) store_id(st, i, st.id_num);
    ph.pos = h.ip;
    return true;
}

__device__ bool stage_cyldet(const mgpu_stage& st, Photon& ph, int64_t i) {
    // Cylinder.intersect (math/geometry.py:470-564) + CircularDetector
    // (optics/detector.py:115-118)
    CylHit ch = cylinder_intersect_dev(st.cyl, ph.pos, ph.dir);
    if (!ch.hit) {
        write_miss_defaults(st, i, 4);
        return false;
    }
    double phi = ch.phi, R = st.cyl[25];
    d3 gp = ch.ip;
    double ly = ch.zl;
    store_col(st.out[0], i, phi);
    store_col(st.out[1], i, ly);
    store_col(st.out[2], i, phi * R / st.p[0] + st.p[1]);
    store_col(st.out[3], i, ly / st.p[0] + st.p[2]);
    if (st.id_out) store_id(st, i, st.id_num);
    ph.pos = gp;
    return true;
}

// candidate search for a grating stage; returns facet index or -1
__device__ __forceinline__ int nearest_facet_grid(const mgpu_stage& st, const Photon& ph,
                                                  bool valid, PlaneHit* best_hit,
                                                  bool* need_brute) {
    const mgpu_grid& g = st.grid;
    *need_brute = false;
    int best = -1;
    best_hit->k = 0.0;
    if (!valid) return -1;
    if (g.cell_start == nullptr) {
        *need_brute = true;
        return -1;
    }
    d3 rel = ph.pos - arr3(g.o);
    double dn = dot3(ph.dir, arr3(g.n));
    double da = dot3(ph.dir, arr3(g.a));
    double db = dot3(ph.dir, arr3(g.b));
    if (!(fabs(da) <= g.slope_max * fabs(dn)) || !(fabs(db) <= g.slope_max * fabs(dn)) ||
        dn == 0.0) {
        *need_brute = true;
        return -1;
    }
    double t0 = -dot3(rel, arr3(g.n)) / dn;
    double u = dot3(rel, arr3(g.a)) + t0 * da;
    double v = dot3(rel, arr3(g.b)) + t0 * db;
    // looked up where the ray meets the depth model of the facet surface
    const double* dq = g.depth;
    const double D = dq[0] + u * (dq[1] + dq[3] * u + dq[4] * v) + v * (dq[2] + dq[5] * v);
    u += (da / dn) * D;
    v += (db / dn) * D;
    double fu = floor((u - g.u0) / g.cell);
    double fv = floor((v - g.v0) / g.cell);
    if (!(fu >= 0.0 && fu < (double)g.nu && fv >= 0.0 && fv < (double)g.nv)) return -1;
    int cell = (int)fu * g.nv + (int)fv;
    int s0 = __ldg(g.cell_start + cell), s1 = min(__ldg(g.cell_start + cell + 1), g.capacity);
    for (int q = s0; q < s1; ++q) {
        int f = __ldg(g.cell_items + q);
        PlaneHit h = stage_facet_hit(st, f, ph.pos, ph.dir);
        if (h.hit && (best < 0 || h.k < best_hit->k || (h.k == best_hit->k && f < best))) {
            best = f;
            *best_hit = h;
        }
    }
    return best;
}

// CATL1L2Stack layers after the membrane (missions/mitsnl/catgrating.py):
// QualityFactor (:160-161), L1 (:196-207), L2Abs (:231-245), L2Diffraction
// (:263-268) through RandomGaussianScatter (optics/scatter.py:109-150).
// Out of line: only stages of stacked facets call it.
__device__ __noinline__ void cat_stack_layers(const mgpu_stage& st, const mgpu_catstack& K, int f,
                                              int m, const PlaneHit& h, double u_l1,
                                              double u_sup, double z_l2, double u_phi,
                                              Photon& ph, int64_t i, uint32_t* status) {
    const mgpu_facet* fc = st.facets + f;
    const d3 n = ldg3(fc->ex);
    // QualityFactor: factor ** (order ** 2)
    const double mm = (double)m;
    const double q = pow(K.qf, mm * mm);
    check_prob(q, status);
    ph.prob = ph.prob * q;
    // L1: a CAT grating with grooves at pi/2, or the support bars
    const d3 l1 = ldg3(K.l1_vec + 6 * f), d1 = ldg3(K.l1_vec + 6 * f + 3);
    const d3 p = normalize3(ph.dir);
    const double wave = kEnergy2Wave / ph.energy;
    const d3 pp = normalize3(p - dot3(p, l1) * l1);
    double cb = fabs(dot3(pp, n));
    cb = fmin(fmax(cb, 0.0), 1.0);
    const double blaze1 = acos(cb);
    double prob1;
    int m1 = select_order(st.selectors[K.l1_selector], ph.energy, u_l1, &prob1, status);
    d3 nd = ph.dir, npol = ph.pol;
    if (u_sup > K.l1_open) {
        m1 = 0;
        prob1 = np_interp(K.l1_trans_e, K.l1_trans_t, K.l1_n_trans, ph.energy, status);
    } else {
        const double pd0 = dot3(p, d1);
        const double sign = (pd0 > 0.0) ? 1.0 : ((pd0 < 0.0) ? -1.0 : (pd0 == 0.0 ? 1.0 : pd0));
        const double p_d = pd0 + sign * (double)m1 * wave / K.l1_d;
        const double p_l = dot3(p, l1);
        const double p_n = sqrt(1.0 - p_d * p_d - p_l * p_l);
        const double pn = dot3(p, n);
        const double direction = (pn > 0.0) ? 1.0 : ((pn < 0.0) ? -1.0 : (pn == 0.0 ? 0.0 : pn));
        nd = p_d * d1 + p_l * l1 + (direction * p_n) * n;
        npol = parallel_transport_dev(ph.dir, nd, ph.pol);
    }
    check_prob(prob1, status);
    ph.dir = nd;
    ph.pol = npol;
    ph.prob = ph.prob * prob1;
    store_col(st.out[6], i, (double)m1);
    store_col(st.out[7], i, blaze1);
    // L2Abs: open fraction minus the shadow of the inclined hexagon walls
    const d3 p3 = normalize3(ph.dir);
    const double angle = acos(fabs(dot3(p3, n)));
    const double a2 = K.l2_open - (K.l2_shadow * sin(angle)) / K.l2_total;
    check_prob(a2, status);
    ph.prob = ph.prob * a2;
    // L2Diffraction: N(0,1) * sigma about dir x guess, then a uniform turn
    const d3 pdir = normalize3(ph.dir);
    const d3 guess = (fabs(pdir.x) < 0.99999) ? d3{1.0, 0.0, 0.0} : d3{0.0, 1.0, 0.0};
    const d3 perp = cross3(pdir, guess);
    const double wave_mm = __dmul_rn(MGPU_HC_KEV_NM / ph.energy, 1e-6);
    const double sigma = (1.22 * 0.4) * asin(wave_mm / K.l2_inner);
    const double ang = z_l2 * sigma;
    d3 o = rot_transpose_apply(perp, ang, pdir);
    o = rot_transpose_apply(pdir, (u_phi * 2.0) * 3.141592653589793, o);
    ph.pol = parallel_transport_dev(ph.dir, o, ph.pol);
    ph.dir = o;
    store_col(st.out[8], i, ang);
    store_col(st.out[4], i, h.ly);
    store_col(st.out[5], i, h.lz);
}

// nearest element of a facet stage (gratings or detectors) the ray crosses:
// the candidate grid, and for photons the grid cannot bound a whole-warp scan
// of all facets with a warp min-reduction on (k, index).  Every lane of the
// warp must call it (the scan is warp-cooperative).
__device__ __forceinline__ int nearest_facet(const mgpu_stage& st, const Photon& ph, bool valid,
                                             PlaneHit* hit) {
    PlaneHit h;
    bool brute;
    int f = nearest_facet_grid(st, ph, valid, &h, &brute);
    // photons the grid cannot bound: the warp scans all facets for each of
    // them, one photon at a time, and min-reduces (k, facet)
    unsigned bm = __ballot_sync(MGPU_FULL_MASK, brute);
    const int lane = threadIdx.x & 31;
    while (bm) {
        int src = __ffs(bm) - 1;
        bm &= bm - 1;
        d3 p{__shfl_sync(MGPU_FULL_MASK, ph.pos.x, src), __shfl_sync(MGPU_FULL_MASK, ph.pos.y, src),
             __shfl_sync(MGPU_FULL_MASK, ph.pos.z, src)};
        d3 d{__shfl_sync(MGPU_FULL_MASK, ph.dir.x, src), __shfl_sync(MGPU_FULL_MASK, ph.dir.y, src),
             __shfl_sync(MGPU_FULL_MASK, ph.dir.z, src)};
        double bk = 0.0;
        int bf = -1;
        for (int q = lane; q < st.n_facets; q += 32) {
            PlaneHit hq = stage_facet_hit(st, q, p, d);
            if (hq.hit && (bf < 0 || hq.k < bk)) {
                bf = q;
                bk = hq.k;
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            double ok = __shfl_xor_sync(MGPU_FULL_MASK, bk, off);
            int of = __shfl_xor_sync(MGPU_FULL_MASK, bf, off);
            bool take = (of >= 0) && (bf < 0 || ok < bk || (ok == bk && of < bf));
            if (take) {
                bk = ok;
                bf = of;
            }
        }
        if (lane == src && bf >= 0) {
            f = bf;
            h = stage_facet_hit(st, bf, ph.pos, ph.dir);
        }
    }
    *hit = h;
    return f;
}

// Parallel of FlatDetectors (a CCD array): FlatDetector.specific_process_photons
// (optics/detector.py:72-75) on the nearest element the ray crosses; per
// element pixel size (dgrat) and centre pixel (l[0], l[1])
__device__ bool stage_detarray(const mgpu_stage& st, Photon& ph, int64_t i, bool valid) {
    PlaneHit h;
    const int f = nearest_facet(st, ph, valid, &h);
    if (!valid) return false;
    if (f < 0) {
        write_miss_defaults(st, i, 4);
        return false;
    }
    const mgpu_facet* fc = st.facets + f;
    const double pix = __ldg(&fc->dgrat);
    store_col(st.out[0], i, h.ly);
    store_col(st.out[1], i, h.lz);
    store_col(st.out[2], i, h.ly / pix + __ldg(&fc->l[0]));
    store_col(st.out[3], i, h.lz / pix + __ldg(&fc->l[1]));
    if (st.id_out) store_id(st, i, __ldg(&fc->id_num));
    ph.pos = h.ip;
    return true;
}

__device__ bool stage_gratings(const mgpu_stage& st, Photon& ph, int64_t i, bool valid,
                               int rng, uint64_t seed, uint64_t row_base, int sidx,
                               uint32_t* status) {
    PlaneHit h;
    const int f = nearest_facet(st, ph, valid, &h);
    if (!valid) return false;
    if (f < 0) {
        write_miss_defaults(st, i, MGPU_MAX_OUT);
        return false;
    }
    // FlatGrating.diffract_photons + specific_process_photons (grating.py:233-277)
    const mgpu_facet* fc = st.facets + f;
    d3 l = ldg3(fc->l), dn = ldg3(fc->dneg), n = ldg3(fc->ex);
    if (st.facet_cyl) {
        // on a Cylinder: the groove frame of e_groove_coos (grating.py:186-207)
        // on Cylinder.get_local_euklid_bases at the hit angle phi
        // (math/geometry.py:602-626): e_phi = M (-sin, cos, 0), e_n = M (cos, sin, 0)
        const double* M = st.facet_cyl + (int64_t)MGPU_FACET_CYL * f;
        double sp, cp;
        sincos(h.ly, &sp, &cp);
        d3 ephi{__dadd_rn(__dmul_rn(M[0], -sp), __dmul_rn(M[1], cp)),
                __dadd_rn(__dmul_rn(M[4], -sp), __dmul_rn(M[5], cp)),
                __dadd_rn(__dmul_rn(M[8], -sp), __dmul_rn(M[9], cp))};
        d3 en{__dadd_rn(__dmul_rn(M[0], cp), __dmul_rn(M[1], sp)),
              __dadd_rn(__dmul_rn(M[4], cp), __dmul_rn(M[5], sp)),
              __dadd_rn(__dmul_rn(M[8], cp), __dmul_rn(M[9], sp))};
        ephi = normalize3(ephi);
        en = normalize3(en);
        const d3 ez = ldg3(fc->ez);
        const double sg = M[32], cg = M[33];            // sin(-groove), cos(-groove)
        l = sg * ephi + cg * ez;
        dn = -1.0 * (cg * ephi - sg * ez);
        n = en;
    }
    d3 p = normalize3(ph.dir);
    double wave = kEnergy2Wave / ph.energy;
    d3 pp = normalize3(p - dot3(p, l) * l);
    double cb = fabs(dot3(pp, n));
    cb = fmin(fmax(cb, 0.0), 1.0);
    double blaze = acos(cb);
    if (st.stack) {
        // NonParallelCATGrating.blaze_angle_modifier (catgrating.py:324-333)
        blaze = __dadd_rn(blaze, __dadd_rn(st.stack->blaze_center,
                                           __dmul_rn(h.ly, st.stack->d_blaze_mm)));
    }
    // a custom blaze_angle_modifier, evaluated on the host at this photon's
    // local coordinates (grating.py:255)
    if (st.blaze_add.ptr) blaze = __dadd_rn(blaze, st.blaze_add.ptr[i * st.blaze_add.stride]);
    double u, u1;
    if (rng == MGPU_RNG_PREDRAWN) {
        if (st.draw[0] == nullptr) {
            atomicOr(status, MGPU_STATUS_BAD_STAGE);
            return false;
        }
        u = st.draw[0][i * st.draw_stride];
        u1 = st.draw[1] ? st.draw[1][i * st.draw_stride] : 0.0;
    } else {
        philox_uniform2(seed, row_base + (uint64_t)i, (uint32_t)sidx, 0u, &u, &u1);
    }
    double selprob;
    const mgpu_selector& sel = st.selectors[__ldg(&fc->selector)];
    int m;
    if (sel.kind == MGPU_SEL_SPLINE) m = select_order_spline(sel, ph.energy, blaze, u, &selprob);
    else m = select_order(sel, ph.energy, u, &selprob, status);
    check_prob(selprob, status);
    double pd0 = dot3(p, dn);
    double sign;
    if (__ldg(&fc->cat)) {
        sign = (pd0 > 0.0) ? 1.0 : ((pd0 < 0.0) ? -1.0 : (pd0 == 0.0 ? 1.0 : pd0));
    } else {
        sign = -1.0;
    }
    // FlatGrating.d (grating.py:209-220): the facet's constant, or the value
    // of its callable at this photon's local coordinates
    double dgr = __ldg(&fc->dgrat);
    if (st.grating_d.ptr) {
        const double v = st.grating_d.ptr[i * st.grating_d.stride];
        if (!isnan(v)) dgr = v;
    }
    double p_d = pd0 + sign * (double)m * wave / dgr;
    double p_l = dot3(p, l);
    double p_n = sqrt(1.0 - p_d * p_d - p_l * p_l);
    double pn = dot3(p, n);
    double direction = (pn > 0.0) ? 1.0 : ((pn < 0.0) ? -1.0 : (pn == 0.0 ? 0.0 : pn));
    if (!__ldg(&fc->transmission)) direction = -direction;
    d3 nd = p_d * dn + p_l * l + (direction * p_n) * n;
    ph.pol = parallel_transport_dev(ph.dir, nd, ph.pol);
    ph.dir = nd;
    ph.prob = ph.prob * selprob;
    store_col(st.out[0], i, h.ly);
    store_col(st.out[1], i, h.lz);
    store_col(st.out[2], i, (double)m);
    store_col(st.out[3], i, blaze);
    if (st.id_out) store_id(st, i, __ldg(&fc->id_num));
    if (st.stack) {
        double u_sup, u_phi, z, z1;
        if (rng == MGPU_RNG_PREDRAWN) {
            if (!st.draw[1] || !st.draw[2] || !st.draw[3] || !st.draw[4]) {
                atomicOr(status, MGPU_STATUS_BAD_STAGE);
                return false;
            }
            u_sup = st.draw[2][i * st.draw_stride];
            z = st.draw[3][i * st.draw_stride];
            u_phi = st.draw[4][i * st.draw_stride];
        } else {
            const uint64_t row = row_base + (uint64_t)i;
            philox_uniform2(seed, row, (uint32_t)sidx, 1u, &u_sup, &u_phi);
            philox_normal2(seed, row, (uint32_t)sidx, 2u, &z, &z1);
        }
        cat_stack_layers(st, *st.stack, f, m, h, u1, u_sup, z, u_phi, ph, i, status);
    }
    ph.pos = h.ip;
    return true;
}

__global__ void __launch_bounds__(kThreads)
chain_fp64_kernel(const __grid_constant__ mgpu_chain chain, const __grid_constant__ mgpu_photons io) {
    __shared__ unsigned int s_hits[MGPU_MAX_STAGES];
    if (threadIdx.x < MGPU_MAX_STAGES) s_hits[threadIdx.x] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t n = io.n;
    const int64_t warp_id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = warp_id * 32; base < n; base += n_warps * 32) {
        const int64_t i = base + lane;
        const bool valid = i < n;
        Photon ph;
        if (valid) {
            ph.pos = load3(io.pos, i);
            ph.dir = load3(io.dir, i);
            ph.pol = load3(io.pol, i);
            ph.energy = io.energy.ptr[i * io.energy.stride];
            ph.prob = io.prob.ptr[i * io.prob.stride];
        } else {
            ph.pos = ph.dir = ph.pol = d3{0.0, 0.0, 0.0};
            ph.energy = 1.0;
            ph.prob = 0.0;
        }
        if (valid && (chain.flags & MGPU_FLAG_CHECK_W)) {
            if (io.pos.ptr[i * io.pos.stride + 3 * io.pos.cstride] != 1.0 ||
                io.dir.ptr[i * io.dir.stride + 3 * io.dir.cstride] != 0.0 ||
                io.pol.ptr[i * io.pol.stride + 3 * io.pol.cstride] != 0.0)
                atomicOr(chain.status, MGPU_STATUS_BAD_W);
        }
        for (int s = 0; s < chain.n_stages; ++s) {
            const mgpu_stage& st = chain.stages[s];
            bool hit = false;
            switch (st.kind) {
            case MGPU_STAGE_GRATINGS:
                hit = stage_gratings(st, ph, i, valid, chain.rng, chain.seed, chain.row_base, s,
                                     chain.status);
                break;
            case MGPU_STAGE_DETARRAY:
                hit = stage_detarray(st, ph, i, valid);
                break;
            case MGPU_STAGE_LENS:
                if (valid) hit = stage_lens(st, ph, i, chain.status);
                break;
            case MGPU_STAGE_SCATTER:
                if (valid) hit = stage_scatter(st, ph, i, chain.rng, chain.seed, chain.row_base, s,
                                             chain.status);
                break;
            case MGPU_STAGE_FLATDET:
                if (valid) hit = stage_flatdet(st, ph, i);
                break;
            case MGPU_STAGE_CYLDET:
                if (valid) hit = stage_cyldet(st, ph, i);
                break;
            case MGPU_STAGE_SUPPORT:
                if (valid && support_absorbs(st, i)) ph.prob = 0.0;
                break;
            default:
                if (valid) atomicOr(chain.status, MGPU_STATUS_BAD_STAGE);
            }
            unsigned m = __ballot_sync(MGPU_FULL_MASK, hit);
            if (lane == 0 && m) atomicAdd(&s_hits[s], (unsigned)__popc(m));
        }
        if (valid) {
            store3(io.pos_out, i, ph.pos);
            store3(io.dir_out, i, ph.dir);
            store3(io.pol_out, i, ph.pol);
            io.prob_out.ptr[i * io.prob_out.stride] = ph.prob;
        }
    }
    __syncthreads();
    if (threadIdx.x < chain.n_stages && s_hits[threadIdx.x])
        atomicAdd(chain.hits + threadIdx.x, (unsigned long long)s_hits[threadIdx.x]);
}

}  // namespace

cudaError_t mgpu_launch_chain_fp64(const mgpu_chain& chain, const mgpu_photons& io,
                                   cudaStream_t stream, int sm_count) {
    if (io.n <= 0) return cudaSuccess;
    int64_t warps = (io.n + 31) / 32;
    int64_t blocks = (warps * 32 + kThreads - 1) / kThreads;
    if (kGridPerSm > 0) {
        const int64_t cap = (int64_t)sm_count * kGridPerSm;
        if (blocks > cap) blocks = cap;
    }
    if (blocks > (1 << 30)) blocks = 1 << 30;   // grid-stride beyond
    chain_fp64_kernel<<<(unsigned)blocks, kThreads, 0, stream>>>(chain, io);
    return cudaGetLastError();
}
