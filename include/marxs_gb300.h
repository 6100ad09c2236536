/*
 * marxs_gb300.h -- C ABI of the GB300 (sm_103a) photon-raytrace backend.
 *
 * Plain C: device pointers, sizes and POD descriptors only; no framework
 * types.  Every entry point is asynchronous on the given CUDA stream
 * (a cudaStream_t passed as void*; NULL = legacy default stream) and
 * returns 0 on a successful launch or a CUDA runtime error code.  Errors
 * found by the kernels themselves (the conditions the reference turns into
 * exceptions) are OR-ed into a device status word that the caller reads
 * after synchronising; see MGPU_STATUS_*.
 *
 * Reference interfaces (paths inside the MARXS source tree) replaced:
 *   mgpu_trace              Sequence/BaseContainer.__call__ over a chain of
 *                           elements, simulator/simulator.py:42-49, each
 *                           leaf being OpticalElement.__call__ +
 *                           process_photons, optics/base.py:144-211
 *   mgpu_facet_grid_build   (no counterpart) nearest-hit candidate lists
 *                           replacing the O(F) facet loop of
 *                           Parallel.__call__, simulator.py:42-49, 206-212
 *   mgpu_plane_intersect    FinitePlane.intersect, math/geometry.py:211-261
 *   mgpu_cylinder_intersect Cylinder.intersect, math/geometry.py:470-564
 *   mgpu_parallel_transport parallel_transport, math/polarization.py:151-170
 *   mgpu_pose_adjoint       (no counterpart) reverse mode of the element
 *                           chain above with discrete choices frozen
 */
#ifndef MARXS_GB300_H
#define MARXS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MGPU_ABI_VERSION 3
#define MGPU_MAX_STAGES 16
#define MGPU_MAX_OUT 10
#define MGPU_MAX_DRAWS 6

/* status bits (device word, OR-ed by kernels) */
#define MGPU_STATUS_PROB_RANGE   0x1u  /* probability factor outside [0,1]: ValueError, optics/base.py:43-46 */
#define MGPU_STATUS_ORDER_EMPTY  0x2u  /* no order with cumulative prob > u (EfficiencyFile would raise) */
#define MGPU_STATUS_BAD_STAGE    0x4u  /* unknown stage kind */
#define MGPU_STATUS_GRID_RANGE   0x8u  /* a facet's footprint leaves the candidate grid */
#define MGPU_STATUS_GRID_FULL    0x10u /* candidate list capacity exceeded */
#define MGPU_STATUS_BAD_W        0x20u /* input pos w != 1 or dir/pol w != 0 (checked on request) */
#define MGPU_STATUS_TABLE_RANGE  0x80u /* value outside an interpolation table (interp1d raises) */

/* mgpu_chain.flags */
#define MGPU_FLAG_CHECK_W        0x1u  /* read the homogeneous w of pos/dir/pol and check it */
#define MGPU_FLAG_NO_GRID        0x4u  /* every facet stage scans all its facets (no candidate
                                          grid; for checking the grids' candidate lists) */
#define MGPU_FLAG_SPLIT_4K       0x8u  /* FP32-local: split the launch every 4096 photons, as
                                          launches beyond 2^30 photons are split (checks the
                                          split: the same results) */
#define MGPU_FLAG_GENERIC        0x2u  /* FP32-local: run the generic stage loop even where a
                                          kernel specialised for the chain applies (the same
                                          results; for checking the specialisations) */

/* precision modes */
#define MGPU_FP64      0  /* float64 throughout, parity mode */
#define MGPU_FP32LOCAL 1  /* float32 ray arithmetic in each element's local frame */

/* randomness */
#define MGPU_RNG_PREDRAWN 0  /* per-photon arrays supplied by the caller */
#define MGPU_RNG_PHILOX   1  /* Philox4x32-10 keyed by (seed, row_base + row, stage, draw) */

/* stage kinds */
#define MGPU_STAGE_LENS     1  /* PerfectLens, optics/mirror.py:53-82 */
#define MGPU_STAGE_SCATTER  2  /* RadialMirrorScatter, optics/scatter.py:49-77 */
#define MGPU_STAGE_FLATDET  3  /* FlatDetector, optics/detector.py:72-75 */
#define MGPU_STAGE_GRATINGS 4  /* Parallel of FlatGrating/CATGrating (or one grating) */
#define MGPU_STAGE_CYLDET   5  /* CircularDetector on a Cylinder */
#define MGPU_STAGE_SUPPORT  6  /* catsupportbars, missions/mitsnl/catgrating.py:314-324:
                                  probability = 0 where the id column at id_out (the facet
                                  column) is < 0, or for every photon when id_out is NULL */
#define MGPU_STAGE_DETARRAY 7  /* Parallel of FlatDetectors (a CCD array), simulator.py:206-441
                                  over optics/detector.py:18-75: the nearest element the ray
                                  crosses, found like the facets of GRATINGS (facets, grid,
                                  facets32); per element the pixel size in mgpu_facet.dgrat and
                                  the centre pixel in l[0], l[1] (FP32-local: mgpu_facet32.l =
                                  1 / pixel size, centre x, centre y) */

/* a float64 photon column: value of photon i at ptr[i * stride] */
typedef struct {
    double* ptr;
    int64_t stride;
} mgpu_col;

/* a 3-vector column: component c of photon i at ptr[i * stride + c * cstride]
 * ((N,4) row-major homogeneous arrays: stride 4, cstride 1; SoA planes:
 * stride 1, cstride = plane pitch) */
typedef struct {
    double* ptr;
    int64_t stride;
    int64_t cstride;
} mgpu_vec;

typedef struct {
    int64_t n;
    mgpu_vec pos, dir, pol;          /* input state */
    mgpu_col energy, prob;
    mgpu_vec pos_out, dir_out, pol_out;  /* output state (may alias inputs) */
    mgpu_col prob_out;
} mgpu_photons;

/* one grating facet (float64).  Unit vectors as MARXS derives them from
 * pos4d (Geometry.__getitem__, math/geometry.py:108-160). */
typedef struct {
    double c[3];      /* centre */
    double ex[3];     /* unit normal e_x */
    double ey[3];     /* unit e_y */
    double ez[3];     /* unit e_z */
    double hy, hz;    /* |v_y|, |v_z| half sizes */
    double l[3];      /* groove direction e_groove (grating.py:203-207) */
    double dneg[3];   /* -e_perp_groove (grating.py:239) */
    double dgrat;     /* grating constant, mm */
    int32_t id_num;   /* value written to the id column */
    int32_t selector; /* index into the selector table */
    int32_t cat;      /* 1: CATGrating sign convention, 0: FlatGrating (-1) */
    int32_t transmission;
} mgpu_facet;

/* Degree-1 tensor-product spline, scipy RectBivariateSpline(kx=1, ky=1) as
 * FITPACK evaluates it (fpbisp): arguments clamped to [tx[1], tx[nx-2]] and
 * [ty[1], ty[ny-2]]; n_surf surfaces share the knots, surface s has the
 * (nx-2)(ny-2) coefficients c[s (nx-2)(ny-2) ...], x-major. */
typedef struct {
    int32_t nx, ny;       /* knot counts (grid points + 2) */
    int32_t n_surf;       /* 0 = no spline */
    int32_t pad;
    const double* tx;
    const double* ty;
    const double* c;
    const float* c32;     /* FP32-local: the coefficients in float32, n_surf + 1 surfaces,
                             the last one the sum of the others */
    const float* tx_ff;   /* FP32-local: the knots as float-float (hi, lo) pairs, nx x 2 */
    const float* ty_ff;   /* ny x 2 */
} mgpu_spline1;

#define MGPU_SEL_CDF    0  /* cumulative rows: OrderSelector, EfficiencyFile */
#define MGPU_SEL_SPLINE 1  /* one spline per order in (wavelength nm, blaze rad):
                              InterpolateEfficiencyTable, missions/mitsnl/catgrating.py:63-144 */

/* order selector: OrderSelector (one row), EfficiencyFile (energy rows) or
 * InterpolateEfficiencyTable (kind SPLINE) */
typedef struct {
    int32_t n_rows;
    int32_t n_orders;
    int32_t by_energy;    /* 1: nearest energy row (argmin |E - e|) */
    int32_t sorted;       /* 1: energy strictly increasing and every cdf row
                             non-decreasing (binary searches allowed) */
    const double* energy; /* n_rows */
    const double* cdf;    /* n_rows * n_orders, normalised cumulative */
    const double* total;  /* n_rows, probability factor */
    const int32_t* orders;/* n_orders */
    const uint64_t* thresholds; /* n_rows * n_orders: ceil(cdf * 2^53); for a draw
                                   u = U * 2^-53, cdf > u  <=>  U < threshold */
    int32_t kind;         /* MGPU_SEL_* */
    int32_t pad;
    mgpu_spline1 spline;  /* SPLINE: n_surf = n_orders surfaces */
    const uint8_t* guide; /* optional, sorted rows only: n_rows x 64, entry b = first order
                             index k with U < threshold[k] for U = b * 2^47 */
    const double* e_mid;  /* optional, sorted energy rows (FP32-local): n_rows - 1 midpoints
                             (E_j + E_j+1) / 2; row j+1 is nearer when e > e_mid[j] */
    float e0_f;           /* FP32-local row guess: E_0 and (n_rows - 1) / (E_last - E_0) */
    float e_scale_f;
} mgpu_selector;

/* FP32-local constants of a flat element (PerfectLens, RadialMirrorScatter,
 * FlatDetector): centre as float-float, frame and parameters in float32 */
typedef struct {
    float c_hi[3], c_lo[3];
    float ex[3], ey[3], ez[3];
    float hy, hz;
    float p[6];            /* kind parameters as in mgpu_stage.p */
} mgpu_flat32;

/* FP32-local facet record: 128 bytes, read by the kernels as eight float4
 * rows from a 16-byte aligned table:
 *   (c_hi, hy) (c_lo, hz) (ex, ey.x) (ey.y, ey.z, ez.x, ez.y)
 *   (ez.z, l) (dneg, wd_hi) (wd_lo, id_num, selector, flags) (pad) */
typedef struct {
    float c_hi[3];
    float hy;
    float c_lo[3];
    float hz;
    float ex[3], ey[3], ez[3];
    float l[3], dneg[3];
    float wd_hi, wd_lo;    /* energy2wave / d as float-float (keV) */
    int32_t id_num;
    int32_t selector;
    int32_t flags;         /* bit 0: CAT sign convention, bit 1: transmission */
    int32_t pad[4];
} mgpu_facet32;

/* FP32-local constants of a grating stage's candidate grid */
typedef struct {
    float o_hi[3], o_lo[3];
    float n[3], a[3], b[3];
    float u0, v0, inv_cell, slope_max;
    int32_t nu, nv;
    float depth[6];        /* mgpu_grid.depth */
} mgpu_grid32;

/* FP32-local constants of a circular cylinder detector.  e1, e2, a are the
 * unit local axes.  Hits are resolved around reference points on the
 * cylinder at the angles k / 1024 rad, k = k0 .. k0 + nk - 1: the stage's
 * table holds per k three float4, (P_k hi, u.x), (P_k lo, u.y), (t_k, u.z),
 * with P_k = c + R u_k the global reference point as float-float,
 * u_k = cos e1 + sin e2 the radial and t_k = -sin e1 + cos e2 the tangential
 * unit vector. */
typedef struct {
    float c_hi[3], c_lo[3];
    float e1[3], e2[3], a[3];
    float R;               /* radius (x zoom) */
    float Rz;              /* half length (z zoom) */
    float w1[2], w2[2];    /* phi_lim borders as unit vectors in the (e1, e2) plane */
    int32_t arc;           /* 0: arc w1 -> w2 spans <= pi, 1: > pi, 2: full circle */
    float rpix_hi, rpix_lo;/* R / pixsize */
    float inv_pix;
    float cp0, cp1;        /* centerpix */
    int32_t k0, nk;
} mgpu_cyl32;

/* uniform candidate grid in a plane (origin o, normal n, in-plane axes a,b).
 * A ray crossing the plane at (u0, v0) with slopes su = d.a/d.n, sv = d.b/d.n
 * is looked up at (u0 + su D, v0 + sv D), D = depth model at (u0, v0): where
 * it meets the facets' surface, up to their deviation from the model (all
 * depth coefficients zero: the plane itself) */
typedef struct {
    double o[3], n[3], a[3], b[3];
    double u0, v0, cell;   /* grid origin (u,v) and cell size, mm */
    int32_t nu, nv;
    double slope_max;      /* |d.a/d.n|, |d.b/d.n| bound for grid lookup */
    double margin;         /* extra footprint margin, mm */
    double depth[6];       /* depth of the facet surface along n over the plane:
                              D(u,v) = d0 + d1 u + d2 v + d3 u^2 + d4 u v + d5 v^2 */
    double depth_lip;      /* bound on |dD/du| + |dD/dv| over the grid's area */
    int32_t* cell_start;   /* nu*nv+1, device */
    int32_t* cell_items;   /* capacity entries, device */
    int32_t capacity;
    int32_t pad;
} mgpu_grid;

/* Layers of a CATL1L2Stack facet after its grating membrane
 * (missions/mitsnl/catgrating.py:147-377), shared by all facets of a stage:
 *   membrane blaze += blaze_center + local y * d_blaze_mm (NonParallelCATGrating)
 *   QualityFactor   probability *= qf ** (order^2)
 *   L1              a CAT grating (grooves l1_vec, period l1_d, selector
 *                   l1_selector) or, when the support draw > l1_open, the ray
 *                   unchanged with order 0 and probability interp(E) of the
 *                   table (l1_trans_e, l1_trans_t) (np.interp / interp1d)
 *   L2Abs           probability *= l2_open - l2_shadow * sin(angle) / l2_total
 *   L2Diffraction   Gaussian turn by N(0,1) * 1.22 * 0.4 * asin(lambda / l2_inner)
 *                   about dir x guess, then a uniform turn about dir
 * Stage outputs: out[0..3] grat_y, grat_z, order, blaze; out[4..5] y, z;
 * out[6..8] order_L1, blaze_L1, L2Diffraction.  Draws: draw[0] order,
 * draw[1] L1 order, draw[2] L1 support, draw[3] L2 N(0,1), draw[4] L2 turn. */
typedef struct mgpu_catstack {
    double blaze_center, d_blaze_mm;
    double qf;
    double l1_open;
    double l1_d;                 /* L1 period, mm */
    const double* l1_vec;        /* n_facets x 6: L1 groove direction, -perp groove direction */
    int32_t l1_selector;         /* index into the stage's selectors */
    int32_t l1_n_trans;
    const double* l1_trans_e;    /* keV, increasing */
    const double* l1_trans_t;
    double l2_open;              /* (inner / period)^2 */
    double l2_shadow;            /* bardepth * inner */
    double l2_total;             /* period^2 / 2 * sqrt(3) */
    double l2_inner;             /* period - barwidth, mm */
    /* FP32-local constants */
    const float* l1_vec32;       /* l1_vec in float32 */
    float l1_wd_hi, l1_wd_lo;    /* energy2wave / L1 period as float-float (keV) */
    float qf32;                  /* qf */
    float l2_open32;             /* l2_open */
    float l2_absorb32;           /* l2_shadow / l2_total */
    float l2_inv_inner32;        /* 1 / l2_inner, 1/mm */
    float blaze_center32, d_blaze32;
    int64_t l1_open_u53;         /* floor(l1_open * 2^53) (>= -1): a Philox draw U
                                    (u = U 2^-53) takes the support when U > l1_open_u53 */
    const float* l1_trans_e32;   /* l1_trans_e, l1_trans_t in float32 */
    const float* l1_trans_t32;
} mgpu_catstack;

typedef struct {
    int32_t kind;
    int32_t id_num;              /* id value for single elements (unused: -9) */
    int32_t first_writer;        /* bit k (k < MGPU_MAX_OUT): out[k] is new -> write NaN
                                    on miss; bit 16: id column new -> write -1 on miss;
                                    bit 17: id column holds int64 (else int32) */
    int32_t n_facets;
    double frame[14];            /* flat: c(3) ex(3) ey(3) ez(3) hy hz */
    double cyl[32];              /* cylinder: pos4d rows 0-2 (12), inverse rows 0-2 (12),
                                    zoom_z, R, b1, b2 (angle_between borders) */
    double p[8];                 /* kind parameters, see below */
    mgpu_col out[MGPU_MAX_OUT];  /* output columns (NULL ptr = not written) */
    void* id_out;                /* id column (int32 or int64, first_writer bit 17) or NULL;
                                    SUPPORT reads it */
    int64_t id_stride;
    const double* draw[MGPU_MAX_DRAWS]; /* pre-drawn per-photon values (RNG_PREDRAWN) */
    int64_t draw_stride;
    const mgpu_facet* facets;    /* GRATINGS */
    const mgpu_selector* selectors;
    int32_t n_selectors;
    int32_t facet_sel0;          /* GRATINGS: 1 when every facet uses selectors[0] */
    mgpu_grid grid;              /* GRATINGS: candidate grid (cell_start NULL = brute force) */
    int32_t aux_size;            /* bytes of aux32 in use (0: none) */
    int32_t pad2;
    uint8_t aux32[128];          /* FP32-local constants inline, so the kernel reads them from
                                    its parameter bank: mgpu_flat32 (flat kinds), mgpu_grid32
                                    (GRATINGS, DETARRAY), mgpu_cyl32 (CYLDET) */
    const mgpu_facet32* facets32;/* GRATINGS, FP32-local, 16-byte aligned */
    const float* table;          /* CYLDET, FP32-local: nk x 12 floats, 16-byte aligned
                                    (see mgpu_cyl32) */
    mgpu_spline1 spline;         /* LENS: reflectivity_interpolator(energy, angle / 4), squared
                                    into the probability (optics/mirror.py:73-79); n_surf 0 = 1 */
    const struct mgpu_catstack* stack; /* GRATINGS: facets are CATL1L2Stacks (NULL: plain) */
    mgpu_selector sel0;          /* GRATINGS: a copy of selectors[0]; with facet_sel0 the
                                    FP32-local kernel reads it from its parameter bank */
    mgpu_col grating_d;          /* GRATINGS, optional: per-photon grating constant (mm) where
                                    it depends on the position on the facet (FlatGrating.d with
                                    a callable _d, optics/grating.py:209-220); NaN = the
                                    facet's own dgrat */
    mgpu_col blaze_add;          /* GRATINGS, optional: per-photon addend to the blaze angle
                                    (a custom blaze_angle_modifier, grating.py:222-231) */
    const double* facet_cyl;     /* GRATINGS, optional (float64 kernel): the facets are gratings
                                    on Cylinder surfaces, MGPU_FACET_CYL doubles each: the
                                    cylinder block of mgpu_stage.cyl (pos4d rows, inverse rows,
                                    zoom_z, R, reduced phi borders; 32) and sin(-groove),
                                    cos(-groove); the facet table then holds each patch's
                                    tangent plane for the candidate grid.  NULL: flat facets */
} mgpu_stage;
#define MGPU_FACET_CYL 34
/* p[] per kind:
 *   LENS:    p[0] focal length, p[1] d_center_optical_axis
 *   SCATTER: p[0] sigma in-plane (rad), p[1] sigma perpendicular (rad)
 *   FLATDET, CYLDET: p[0] pixsize, p[1] centerpix x, p[2] centerpix y
 * out[] per kind:
 *   LENS:     loc0, loc1
 *   SCATTER:  loc0, loc1, inplanescatter, perpplanescatter
 *   FLATDET:  loc0 (det_x), loc1 (det_y), detpix_x, detpix_y
 *   GRATINGS: loc0 (grat_y), loc1 (grat_z), order, blaze   (+ id_out: facet)
 *   DETARRAY: loc0 (det_x), loc1 (det_y), detpix_x, detpix_y (+ id_out: e.g. CCD_ID)
 *   CYLDET:   loc0 (det_phi), loc1 (det_y), detpix_x, detpix_y
 */

typedef struct {
    int32_t n_stages;
    int32_t precision;           /* MGPU_FP64 / MGPU_FP32LOCAL */
    int32_t rng;                 /* MGPU_RNG_PREDRAWN / MGPU_RNG_PHILOX */
    uint32_t flags;              /* MGPU_FLAG_* */
    uint64_t seed;
    uint64_t row_base;           /* global id of photon row 0 (Philox counter) */
    uint32_t* status;            /* device status word */
    unsigned long long* hits;    /* device, n_stages counters (added to) */
    mgpu_stage stages[MGPU_MAX_STAGES];
} mgpu_chain;

/* library ABI version (MGPU_ABI_VERSION) */
int mgpu_abi_version(void);

/* Trace photons through the chain.  Photon state is read from the input
 * columns and the final state written to the output columns for every
 * photon; stage columns are written for hits (and defaults for misses
 * where first_writer says so).  FP32-local addresses photon rows with
 * 32-bit offsets: every column stride must stay below 2^28 elements
 * (cudaErrorInvalidValue otherwise), and launches beyond 2^30 photons are
 * split internally. */
int mgpu_trace(const mgpu_chain* chain, const mgpu_photons* photons, void* stream);

/* Build the candidate lists of a grating stage's grid on the device:
 * grid->cell_start / cell_items are filled from the facet table.
 * n_facets < 0, or facets NULL with n_facets > 0, is cudaErrorInvalidValue.
 * ``counts`` is caller-provided scratch of nu*nv + 1 + ceil(nu*nv / 4096) int32. */
int mgpu_facet_grid_build(const mgpu_facet* facets, int32_t n_facets, mgpu_grid* grid,
                          int32_t* counts, uint32_t* status, void* stream);

/* Allocation-free variant of mgpu_facet_grid_build; it has no counterpart in
 * the reference.  For callers that cannot allocate device memory when they
 * rebuild the grid (a host whose own pool owns the device memory, or a loop
 * where cudaMalloc/cudaFree would synchronise the device): the per-cell
 * scratch lives in a fixed device array of MGPU_NOALLOC_MAX_CELLS + 1 cell
 * counters plus one int32 scan sum per 4096 cells (65,553 int32 = 262,212 B,
 * held on every GPU that loads the library until the process exits), and
 * the entry point calls no allocator.  The caller still passes
 * the facets, the grid with its cell_start / cell_items outputs, and the
 * status word.  Grids with nu * nv > MGPU_NOALLOC_MAX_CELLS are rejected with
 * MGPU_ERR_NOALLOC_LIMIT before anything is launched.  The first call on a
 * device looks up the array's device address with that device current; make
 * that first call before any stream capture.  The address is kept for the
 * life of the process: after cudaDeviceReset, or with another context made
 * current on the same device, it is stale, so do not call this entry point
 * across a reset.  All calls share the array:
 * each call clears it before use, and calls that overlap on the GPU (other
 * streams, other host threads) race on it. */
#define MGPU_NOALLOC_MAX_CELLS 65536
#define MGPU_ERR_NOALLOC_LIMIT (-2)
int mgpu_facet_grid_build_noalloc(const mgpu_facet* facets, int32_t n_facets, mgpu_grid* grid,
                                  uint32_t* status, void* stream);

/* FinitePlane.intersect for one element frame (c, ex, ey, ez, hy, hz as in
 * mgpu_stage.frame).  Outputs: hit (uint8), interpos (vec), local (2 cols). */
int mgpu_plane_intersect(const double* frame14, int64_t n, mgpu_vec pos, mgpu_vec dir,
                         uint8_t* hit, mgpu_vec interpos, mgpu_col loc0, mgpu_col loc1,
                         void* stream);

/* Cylinder.intersect for one element (cyl block as in mgpu_stage.cyl). */
int mgpu_cylinder_intersect(const double* cyl32, int64_t n, mgpu_vec pos, mgpu_vec dir,
                            uint8_t* hit, mgpu_vec interpos, mgpu_col loc0, mgpu_col loc1,
                            void* stream);

/* parallel_transport(dir_old, dir_new, pol) -> pol_out */
int mgpu_parallel_transport(int64_t n, mgpu_vec dir_old, mgpu_vec dir_new, mgpu_vec pol,
                            mgpu_vec pol_out, void* stream);

/* number of SMs of the current device (for launch sizing by callers) */
int mgpu_device_sm_count(void);

/* ---- photon generation on the device ----
 *
 * A point source seen through a CircleAperture, written straight into
 * device photon columns (replaces, for this source/aperture pair,
 * Source.generate_photons -> FixedPointing -> CircleAperture):
 *   energy   constant, or RandomArbitraryPdf (math/random.py:4-95):
 *            choice = cdf[last] * u0, i = first index with cdf[i] >= choice,
 *            j = index[i], E = x[j - 1] + width[j] * u1 (x[-1] = last edge)
 *   angle    constant, or 2 pi * u2 (unpolarized, source/basesources.py:203-204)
 *   pol      v1 cos(angle) + v2 sin(angle) (polarization_vectors,
 *            math/polarization.py:12-63, basis of the fixed direction)
 *   position CircleAperture.generate_local_xy (optics/aperture.py:138-146):
 *            phi = phi0 + (phi1 - phi0) u3, r = sqrt(ri2 + (1 - ri2) u4),
 *            pos = centre + r cos(phi) v_y + r sin(phi) v_z
 *   prob     clip(dir . -e_x, 0, 1) (aperture.py:72-76)
 * Uniforms: Philox keyed by (seed, row_base + row, 0x5000 + k) or pre-drawn
 * (draws[k * n + row], k = 0..4).
 * precision MGPU_FP32LOCAL (Philox only): the same distributions with the
 * bin chosen by integer thresholds on a 32-bit draw, float32 sines,
 * cosines and square root (24-bit uniforms, stages 0x5003-0x5004), and
 * float-float sums for energy and position; no float64 arithmetic but the
 * final float-float to float64 conversion (4 adds per photon). */
typedef struct {
    int64_t n;
    uint64_t seed, row_base;
    int32_t rng;             /* MGPU_RNG_* */
    int32_t n_bins;          /* energy pdf bins (0: constant energy) */
    double energy;           /* keV, when n_bins == 0 */
    const double* e_x;       /* n_bins upper bin edges */
    const double* e_width;   /* n_bins bin widths (e_width[0] = 0) */
    const double* e_cdf;     /* n_bins cumulative sum of the (sorted) pdf * width */
    const int32_t* e_index;  /* n_bins sort index (identity when unsorted) */
    int32_t pol_random;      /* 1: angle = 2 pi u2; 0: pol_angle */
    int32_t precision;       /* MGPU_FP64 or MGPU_FP32LOCAL */
    double pol_angle;
    double dir[3];           /* unit direction of travel */
    double pol_v1[3], pol_v2[3];
    double center[3], v_y[3], v_z[3];
    double phi0, phi1, r_inner2;
    double prob;             /* probability of every photon */
    const double* draws;     /* RNG_PREDRAWN: 5 x n uniforms */
    /* MGPU_FP32LOCAL energy tables, n_bins entries each */
    const float* e_lo_ff;    /* 2 n_bins: the energy at u1 = 0 of bin j (x[j - 1], or x[j]
                                without randomize_in_bin) as float-float (hi, lo) */
    const float* e_width_f;  /* bin widths (0 without randomize_in_bin) */
    const uint64_t* e_thresh;/* floor(cdf[i] / cdf[last] * 2^32) + 1: entry i is the first
                                with U < e_thresh[i], U a 32-bit draw */
} mgpu_source;

int mgpu_generate_photons(const mgpu_source* src, mgpu_vec pos, mgpu_vec dir, mgpu_vec pol,
                          mgpu_col energy, mgpu_col prob, void* stream);

/* ---- pose adjoint: detector moments of frozen photons and their gradient ----
 *
 * No single reference interface: it differentiates the forward of
 * PerfectLens (optics/mirror.py:53-82) -> RadialMirrorScatter
 * (optics/scatter.py:49-77) -> one FlatGrating/CATGrating facet of a Parallel
 * array (optics/grating.py:233-277) -> FlatDetector (math/geometry.py:211-261)
 * or CircularDetector (math/geometry.py:470-564) with every photon's discrete
 * choices frozen (hits, facet, order, scatter angles, order sign, normal side,
 * cylinder root).  Parameters theta (device, 7 + 6 F doubles):
 *   theta[0]            focal length of the lens (absolute, mm)
 *   theta[1 + 6j + 0..2] translation of facet j's centre (mm)
 *   theta[1 + 6j + 3..5] rotation of facet j about its centre,
 *                        R = Rz(a2) Ry(a1) Rx(a0) (static x, y, z Euler angles,
 *                        as elem_uncertainty uses, design/uncertainties.py:36-38)
 *   theta[1 + 6F + 0..5] the same six for the detector.
 * A perturbed element has pos4d = [R M | c + t] for base pos4d = [M | c].
 * Photons are split into groups (an order, an energy ...); per group g the
 * kernel sums, over its photons with weight w and detector coordinates (x, y)
 * taken relative to the group centre ref[2g], ref[2g+1]:
 *   moments[5g + 0..4] = sum w, sum w x, sum w y, sum w x^2, sum w y^2.
 * FLAT: (x, y) = det_x, det_y (mm).  CYL: x = det_phi * R (mm), y = det_y (mm).
 * BACKWARD takes seeds[4g + 0..3] = dL/d(sum w x), dL/d(sum w x^2),
 * dL/d(sum w y), dL/d(sum w y^2) and adds dL/dtheta to grad, so any loss of
 * the moments (spot width, centroid offset, resolving power) differentiates
 * through one launch.  Backward recomputes the forward from the photon input
 * and keeps each stage's output (position, direction) as its checkpoint;
 * each stage's internals are recomputed inside its reverse step.
 * Calls that share one problem must not overlap (rot is their scratch). */
#define MGPU_ADJ_FREEZE   0   /* write sign / nsign / root from the forward at theta */
#define MGPU_ADJ_FORWARD  1   /* add moments; x_out / y_out if non-NULL */
#define MGPU_ADJ_BACKWARD 2   /* add dL/dtheta to grad */
#define MGPU_ADJ_DET_FLAT 0
#define MGPU_ADJ_DET_CYL  1
#define MGPU_ADJ_NMOM     5
#define MGPU_ADJ_NSEED    4
#define MGPU_ADJ_MAX_GROUPS 64
#define MGPU_ADJ_MAX_FACETS 4096
#define MGPU_ADJ_FACET_CAT          0x1u
#define MGPU_ADJ_FACET_TRANSMISSION 0x2u
#define MGPU_STATUS_ADJ_RANGE 0x40u  /* facet or group index out of range, or no cylinder root */

typedef struct {
    int64_t n;                  /* photons */
    int32_t n_facets;
    int32_t n_groups;
    int32_t det_kind;           /* MGPU_ADJ_DET_* */
    int32_t precision;          /* MGPU_FP64, or MGPU_FP32LOCAL for FORWARD / BACKWARD with a
                                 * flat detector (FREEZE runs in float64 either way); FP32LOCAL
                                 * needs rot of (n_facets + 3) * 192 bytes */
    const double* pos;          /* 3 x n (SoA), position before the lens */
    const double* dir;          /* 3 x n, direction before the lens */
    const double* alpha;        /* in-plane scatter angle (rad; 0 = no rotation) */
    const double* beta;         /* perpendicular scatter angle (rad) */
    const double* energy;       /* keV */
    const double* weight;       /* photon weight in the moments */
    const int32_t* facet;       /* index into facets */
    const int32_t* order;       /* diffraction order */
    const int32_t* group;       /* moment group; < 0 = photon not counted */
    int8_t* sign;               /* frozen order sign (written by FREEZE) */
    int8_t* nsign;              /* frozen normal side (written by FREEZE) */
    int8_t* root;               /* CYL: frozen root +1 / -1 (written by FREEZE) */
    double lens[10];            /* centre (3), unit normal e_x (3), unit e_z (3), d_center_optical_axis */
    double scatter[6];          /* centre (3), unit normal e_x (3) */
    const double* facets;       /* F x 13: centre, unit normal, groove e_l, -e_perp, grating constant */
    const uint8_t* facet_flags; /* MGPU_ADJ_FACET_* */
    double det[32];             /* FLAT: centre, unit e_x, e_y, e_z.  CYL: centre (3), M (9, row
                                 * major), inverse of M (9), radius, zoom_z, phi_lim lo, hi */
    const double* ref;          /* device, n_groups x 2 moment centres */
    double* x_out;              /* optional, FORWARD: per-photon x */
    double* y_out;              /* optional, FORWARD: per-photon y */
    double* rot;                /* device scratch, 36 (F + 1) doubles (FP32LOCAL: at least
                                 * 24 (F + 3)) */
    uint32_t* status;           /* device status word */
} mgpu_adjoint_problem;

int mgpu_pose_adjoint(const mgpu_adjoint_problem* prob, const double* theta, int32_t mode,
                      const double* seeds, double* moments, double* grad, void* stream);

/* ---- per-order statistics of a photon list (analysis reductions) ----
 *
 * Replaces, for device-resident event columns, the per-order loops of
 *   resolvingpower_from_photonlist  analysis/gratings.py:215-270
 *   effectivearea_from_photonlist   analysis/gratings.py:333-363
 *   CaptureResAeff.__call__         analysis/gratings.py:470-501
 * and astropy.stats.sigma_clipped_stats with the defaults those call it with
 * (cenfunc median, stdfunc std, std_ddof 0, sigma 3, maxiters 5).
 *
 * Photons are grouped by the value of their order column: group g holds the
 * photons whose order equals orders[g] (order_type MGPU_ORDER_NONE: every
 * photon is in group 0).  Per group the call computes
 *   n_member  photons in the group that pass the filter (RES_FILTER: finite
 *             value and probability > 0), the count the reference compares
 *             with 20;
 *   the sigma-clipped mean, median and std of the group's finite values;
 *   aeff_sum  sum of probability over the group's photons (aeff_mask != 0
 *             when a mask is given), no other filter.
 * All sums are deterministic (fixed reduction order); the median is exact. */
#define MGPU_STATS_MAX_GROUPS 64
#define MGPU_STATS_NRES 8
/* result columns, n_groups x MGPU_STATS_NRES doubles */
#define MGPU_STATS_MEAN     0
#define MGPU_STATS_MEDIAN   1
#define MGPU_STATS_STD      2
#define MGPU_STATS_N_CLIP   3  /* values left after clipping */
#define MGPU_STATS_N_MEMBER 4
#define MGPU_STATS_AEFF     5
#define MGPU_STATS_N_FINITE 6  /* finite members: the values that enter the clipping */
#define MGPU_STATS_ROUNDS   7  /* clipping iterations run */
#define MGPU_ORDER_NONE 0
#define MGPU_ORDER_F64  1
#define MGPU_ORDER_I32  2
#define MGPU_ORDER_I64  3
#define MGPU_STATS_RES_FILTER 0x1u  /* members need a finite value and probability > 0 */
#define MGPU_STATS_AEFF_ONLY  0x2u  /* counts and aeff_sum only: no clipping (statistics NaN) */

typedef struct {
    int64_t n;                  /* photons */
    mgpu_col value;             /* the dispersion coordinate (f64) */
    const void* order;          /* order column (order_type), element i at order[i * order_stride] */
    int64_t order_stride;
    int32_t order_type;         /* MGPU_ORDER_* */
    int32_t n_groups;           /* 1 .. MGPU_STATS_MAX_GROUPS */
    mgpu_col prob;              /* probability (f64); ptr NULL = 1 for every photon */
    const uint8_t* aeff_mask;   /* optional: photons counted in aeff_sum (nonzero) */
    uint32_t flags;             /* MGPU_STATS_* */
    int32_t maxiters;           /* clipping iterations (>= 1) */
    double sigma;               /* clip at median -/+ sigma * std */
    double orders[MGPU_STATS_MAX_GROUPS];
    void* work;                 /* device workspace, mgpu_order_stats_workspace bytes, 256-B aligned */
    int64_t work_bytes;
    double* result;             /* device, n_groups x MGPU_STATS_NRES */
} mgpu_stats_problem;

int64_t mgpu_order_stats_workspace(int64_t n, int32_t n_groups);
int mgpu_order_stats(const mgpu_stats_problem* prob, void* stream);

/* ---- facet poses of a Parallel on the device (tolerancing) ----
 *
 * Replaces Parallel.generate_elements (simulator/simulator.py:384-440) for
 * the facets of one grating stage after wiggle / moveglobal /
 * moveindividual (design/tolerancing.py:45-111): element i is posed as
 *   pos4d_i = outer T(t_i) T(c_i) R(a_i) M_i
 * where outer = the Parallel's pos4d times its global uncertainty, (c_i, M_i)
 * the uncertainty-free local pose, t_i the translation and R(a_i) the Euler
 * sxyz rotation of the element uncertainty.  DRAW takes (t_i, a_i) as
 * offset + sigma * z with z standard normals from Philox keyed by (seed,
 * facet index) -- the distribution of generate_facet_uncertainty,
 * design/uncertainties.py:8-39.  The facet frame (c, e_x, e_y, e_z, hy, hz,
 * groove l, -e_perp) is rewritten in place; the other facet fields are
 * kept.  Rebuild the candidate grid with mgpu_facet_grid_build afterwards. */
#define MGPU_POSE_ZERO  0   /* no element uncertainty */
#define MGPU_POSE_DRAW  1   /* Gaussian draws */
#define MGPU_POSE_GIVEN 2   /* given[6 i ...] = dx, dy, dz (mm), rx, ry, rz (rad) */

typedef struct {
    int32_t n_facets;
    int32_t mode;               /* MGPU_POSE_* */
    uint64_t seed;              /* DRAW */
    double sigma[6];            /* DRAW: Gaussian sigma of dx, dy, dz, rx, ry, rz */
    double offset[6];           /* DRAW: mean of the same */
    const double* given;        /* GIVEN: device, n_facets x 6 */
    double* perturb_out;        /* optional, device, n_facets x 6: the (t, a) used */
    double outer[16];           /* row-major 4x4: Parallel pos4d times its uncertainty */
    const double* local;        /* device, n_facets x 12: c (3), M (3x3 row-major) */
    const double* groove;       /* device, n_facets x 2: sin(-groove angle), cos(-groove angle) */
    mgpu_facet* facets;         /* device, rewritten in place */
    mgpu_facet32* facets32;     /* optional, device: FP32-local records rewritten */
} mgpu_pose_update;

int mgpu_facet_poses(const mgpu_pose_update* update, void* stream);

/* ---- measurement (no counterpart in the reference) ----
 * FMA-chain throughput probe: ``blocks`` blocks of 256 threads, each thread
 * running 8 independent chains of ``iters`` fused multiply-adds in float32
 * (precision MGPU_FP32LOCAL) or float64 (MGPU_FP64); out receives one value
 * per thread (blocks * 256 floats or doubles).  2 * 8 * iters * 256 * blocks
 * flops per launch: the measured FMA peak of the pipe the intersect stage's
 * arithmetic runs on. */
int mgpu_fma_probe(int32_t precision, int32_t blocks, int32_t iters, void* out, void* stream);

/* The Philox4x32-10 generator every stochastic stage draws from, evaluated
 * on caller-given inputs; it has no counterpart in the reference (whose
 * draws come from numpy's global Mersenne Twister) and exists so that tests
 * can hold the device generator to the published Random123 known-answer
 * vectors.  in: n x 6 uint32 (counter words 0..3, key words 0..1), out:
 * n x 4 uint32, both device memory. */
int mgpu_philox4x32_10(const uint32_t* in, uint32_t* out, int64_t n, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MARXS_GB300_H */
