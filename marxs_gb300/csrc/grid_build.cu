// Uniform candidate grid for a facet array (nearest-hit lookup).
//
// MARXS has no acceleration structure: Parallel.__call__ intersects every
// facet with every photon (simulator.py:42-49).  Here each facet's
// rectangle is projected onto the array's mean plane (origin o, normal n,
// axes a, b).  A ray with slopes su = d.a / d.n, sv = d.b / d.n below
// slope_max crosses the plane at (u0, v0) and is looked up at
// (u1, v1) = (u0, v0) + (su, sv) D(u0, v0), D the depth model of the facet
// surface (a quadric in (u, v), or zero: the plane itself); steeper rays go
// to an all-facet scan.  A ray that hits a facet at X (coordinates uX, vX,
// depth hX) has u1 - uX = -su (hX - D(u0, v0)), and
//   |hX - D(u0, v0)| <= |hX - D(uX, vX)| + L slope_max |hX|
// with L >= |dD/du| + |dD/dv| over the grid (the drift (u0 - uX, v0 - vX)
// is at most slope_max |hX| per axis).  So registering the facet in every
// cell its footprint box, grown by
//   slope_max (max |h - D| over the facet + L slope_max max |h|) + margin,
// overlaps gives each cell a superset of the facets a ray looked up there
// can hit.  (With D = 0 the growth is max|h| slope_max + margin.)  Lists
// are built as counts -> exclusive scan -> fill (CSR).
#include <atomic>
#include <cuda_runtime.h>
#include "mgpu_device.cuh"

namespace {

struct CellRange {
    int iu0, iu1, iv0, iv1;
    bool inside;
};

__device__ __forceinline__ double depth_at(const mgpu_grid& g, double u, double v) {
    const double* d = g.depth;
    return d[0] + u * (d[1] + d[3] * u + d[4] * v) + v * (d[2] + d[5] * v);
}

// max over the facet rectangle of |depth - D(u, v)|: a quadratic in the
// rectangle's coordinates (s, t) in [-1, 1]^2, largest in magnitude at a
// corner, at an edge's stationary point or at the interior one
__device__ double facet_depth_deviation(d3 c, d3 ey, d3 ez, double hy, double hz,
                                        const mgpu_grid& g) {
    const d3 o = arr3(g.o), n = arr3(g.n), a = arr3(g.a), b = arr3(g.b);
    auto q = [&](double s, double t) {
        const d3 p = c + (s * hy) * ey + (t * hz) * ez - o;
        return dot3(p, n) - depth_at(g, dot3(p, a), dot3(p, b));
    };
    const double q0 = q(0.0, 0.0), qp0 = q(1.0, 0.0), qm0 = q(-1.0, 0.0);
    const double q0p = q(0.0, 1.0), q0m = q(0.0, -1.0);
    const double qs = 0.5 * (qp0 - qm0), qt = 0.5 * (q0p - q0m);
    const double qss = 0.5 * (qp0 + qm0) - q0, qtt = 0.5 * (q0p + q0m) - q0;
    const double qst = 0.25 * (q(1.0, 1.0) - q(1.0, -1.0) - q(-1.0, 1.0) + q(-1.0, -1.0));
    auto Q = [&](double s, double t) {
        return fabs(q0 + qs * s + qt * t + qss * s * s + qst * s * t + qtt * t * t);
    };
    double best = 0.0;
    for (int k = 0; k < 4; ++k) best = fmax(best, Q((k & 1) ? 1.0 : -1.0, (k & 2) ? 1.0 : -1.0));
    for (int k = 0; k < 2; ++k) {
        const double e = k ? 1.0 : -1.0;
        const double ts = -(qt + e * qst) / (2.0 * qtt);       // edge s = e
        if (isfinite(ts) && fabs(ts) < 1.0) best = fmax(best, Q(e, ts));
        const double ss = -(qs + e * qst) / (2.0 * qss);       // edge t = e
        if (isfinite(ss) && fabs(ss) < 1.0) best = fmax(best, Q(ss, e));
    }
    const double det = 4.0 * qss * qtt - qst * qst;
    const double si = (-2.0 * qtt * qs + qst * qt) / det, ti = (-2.0 * qss * qt + qst * qs) / det;
    if (isfinite(si) && isfinite(ti) && fabs(si) < 1.0 && fabs(ti) < 1.0) best = fmax(best, Q(si, ti));
    return best;
}

__device__ CellRange facet_cells(const mgpu_facet& f, const mgpu_grid& g) {
    d3 c = arr3(f.c), ey = arr3(f.ey), ez = arr3(f.ez);
    d3 o = arr3(g.o), n = arr3(g.n), a = arr3(g.a), b = arr3(g.b);
    double umin = 1e300, umax = -1e300, vmin = 1e300, vmax = -1e300, dmax = 0.0;
    for (int s = 0; s < 4; ++s) {
        double sy = (s & 1) ? 1.0 : -1.0, sz = (s & 2) ? 1.0 : -1.0;
        d3 corner = c + (sy * f.hy) * ey + (sz * f.hz) * ez;
        d3 rel = corner - o;
        double u = dot3(rel, a), v = dot3(rel, b), dep = fabs(dot3(rel, n));
        umin = fmin(umin, u);
        umax = fmax(umax, u);
        vmin = fmin(vmin, v);
        vmax = fmax(vmax, v);
        dmax = fmax(dmax, dep);
    }
    const double dev = facet_depth_deviation(c, ey, ez, f.hy, f.hz, g);
    double grow = g.slope_max * (dev + g.depth_lip * g.slope_max * dmax) + g.margin;
    double fu0 = floor((umin - grow - g.u0) / g.cell), fu1 = floor((umax + grow - g.u0) / g.cell);
    double fv0 = floor((vmin - grow - g.v0) / g.cell), fv1 = floor((vmax + grow - g.v0) / g.cell);
    CellRange r;
    r.inside = fu0 >= 0.0 && fv0 >= 0.0 && fu1 < (double)g.nu && fv1 < (double)g.nv;
    r.iu0 = (int)fmax(fu0, 0.0);
    r.iv0 = (int)fmax(fv0, 0.0);
    r.iu1 = (int)fmin(fu1, (double)(g.nu - 1));
    r.iv1 = (int)fmin(fv1, (double)(g.nv - 1));
    return r;
}

// one warp per facet: the lanes share the facet's cell rectangle
__global__ void grid_count_kernel(const mgpu_facet* facets, int n_facets, mgpu_grid g,
                                  int* counts, uint32_t* status) {
    const int f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (f >= n_facets) return;
    CellRange r = facet_cells(facets[f], g);
    if (!r.inside && lane == 0) atomicOr(status, MGPU_STATUS_GRID_RANGE);
    const int nv = r.iv1 - r.iv0 + 1, nu = r.iu1 - r.iu0 + 1;
    if (nu <= 0 || nv <= 0) return;
    for (int k = lane; k < nu * nv; k += 32)
        atomicAdd(counts + (r.iu0 + k / nv) * g.nv + (r.iv0 + k % nv), 1);
}

// Exclusive scan of the n cell counts into start[0..n] in three steps: the
// sum of every kScanChunk-cell chunk, a scan of those sums (one block), and
// a block scan of each chunk from its offset.  counts is overwritten with
// the start offsets (the fill cursors); sums is scratch of one int per chunk.
constexpr int kScanThreads = 256;
constexpr int kScanPer = 16;
constexpr int kScanChunk = kScanThreads * kScanPer;

__device__ __forceinline__ int block_exclusive_scan(int v, int* s_warp) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(MGPU_FULL_MASK, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[w] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int k = 0; k < kScanThreads / 32; ++k) {
            const int t = s_warp[k];
            s_warp[k] = run;
            run += t;
        }
        s_warp[kScanThreads / 32] = run;
    }
    __syncthreads();
    return s_warp[w] + x - v;
}

__global__ void __launch_bounds__(kScanThreads)
grid_scan_sums(const int* counts, int n, int* sums) {
    __shared__ int s_warp[kScanThreads / 32 + 1];
    const int a = blockIdx.x * kScanChunk + threadIdx.x * kScanPer;
    int v = 0;
    for (int j = 0; j < kScanPer; ++j)
        if (a + j < n) v += counts[a + j];
    block_exclusive_scan(v, s_warp);
    if (threadIdx.x == 0) sums[blockIdx.x] = s_warp[kScanThreads / 32];
}

__global__ void __launch_bounds__(kScanThreads)
grid_scan_top(int* sums, int nb, int* total) {
    __shared__ int s_warp[kScanThreads / 32 + 1];
    // nb sums in chunks of kScanThreads, each scanned by the block and offset
    int carry = 0;
    for (int c0 = 0; c0 < nb; c0 += kScanThreads) {
        const int i = c0 + threadIdx.x;
        const int v = i < nb ? sums[i] : 0;
        const int ex = block_exclusive_scan(v, s_warp);
        if (i < nb) sums[i] = carry + ex;
        carry += s_warp[kScanThreads / 32];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(kScanThreads)
grid_scan_apply(int* counts, int n, int* start, const int* sums) {
    __shared__ int s_warp[kScanThreads / 32 + 1];
    const int a = blockIdx.x * kScanChunk + threadIdx.x * kScanPer;
    int c[kScanPer];
    int v = 0;
#pragma unroll
    for (int j = 0; j < kScanPer; ++j) {
        c[j] = (a + j < n) ? counts[a + j] : 0;
        v += c[j];
    }
    int run = sums[blockIdx.x] + block_exclusive_scan(v, s_warp);
#pragma unroll
    for (int j = 0; j < kScanPer; ++j) {
        if (a + j < n) {
            start[a + j] = run;
            counts[a + j] = run;
        }
        run += c[j];
    }
}

__global__ void grid_fill_kernel(const mgpu_facet* facets, int n_facets, mgpu_grid g,
                                 int* cursor, uint32_t* status) {
    const int f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (f >= n_facets) return;
    CellRange r = facet_cells(facets[f], g);
    const int nv = r.iv1 - r.iv0 + 1, nu = r.iu1 - r.iu0 + 1;
    if (nu <= 0 || nv <= 0) return;
    for (int k = lane; k < nu * nv; k += 32) {
        const int slot = atomicAdd(cursor + (r.iu0 + k / nv) * g.nv + (r.iv0 + k % nv), 1);
        if (slot < g.capacity) g.cell_items[slot] = f;
        else atomicOr(status, MGPU_STATUS_GRID_FULL);
    }
}

__global__ void grid_sort_kernel(const int* start, int n_cells, int capacity, int* items) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_cells) return;
    int s0 = min(start[c], capacity), s1 = min(start[c + 1], capacity);
    for (int i = s0 + 1; i < s1; ++i) {
        int v = items[i], j = i - 1;
        while (j >= s0 && items[j] > v) {
            items[j + 1] = items[j];
            --j;
        }
        items[j + 1] = v;
    }
}

}  // namespace

cudaError_t mgpu_launch_grid_build(const mgpu_facet* facets, int n_facets, const mgpu_grid& g,
                                   int* counts, uint32_t* status, cudaStream_t stream) {
    const int n_cells = g.nu * g.nv;
    const int nb = (n_cells + kScanChunk - 1) / kScanChunk;
    int* sums = counts + n_cells + 1;          // scratch after the counters
    cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int) * (size_t)(n_cells + 1), stream);
    if (e != cudaSuccess) return e;
    const int T = 128;                         // 4 facets (warps) per block
    const int fb = (int)(((int64_t)n_facets * 32 + T - 1) / T);
    if (n_facets > 0) {
        grid_count_kernel<<<fb, T, 0, stream>>>(facets, n_facets, g, counts, status);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (nb > 0) {
        grid_scan_sums<<<nb, kScanThreads, 0, stream>>>(counts, n_cells, sums);
        grid_scan_top<<<1, kScanThreads, 0, stream>>>(sums, nb, g.cell_start + n_cells);
        grid_scan_apply<<<nb, kScanThreads, 0, stream>>>(counts, n_cells, g.cell_start, sums);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (n_facets > 0) {
        grid_fill_kernel<<<fb, T, 0, stream>>>(facets, n_facets, g, counts, status);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    grid_sort_kernel<<<(n_cells + T - 1) / T, T, 0, stream>>>(g.cell_start, n_cells, g.capacity,
                                                               g.cell_items);
    return cudaGetLastError();
}

static __device__ __align__(256) int32_t
    g_noalloc_counts[MGPU_NOALLOC_MAX_CELLS + 1 + (MGPU_NOALLOC_MAX_CELLS + kScanChunk - 1) / kScanChunk];

namespace {
constexpr int kNoallocMaxDevices = 64;
std::atomic<void*> g_noalloc_addr[kNoallocMaxDevices];
}  // namespace

extern "C" int mgpu_facet_grid_build_noalloc(const mgpu_facet* facets, int32_t n_facets,
                                             mgpu_grid* grid, uint32_t* status, void* stream) {
    if (grid == nullptr || status == nullptr) return (int)cudaErrorInvalidValue;
    if (n_facets < 0 || (n_facets > 0 && facets == nullptr)) return (int)cudaErrorInvalidValue;
    if (grid->nu <= 0 || grid->nv <= 0 || grid->cell_start == nullptr || grid->cell_items == nullptr)
        return (int)cudaErrorInvalidValue;
    if ((long long)grid->nu * (long long)grid->nv > MGPU_NOALLOC_MAX_CELLS)
        return MGPU_ERR_NOALLOC_LIMIT;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    if (dev < 0 || dev >= kNoallocMaxDevices) return (int)cudaErrorInvalidDevice;
    // the host-side name of the array is not a device address: look the
    // address up once per device, with that device current (first call)
    void* scratch = g_noalloc_addr[dev].load(std::memory_order_acquire);
    if (scratch == nullptr) {
        e = cudaGetSymbolAddress(&scratch, g_noalloc_counts);
        if (e != cudaSuccess) return (int)e;
        g_noalloc_addr[dev].store(scratch, std::memory_order_release);
    }
    // mgpu_launch_grid_build clears the counters before use, so a call never
    // sees the previous call's contents
    return (int)mgpu_launch_grid_build(facets, n_facets, *grid, (int*)scratch, status,
                                       (cudaStream_t)stream);
}
