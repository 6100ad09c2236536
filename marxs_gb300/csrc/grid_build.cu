// Uniform candidate grid for a facet array (nearest-hit lookup).
//
// MARXS has no acceleration structure: Parallel.__call__ intersects every
// facet with every photon (simulator.py:42-49).  Here each facet's
// rectangle is projected onto the array's mean plane (origin o, normal n,
// axes a, b).  A ray that hits the facet at depth delta = (P - o).n crosses
// the mean plane within |delta| * slope_max of the hit point (u, v), as
// long as its slopes |d.a / d.n|, |d.b / d.n| stay below slope_max; the
// kernels send steeper rays to an all-facet scan.  So registering the facet
// in every cell its footprint box, grown by max|delta| * slope_max + margin,
// overlaps gives each cell a superset of the facets a ray through that cell
// can hit.  Lists are built as counts -> exclusive scan -> fill (CSR).
#include <atomic>
#include <cuda_runtime.h>
#include "mgpu_device.cuh"

namespace {

struct CellRange {
    int iu0, iu1, iv0, iv1;
    bool inside;
};

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
    double grow = dmax * g.slope_max + g.margin;
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

__global__ void grid_count_kernel(const mgpu_facet* facets, int n_facets, mgpu_grid g,
                                  int* counts, uint32_t* status) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_facets) return;
    CellRange r = facet_cells(facets[f], g);
    if (!r.inside) atomicOr(status, MGPU_STATUS_GRID_RANGE);
    for (int iu = r.iu0; iu <= r.iu1; ++iu)
        for (int iv = r.iv0; iv <= r.iv1; ++iv) atomicAdd(counts + iu * g.nv + iv, 1);
}

// exclusive scan of n counts into start[0..n] by one block; counts is
// overwritten with the start offsets (used as fill cursors)
__global__ void grid_scan_kernel(int* counts, int n, int* start) {
    __shared__ int s_part[1024];
    const int t = threadIdx.x, T = blockDim.x;
    const int chunk = (n + T - 1) / T;
    const int lo = min(n, t * chunk), hi = min(n, lo + chunk);
    int sum = 0;
    for (int j = lo; j < hi; ++j) sum += counts[j];
    s_part[t] = sum;
    __syncthreads();
    for (int off = 1; off < T; off <<= 1) {
        int v = (t >= off) ? s_part[t - off] : 0;
        __syncthreads();
        s_part[t] += v;
        __syncthreads();
    }
    int run = s_part[t] - sum;
    for (int j = lo; j < hi; ++j) {
        int c = counts[j];
        start[j] = run;
        counts[j] = run;
        run += c;
    }
    if (t == T - 1) start[n] = s_part[T - 1];
}

__global__ void grid_fill_kernel(const mgpu_facet* facets, int n_facets, mgpu_grid g,
                                 int* cursor, uint32_t* status) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_facets) return;
    CellRange r = facet_cells(facets[f], g);
    for (int iu = r.iu0; iu <= r.iu1; ++iu)
        for (int iv = r.iv0; iv <= r.iv1; ++iv) {
            int slot = atomicAdd(cursor + iu * g.nv + iv, 1);
            if (slot < g.capacity) g.cell_items[slot] = f;
            else atomicOr(status, MGPU_STATUS_GRID_FULL);
        }
}

// candidate order inside a cell does not change results (ties resolve to
// the lower facet index); sorting keeps the lists reproducible anyway
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
    cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int) * (size_t)(n_cells + 1), stream);
    if (e != cudaSuccess) return e;
    const int T = 128;
    if (n_facets > 0) {
        grid_count_kernel<<<(n_facets + T - 1) / T, T, 0, stream>>>(facets, n_facets, g, counts, status);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    grid_scan_kernel<<<1, 1024, 0, stream>>>(counts, n_cells, g.cell_start);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (n_facets > 0) {
        grid_fill_kernel<<<(n_facets + T - 1) / T, T, 0, stream>>>(facets, n_facets, g, counts, status);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    grid_sort_kernel<<<(n_cells + T - 1) / T, T, 0, stream>>>(g.cell_start, n_cells, g.capacity,
                                                               g.cell_items);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Allocation-free grid build.
//
// Some callers cannot allocate device memory when they (re)build the facet
// candidate grid: a host application that has handed (nearly) all device
// memory to its own pool, or a loop that must not call cudaMalloc/cudaFree
// because those synchronise the device and stall its other streams.  This
// variant keeps the build's scratch -- one counter per grid cell -- in the
// fixed array below instead of caller-provided memory.  The array holds
// MGPU_NOALLOC_MAX_CELLS + 1 int32 (256 KiB) on every GPU that loads the
// library, for the life of the process.
// ---------------------------------------------------------------------------
static __device__ __align__(256) int32_t g_noalloc_counts[MGPU_NOALLOC_MAX_CELLS + 1];

namespace {
constexpr int kNoallocMaxDevices = 64;
std::atomic<void*> g_noalloc_addr[kNoallocMaxDevices];
}  // namespace

extern "C" int mgpu_facet_grid_build_noalloc(const mgpu_facet* facets, int32_t n_facets,
                                             mgpu_grid* grid, uint32_t* status, void* stream) {
    if (grid == nullptr || status == nullptr) return (int)cudaErrorInvalidValue;
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
