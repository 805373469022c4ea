// gom_noalloc.cu -- the free-surface Jacobi-PCG solve for callers that cannot allocate device
// memory.
//
// Who needs it: a host program whose device memory comes from a runtime it does not control --
// e.g. a Fortran driver whose arrays live in OpenACC or CUDA Fortran data regions, or code that
// runs where cudaMalloc is forbidden (inside a memory-pool-managed service, or a component that
// must not grow the device footprint after start-up).  Such a caller has its matrix, right-hand
// side and solution in device memory already but no way to create the solver's work vectors.
//
// This entry point keeps those work vectors in one file-scope device array of fixed size, so a
// call allocates nothing: no cudaMalloc, no cudaFree, no allocating library routine.  The array
// exists on every GPU that loads the library for the life of the process.
//
// Limits and rules:
//   * at most GOM_NOALLOC_MAX_CELLS rows (262144): 6 work vectors of that length plus the
//     reduction partials, about 12 MB per GPU;
//   * every call shares the one array, and a call leaves its contents behind: the barrier
//     counters, iteration count and status are cleared at the start of each call, the vectors are
//     fully rewritten before they are read; calls that overlap on the GPU (two streams, two
//     threads) race on the array and must be serialised by the caller;
//   * the first call on a device looks up the array's device address (cudaGetSymbolAddress) and
//     the solver's occupancy; make that first call before any stream capture.
#include <mutex>

#include "gom_launch.h"
#include "gom_pcg.cuh"

#define GOM_NOALLOC_MAX_CELLS 262144
#define GOM_NOALLOC_MAX_BLOCKS 1024
#define GOM_NOALLOC_MAX_DEVICES 64

namespace {

using namespace gom;

// doubles: minv | r | s | q | d0 | d1 (6 x MAX_CELLS) | partial_dq | partial_delta (MAX_BLOCKS each)
// | control block (barrier counters, iteration count, status)
constexpr size_t kVec = GOM_NOALLOC_MAX_CELLS;
constexpr size_t kControlDoubles = 16;
constexpr size_t kScratchDoubles = 6 * kVec + 2 * GOM_NOALLOC_MAX_BLOCKS + kControlDoubles;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

struct ScratchInfo {
    double *base = nullptr;   // device address of g_noalloc_scratch on this device
    int per_sm = 0;
    int num_sms = 0;
    bool ready = false;
};

std::mutex g_setup_mutex;
ScratchInfo g_devices[GOM_NOALLOC_MAX_DEVICES];

// Once per device, with that device current: the array's device address and launch geometry.
int setup_device(int dev, ScratchInfo **out) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    ScratchInfo &s = g_devices[dev];
    if (!s.ready) {
        double *ptr = nullptr;
        if (cudaGetSymbolAddress((void **)&ptr, g_noalloc_scratch) != cudaSuccess) return GOM_E_CUDA;
        int per_sm = 0, sms = 0, coop = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg, PCG_THREADS, 0) != cudaSuccess)
            return GOM_E_CUDA;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GOM_E_CUDA;
        if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop)
            return GOM_E_CUDA;
        s.base = ptr;
        s.per_sm = per_sm;
        s.num_sms = sms;
        s.ready = true;
    }
    *out = &s;
    return GOM_OK;
}

}  // namespace

extern "C" int gom_pcg_solve_noalloc(int32_t n_cells, const int32_t *tri_or_quad, const int32_t *adj_cellnum_at_cell,
                                     const double *sparsem, const double *rhs, double *x, int32_t max_iteration,
                                     double error_tolerance, void *stream, int32_t *iterations) {
    if (n_cells <= 0 || n_cells > GOM_NOALLOC_MAX_CELLS) return GOM_E_ARG;   // beyond the fixed scratch
    if (!tri_or_quad || !adj_cellnum_at_cell || !sparsem || !rhs || !x || max_iteration < 0) return GOM_E_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= GOM_NOALLOC_MAX_DEVICES) return GOM_E_CUDA;
    ScratchInfo *info = nullptr;
    int rc = setup_device(dev, &info);
    if (rc != GOM_OK) return rc;
    const int blocks = pcg_blocks_for(n_cells, info->per_sm, info->num_sms);
    if (blocks > GOM_NOALLOC_MAX_BLOCKS) return GOM_E_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    double *base = info->base;
    double *control = base + 6 * kVec + 2 * GOM_NOALLOC_MAX_BLOCKS;
    unsigned *bar = reinterpret_cast<unsigned *>(control);                  // [count, generation]
    int *iters_dev = reinterpret_cast<int *>(control + 1);
    gom_status *status_dev = reinterpret_cast<gom_status *>(control + 2);    // 24 bytes
    // the barrier, iteration count and status must start at zero; the vectors are written
    // before they are read
    if (cudaMemsetAsync(control, 0, kControlDoubles * sizeof(double), st) != cudaSuccess) return GOM_E_CUDA;
    Geom g = {};
    g.NC = n_cells;
    g.tri_or_quad = tri_or_quad;
    g.adj_cellnum_at_cell = adj_cellnum_at_cell;
    PcgArgs a;
    a.g = g;
    a.sp = sparsem;
    a.b = rhs;
    a.x = x;
    a.minv = base + 0 * kVec;
    a.r = base + 1 * kVec;
    a.s = base + 2 * kVec;
    a.q = base + 3 * kVec;
    a.dA = base + 4 * kVec;
    a.dB = base + 5 * kVec;
    a.pdq = base + 6 * kVec;
    a.pdelta = base + 6 * kVec + GOM_NOALLOC_MAX_BLOCKS;
    a.bar = bar;
    a.iters = iters_dev;
    a.maxit = max_iteration;
    a.tol = error_tolerance;
    a.st = status_dev;
    a.phantom = 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(PCG_THREADS);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, k_pcg, a) != cudaSuccess) return GOM_E_CUDA;
    if (!iterations) return GOM_OK;   // asynchronous: the caller orders its own reads on `stream`
    struct {
        int iters;
        gom_status status;
    } out = {};
    if (cudaMemcpyAsync(&out.iters, iters_dev, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&out.status, status_dev, sizeof(gom_status), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return GOM_E_CUDA;
    *iterations = out.iters;
    return out.status.code;
}
