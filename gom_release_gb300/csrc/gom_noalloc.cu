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
//   * at most GOM_NOALLOC_MAX_CELLS rows (262144): 9 work vectors of that length plus the
//     reduction partials, about 19 MB per GPU;
//   * every call shares the one array, and a call leaves its contents behind: the barrier
//     counter, iteration count and status are cleared at the start of each call, the vectors are
//     fully rewritten before they are read; calls that overlap on the GPU (two streams, two
//     threads) race on the array and must be serialised by the caller;
//   * the solver is a cooperative kernel that spins on grid barriers: it must not run at the same
//     time as another spinning solve of this library (a context's free-surface phase), or the two
//     grids can each wait for blocks the other holds until the barrier's time limit reports
//     GOM_E_TIMEOUT -- order such work on one stream (gom_stream of the context) or serialise it;
//   * the first call on a device reads the solver's occupancy and the SM count once; make that
//     first call before any stream capture.  The array's device address is looked up with
//     cudaGetSymbolAddress on every call, in the caller's current context, so it never goes stale.
#include <mutex>

#include "gom_launch.h"
#include "gom_pcg.cuh"

#define GOM_NOALLOC_MAX_CELLS 262144
#define GOM_NOALLOC_MAX_BLOCKS 1024
#define GOM_NOALLOC_MAX_DEVICES 64

namespace {

using namespace gom;

// doubles: dr | xs | p | r0 | r1 | s0 | s1 | w0 | w1 (9 x MAX_CELLS) | gamma and delta partials
// (2 halves x MAX_BLOCKS each) | control block (barrier counter, iteration count, status)
constexpr size_t kVec = GOM_NOALLOC_MAX_CELLS;
constexpr size_t kNumVec = 9;
constexpr size_t kPartials = 2 * GOM_NOALLOC_MAX_BLOCKS;
constexpr size_t kControlDoubles = 16;
constexpr size_t kScratchDoubles = kNumVec * kVec + 2 * kPartials + kControlDoubles;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

struct LaunchInfo {
    int num_sms = 0;
    bool ready = false;
};

std::mutex g_setup_mutex;
LaunchInfo g_devices[GOM_NOALLOC_MAX_DEVICES];

// Once per device, with that device current: the SM count, and checks that one block of either
// solver form fits on an SM and that the device runs cooperative launches.
int setup_device(int dev, int *num_sms) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    LaunchInfo &s = g_devices[dev];
    if (!s.ready) {
        int per_sm = 0, sms = 0, coop = 0;
        for (const void *k : {(const void *)k_pcg_cg1<PCG_CG_ROWS>, (const void *)k_pcg_cg1<0>})
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, PCG_CG_THREADS, 0) != cudaSuccess ||
                per_sm < 1)
                return GOM_E_CUDA;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GOM_E_CUDA;
        if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop)
            return GOM_E_CUDA;
        s.num_sms = sms;
        s.ready = true;
    }
    *num_sms = s.num_sms;
    return GOM_OK;
}

}  // namespace

extern "C" int gom_pcg_solve_noalloc(int32_t n_cells, const int32_t *tri_or_quad, const int32_t *adj_cellnum_at_cell,
                                     const double *sparsem, const double *rhs, double *x, int32_t max_iteration,
                                     double error_tolerance, void *stream, int32_t *iterations,
                                     int32_t *device_result) {
    if (n_cells <= 0 || n_cells > GOM_NOALLOC_MAX_CELLS) return GOM_E_ARG;   // beyond the fixed scratch
    if (!tri_or_quad || !adj_cellnum_at_cell || !sparsem || !rhs || !x || max_iteration < 0) return GOM_E_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= GOM_NOALLOC_MAX_DEVICES) return GOM_E_CUDA;
    int num_sms = 0;
    int rc = setup_device(dev, &num_sms);
    if (rc != GOM_OK) return rc;
    if (num_sms > GOM_NOALLOC_MAX_BLOCKS) return GOM_E_ARG;   // the grid has at most one block per SM
    // the device address of the array in the current context (host code cannot use its name)
    double *base = nullptr;
    if (cudaGetSymbolAddress((void **)&base, g_noalloc_scratch) != cudaSuccess || !base) return GOM_E_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    double *control = base + kNumVec * kVec + 2 * kPartials;
    unsigned *bar = reinterpret_cast<unsigned *>(control);                  // barrier counter
    int *iters_dev = reinterpret_cast<int *>(control + 1);
    gom_status *status_dev = reinterpret_cast<gom_status *>(control + 2);    // 32 bytes
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
    a.dr = base + 0 * kVec;
    a.xs = base + 1 * kVec;
    a.p = base + 2 * kVec;
    a.r[0] = base + 3 * kVec;
    a.r[1] = base + 4 * kVec;
    a.s[0] = base + 5 * kVec;
    a.s[1] = base + 6 * kVec;
    a.w[0] = base + 7 * kVec;
    a.w[1] = base + 8 * kVec;
    a.pg = base + kNumVec * kVec;
    a.pd = base + kNumVec * kVec + kPartials;
    a.bar = bar;
    a.iters = iters_dev;
    a.maxit = max_iteration;
    a.tol = error_tolerance;
    a.st = status_dev;
    a.phantom = 0;
    a.check_diag = 1;   // the caller built the system: a non-positive diagonal is GOM_E_NOT_SPD
    cudaLaunchConfig_t cfg = {};
    cfg.stream = st;
    if (launch_pcg_cg1(cfg, a, num_sms) != cudaSuccess) return GOM_E_CUDA;
    // status code and iteration count into the caller's device memory, ordered on `stream`
    if (device_result) {
        if (cudaMemcpyAsync(device_result, &status_dev->code, sizeof(int32_t), cudaMemcpyDeviceToDevice, st) !=
                cudaSuccess ||
            cudaMemcpyAsync(device_result + 1, iters_dev, sizeof(int32_t), cudaMemcpyDeviceToDevice, st) !=
                cudaSuccess)
            return GOM_E_CUDA;
    }
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
