// gom_core.cu -- the C ABI of include/gom_core.h on a GB300 (sm_103a).
//
// A context owns: the static geometry copied to HBM once, every state array of the time loop
// resident in HBM in the reference's (k, entity) layout, the work buffers of the phases, one
// CUDA stream, pinned staging for the per-step forcing, and a CUDA graph of the whole timestep
// (captured on first use of gom_step_all).  Host arrays are read only during a call.
#include <cmath>
#include <cstdio>
#include <mutex>
#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "gom_launch.h"
#include "gom_scan.cuh"

using namespace gom;

namespace {

struct FieldDesc {
    void **dev;      // address of the State member
    int lo;          // -1: 1-D entity array; else lower layer bound (0 or 1)
    int kind;        // 0 cells, 1 faces, 2 nodes, 3 river cells
    int is_int;
    int dev_bytes;   // element size on the device: 4 (int32 or FP32 storage) or 8
};

}  // namespace

struct gom_ctx {
    gom_dims d{};
    gom_params hp{};
    Launch x;             // FP64 context; in a mixed context it holds the shared pieces
    LaunchT<float> xf;    // mixed context: FP32 layered state, shared geometry/forcing/PCG work
    bool mixed = false;
    int device = 0;
    std::vector<void *> allocs;
    size_t bytes = 0;     // device memory held by the context
    std::vector<int> run_starts[4];   // packed runs: host copies of run_{cell,face,node,ob}_start
    std::string msg;
    FieldDesc fields[GOM_F_COUNT];
    // forcing arrays on the device (the Forcing view points into these)
    double *f_scal = nullptr;
    double *f_eta_old = nullptr, *f_eta_new = nullptr, *f_q_add = nullptr, *f_wsn = nullptr, *f_wst = nullptr,
           *f_gamma_t = nullptr, *f_air_p = nullptr, *f_con_ob = nullptr, *f_con_qb = nullptr, *f_phi_sw = nullptr,
           *f_phi_sz = nullptr;
    // pinned host mirrors
    gom_status *h_status = nullptr;
    int *h_iters = nullptr;
    double *h_cons = nullptr;
    double *h_stage = nullptr;      // two halves, used alternately by consecutive uploads
    size_t stage_len = 0;           // doubles per half
    int stage_half = 0;
    cudaEvent_t stage_done[2] = {nullptr, nullptr};
    bool step_pending = false;
    long long pcg_total = 0;
    // the timestep as three captured graphs: before the free surface, the free surface (whose
    // cooperative PCG runs on the process-wide solver stream, one solve at a time on the GPU),
    // after it
    cudaGraphExec_t graph = nullptr, graph_fs = nullptr, graph_post = nullptr;
    cudaEvent_t ev_to_solver = nullptr, ev_from_solver = nullptr;
    bool graph_failed = false;
    // device-side storm forcing (gom_set_storms)
    double *d_storms = nullptr, *storm_wu = nullptr, *storm_wv = nullptr;
    int n_storms = 0;
    // device-side boundary series (gom_set_boundary_series): their own device allocations
    SeriesDev series{};
    bool has_series = false;
    std::vector<void *> series_allocs;
    size_t series_bytes = 0;
    // asynchronous output snapshots (gom_snapshot_begin): device staging area, copy stream
    char *snap_dev = nullptr;
    size_t snap_cap = 0;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_snap_staged = nullptr, ev_snap_done = nullptr;
    bool snap_pending = false;
    // station time series (gom_set_stations): station ids and the records, on the device
    int *st_ids = nullptr;
    double *st_out = nullptr;
    int st_n = 0, st_hloc = 0;
};

namespace {

int set_cuda_error(gom_ctx *c, cudaError_t e, const char *where) {
    if (e == cudaSuccess) return GOM_OK;
    if (c) {
        c->msg = std::string(where) + ": " + cudaGetErrorString(e);
        if (c->h_status && c->h_status->code == 0) c->h_status->code = GOM_E_CUDA;
    }
    return e == cudaErrorMemoryAllocation ? GOM_E_NOMEM : GOM_E_CUDA;
}

#define CK(call)                                                          \
    do {                                                                  \
        cudaError_t _e = (call);                                          \
        if (_e != cudaSuccess) return set_cuda_error(c, _e, #call);      \
    } while (0)

// Host-side setup writes (zeroing, uploads) go through the legacy default stream, which does not
// order with the context's non-blocking streams; each one is completed before the call returns,
// so no kernel of the context can run before (or under) it.
cudaError_t legacy_done() { return cudaStreamSynchronize(0); }

template <typename T> cudaError_t dalloc(gom_ctx *c, T **p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e == cudaSuccess) {
        c->allocs.push_back(*p);
        c->bytes += n * sizeof(T);
        e = cudaMemset(*p, 0, n * sizeof(T));
        if (e == cudaSuccess) e = legacy_done();
    }
    return e;
}

// transport and node-velocity work arrays in the layered-state type
template <typename R> cudaError_t alloc_layered_work(gom_ctx *c, WorkT<R> &W) {
    const size_t NC = c->d.n_cells, NF = c->d.n_faces, L = c->d.n_layers;
    const size_t NOB = (size_t)c->d.n_ob, NQB = (size_t)c->d.n_qb;
    cudaError_t e = cudaSuccess;
    R **two[] = {&W.con, &W.con2};
    for (R **p : two)
        if (e == cudaSuccess) e = dalloc(c, p, (L + 2) * NC * 2);
    R **face_l[] = {&W.qj, &W.dj, &W.phij};
    for (R **p : face_l)
        if (e == cudaSuccess) e = dalloc(c, p, L * NF);
    R **cell_l0[] = {&W.qi, &W.di, &W.phii};
    for (R **p : cell_l0)
        if (e == cudaSuccess) e = dalloc(c, p, (L + 1) * NC);
    if (e == cudaSuccess) e = dalloc(c, &W.psij, L * NF * 2);
    if (e == cudaSuccess) e = dalloc(c, &W.psii, (L + 1) * NC * 2);
    if (e == cudaSuccess) e = dalloc(c, &W.sa1, L * NC * 2);
    if (e == cudaSuccess) e = dalloc(c, &W.sa2, L * NC * 2);
    if (e == cudaSuccess) e = dalloc(c, &W.obk, L * NOB * 2);
    if (e == cudaSuccess) e = dalloc(c, &W.qbk, L * NQB * 2);
    if (e == cudaSuccess) e = dalloc(c, &W.uflf, (L + 1) * NF);
    if (e == cudaSuccess) e = dalloc(c, &W.vflf, (L + 1) * NF);
    if (e == cudaSuccess && c->hp.turbulence_flag != 0) e = dalloc(c, &W.kvf, (L + 1) * NF);
    // rows of the vertical systems: the FP32 transport, and the FP64 list-form solve variant
    if (c->hp.transport_flag) {
        R **rows[] = {&W.tr_a, &W.tr_b, &W.tr_c};
        for (R **p : rows)
            if (e == cudaSuccess) e = dalloc(c, p, L * NC);
        if (e == cudaSuccess) e = dalloc(c, &W.tr_rhs, L * NC * 2);
    }
    // the wet cell-layer list and the top-layer limiter sums: always in the FP32 path, in the FP64
    // path for its list-form limiter variant
    if (c->hp.transport_flag) {
        if (e == cudaSuccess) e = dalloc(c, &W.tr_last, 4 * NC);
        if (e == cudaSuccess) e = dalloc(c, &W.cl_list, L * NC);
        if (e == cudaSuccess) e = dalloc(c, &W.cl_off, NC);
        if (e == cudaSuccess) e = dalloc(c, &W.cl_bsum, NC / 1024 + 2);
        if (e == cudaSuccess) e = dalloc(c, &W.cl_count, 2);
    }
    return e;
}

template <typename T> cudaError_t upload(gom_ctx *c, const T **dst, const T *src, size_t n, bool required) {
    T *p = nullptr;
    cudaError_t e = dalloc(c, &p, n);
    if (e != cudaSuccess) return e;
    if (src) e = cudaMemcpy(p, src, n * sizeof(T), cudaMemcpyHostToDevice);
    else if (required) e = cudaErrorInvalidValue;
    if (e == cudaSuccess) e = legacy_done();   // the DMA of a pageable copy may still be running
    *dst = p;
    return e;
}

int64_t field_count(const gom_dims &d, const FieldDesc &f) {
    int64_t n = f.kind == 0 ? d.n_cells : f.kind == 1 ? d.n_faces : f.kind == 2 ? d.n_nodes : f.kind == 3 ? d.n_qb : d.n_ob;
    if (f.lo < 0) return n;
    return n * (int64_t)(d.n_layers - f.lo + 1);
}

// R: storage type of the layered state (double fields stay FP64 in every context)
template <typename R> void describe_fields(gom_ctx *c, StateT<R> &s) {
    auto E = [&](int id, double **m, int lo, int kind) { c->fields[id] = FieldDesc{(void **)m, lo, kind, 0, 8}; };
    auto D = [&](int id, R **m, int lo, int kind) {
        c->fields[id] = FieldDesc{(void **)m, lo, kind, 0, (int)sizeof(R)};
    };
    auto I = [&](int id, int **m, int lo, int kind) { c->fields[id] = FieldDesc{(void **)m, lo, kind, 1, 4}; };
    for (int f = 0; f < GOM_F_COUNT; ++f) c->fields[f] = FieldDesc{nullptr, -2, 0, 0, 8};
    E(GOM_F_ETA_CELL, &s.eta_cell, -1, 0);
    E(GOM_F_ETA_CELL_NEW, &s.eta_cell_new, -1, 0);
    E(GOM_F_ETA_NODE, &s.eta_node, -1, 2);
    I(GOM_F_WETDRY_NODE, &s.wetdry_node, -1, 2);
    D(GOM_F_UN_FACE, &s.un_face, 1, 1);
    D(GOM_F_VN_FACE, &s.vn_face, 1, 1);
    D(GOM_F_UN_FACE_NEW, &s.un_face_new, 1, 1);
    D(GOM_F_VN_FACE_NEW, &s.vn_face_new, 1, 1);
    D(GOM_F_UN_ELM, &s.un_elm, 1, 1);
    D(GOM_F_VN_ELM, &s.vn_elm, 1, 1);
    D(GOM_F_WN_CELL, &s.wn_cell, 0, 0);
    D(GOM_F_WN_CELL_NEW, &s.wn_cell_new, 0, 0);
    D(GOM_F_U_NODE, &s.u_node, 0, 2);
    D(GOM_F_V_NODE, &s.v_node, 0, 2);
    D(GOM_F_W_NODE, &s.w_node, 0, 2);
    D(GOM_F_U_FACE_LEVEL, &s.u_face_level, 0, 1);
    D(GOM_F_V_FACE_LEVEL, &s.v_face_level, 0, 1);
    D(GOM_F_DZ_CELL, &s.dz_cell, 1, 0);
    D(GOM_F_DZ_CELL_NEW, &s.dz_cell_new, 1, 0);
    D(GOM_F_DZHALF_CELL, &s.dzhalf_cell, 0, 0);
    D(GOM_F_DZHALF_CELL_NEW, &s.dzhalf_cell_new, 0, 0);
    D(GOM_F_DZ_FACE, &s.dz_face, 1, 1);
    D(GOM_F_DZ_FACE_NEW, &s.dz_face_new, 1, 1);
    D(GOM_F_DZHALF_FACE, &s.dzhalf_face, 0, 1);
    D(GOM_F_DZHALF_FACE_NEW, &s.dzhalf_face_new, 0, 1);
    D(GOM_F_DZ_NODE, &s.dz_node, 1, 2);
    D(GOM_F_DZ_NODE_NEW, &s.dz_node_new, 1, 2);
    D(GOM_F_DZHALF_NODE, &s.dzhalf_node, 0, 2);
    D(GOM_F_DZHALF_NODE_NEW, &s.dzhalf_node_new, 0, 2);
    I(GOM_F_TOP_LAYER_CELL, &s.top_cell, -1, 0);
    I(GOM_F_TOP_LAYER_FACE, &s.top_face, -1, 1);
    I(GOM_F_TOP_LAYER_NODE, &s.top_node, -1, 2);
    D(GOM_F_AINVG1, &s.ainvg1, 1, 1);
    D(GOM_F_AINVG2, &s.ainvg2, 1, 1);
    D(GOM_F_AINVDZ1, &s.ainvdz1, 1, 1);
    D(GOM_F_AINVDZ2, &s.ainvdz2, 1, 1);
    D(GOM_F_KH, &s.kh, 1, 1);
    D(GOM_F_AV, &s.av, 0, 1);
    D(GOM_F_KV, &s.kv, 0, 0);
    D(GOM_F_SALT_CELL, &s.salt_cell, 1, 0);
    D(GOM_F_SALT_CELL_NEW, &s.salt_cell_new, 1, 0);
    D(GOM_F_TEMP_CELL, &s.temp_cell, 1, 0);
    D(GOM_F_TEMP_CELL_NEW, &s.temp_cell_new, 1, 0);
    D(GOM_F_SALT_NODE, &s.salt_node, 1, 2);
    D(GOM_F_TEMP_NODE, &s.temp_node, 1, 2);
    D(GOM_F_SALT_FACE, &s.salt_face, 1, 1);
    D(GOM_F_TEMP_FACE, &s.temp_face, 1, 1);
    E(GOM_F_RHO_CELL, &s.rho_cell, 1, 0);
    E(GOM_F_RHO_NODE, &s.rho_node, 1, 2);
    E(GOM_F_RHO_FACE, &s.rho_face, 1, 1);
    I(GOM_F_NUM_SUB_ELM, &s.num_sub_elm, 1, 2);
    D(GOM_F_CDB, &s.cdb, -1, 1);
    D(GOM_F_GAMMA_B, &s.gamma_b, -1, 1);
    E(GOM_F_QU_BOUNDARY, &s.qu_boundary, -1, 3);
    I(GOM_F_ELM_FOOT, &s.elm_foot, 1, 1);
    I(GOM_F_ELM_NEAR_EDGE, &s.elm_near_edge, 1, 1);
    // forcing arrays (allocated with the forcing, not with the state)
    E(GOM_F_WIND_STRESS_NORMAL, &c->f_wsn, -1, 1);
    E(GOM_F_WIND_STRESS_TANGNT, &c->f_wst, -1, 1);
    E(GOM_F_GAMMA_T, &c->f_gamma_t, -1, 1);
    E(GOM_F_AIR_P, &c->f_air_p, -1, 2);
    E(GOM_F_ETA_AT_OB_OLD, &c->f_eta_old, -1, 4);
    E(GOM_F_ETA_AT_OB_NEW, &c->f_eta_new, -1, 4);
    E(GOM_F_Q_ADD, &c->f_q_add, -1, 3);
    E(GOM_F_PHI_SW, &c->f_phi_sw, -1, 0);
    E(GOM_F_PHI_SZ, &c->f_phi_sz, 1, 0);
}

bool is_forcing_field(int f) { return f >= GOM_F_WIND_STRESS_NORMAL && f <= GOM_F_PHI_SZ; }

// state arrays that update_variables.f90:16-31 copies from *_new to the old name
const int kSwapPairs[][2] = {{GOM_F_ETA_CELL, GOM_F_ETA_CELL_NEW},   {GOM_F_WN_CELL, GOM_F_WN_CELL_NEW},
                             {GOM_F_DZ_CELL, GOM_F_DZ_CELL_NEW},     {GOM_F_DZHALF_CELL, GOM_F_DZHALF_CELL_NEW},
                             {GOM_F_SALT_CELL, GOM_F_SALT_CELL_NEW}, {GOM_F_TEMP_CELL, GOM_F_TEMP_CELL_NEW},
                             {GOM_F_UN_FACE, GOM_F_UN_FACE_NEW},     {GOM_F_VN_FACE, GOM_F_VN_FACE_NEW},
                             {GOM_F_DZ_FACE, GOM_F_DZ_FACE_NEW},     {GOM_F_DZHALF_FACE, GOM_F_DZHALF_FACE_NEW},
                             {GOM_F_DZ_NODE, GOM_F_DZ_NODE_NEW},     {GOM_F_DZHALF_NODE, GOM_F_DZHALF_NODE_NEW}};

cudaError_t enqueue_swap(gom_ctx *c) {
    for (auto &pr : kSwapPairs) {
        const FieldDesc &a = c->fields[pr[0]];
        const FieldDesc &b = c->fields[pr[1]];
        size_t bytes = (size_t)field_count(c->d, a) * a.dev_bytes;
        cudaError_t e = cudaMemcpyAsync(*a.dev, *b.dev, bytes, cudaMemcpyDeviceToDevice, c->x.stream);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// the phases of main.f90:94-272 in order; part 0 = up to the momentum equation, 1 = the free
// surface, 2 = the rest, -1 = all
template <typename R> cudaError_t enqueue_step_t(gom_ctx *c, const LaunchT<R> &x, int part) {
    cudaError_t e;
    if (part <= 0) {
        if (c->has_series && (e = launch_series_forcing(x.g, x.f, x.p, c->series, x.s.eta_cell, x.status, x.stream))) return e;
        if (c->n_storms > 0 &&
            (e = launch_storm_forcing(x.g, x.f, x.p, x.stream, c->d_storms, c->storm_wu, c->storm_wv)))
            return e;
        if ((e = launch_bottom_friction(x))) return e;
        if ((e = launch_boundary_velocity(x))) return e;
        if ((e = launch_advection(x))) return e;
        if ((e = launch_momentum(x))) return e;
        if (part == 0) return cudaSuccess;
    }
    if (part <= 1) {
        if ((e = launch_free_surface(x))) return e;
        if (part == 1) return cudaSuccess;
    }
    if ((e = launch_velocities(x))) return e;
    if ((e = launch_layers(x))) return e;
    if ((e = launch_node_velocity(x))) return e;
    if (c->has_series && c->series.heat_flag == 1 && (e = launch_heat_terms(x.g, x.f, x.s, c->series, x.stream)))
        return e;
    if ((e = launch_transport(x))) return e;
    if ((e = launch_density(x))) return e;
    if ((e = launch_turbulence(x))) return e;
    return enqueue_swap(c);
}

cudaError_t enqueue_step(gom_ctx *c, int part = -1) {
    return c->mixed ? enqueue_step_t(c, c->xf, part) : enqueue_step_t(c, c->x, part);
}

// One stream per device shared by every context of the process for the free-surface phase: its
// cooperative PCG kernel spins on grid barriers, and two such grids resident at once on one GPU
// (contexts stepped concurrently on their own streams) could each wait for blocks the other
// holds.  Queuing the free-surface graphs of all contexts on one stream runs one solve at a time.
std::mutex g_solver_mutex;
cudaStream_t g_solver_stream[64] = {};

cudaError_t solver_stream(int device, cudaStream_t *out) {
    if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_solver_mutex);
    if (!g_solver_stream[device]) {
        cudaError_t e = cudaStreamCreateWithFlags(&g_solver_stream[device], cudaStreamNonBlocking);
        if (e != cudaSuccess) return e;
    }
    *out = g_solver_stream[device];
    return cudaSuccess;
}

cudaError_t capture(gom_ctx *c, int part, cudaGraphExec_t *out) {
    cudaGraph_t gr = nullptr;
    cudaError_t e = cudaStreamBeginCapture(c->x.stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t e2 = enqueue_step(c, part);
        e = cudaStreamEndCapture(c->x.stream, &gr);
        if (e2 != cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(out, gr, 0);
    if (gr) cudaGraphDestroy(gr);
    return e;
}

void drop_graphs(gom_ctx *c) {
    for (cudaGraphExec_t *g : {&c->graph, &c->graph_fs, &c->graph_post}) {
        if (*g) cudaGraphExecDestroy(*g);
        *g = nullptr;
    }
}

// a phase launcher on the context's state type
#define GOM_PHASE(fn) [](gom_ctx *c) { return c->mixed ? fn(c->xf) : fn(c->x); }

// copy status and PCG iterations to pinned memory, wait, translate to a return code
int finish(gom_ctx *c, int32_t *pcg_iters, bool had_pcg) {
    CK(cudaMemcpyAsync(c->h_status, c->x.status, sizeof(gom_status), cudaMemcpyDeviceToHost, c->x.stream));
    if (had_pcg) CK(cudaMemcpyAsync(c->h_iters, c->x.w.pcg_iters, sizeof(int), cudaMemcpyDeviceToHost, c->x.stream));
    CK(cudaStreamSynchronize(c->x.stream));
    if (had_pcg) {
        c->pcg_total += *c->h_iters;
        if (pcg_iters) *pcg_iters = *c->h_iters;
    }
    return c->h_status->code;
}

// the packed run holding the entity a status names (0 in a single-run context, -1 if not known)
int status_run(const gom_ctx *c, const gom_status &st) {
    const int kind = st.entity_kind;
    if (st.code == 0 || kind < GOM_ENTITY_CELL || kind > GOM_ENTITY_NODE || st.entity < 1) return -1;
    if (c->d.n_runs <= 1) return 0;
    const std::vector<int> &v = c->run_starts[kind == GOM_ENTITY_CELL ? 0 : kind == GOM_ENTITY_FACE ? 1 : 2];
    // run r holds the 0-based entities [v[r], v[r+1])
    auto it = std::upper_bound(v.begin(), v.end(), st.entity - 1);
    int r = (int)(it - v.begin()) - 1;
    return (r >= 0 && r < c->d.n_runs) ? r : -1;
}

template <typename Fn> int run_phase(gom_ctx *c, Fn fn) {
    if (!c) return GOM_E_ARG;
    CK(fn(c));
    return finish(c, nullptr, false);
}

}  // namespace

extern "C" {

int gom_abi_version(void) { return GOM_ABI_VERSION; }

const char *gom_errstr(int code) {
    switch (code) {
    case GOM_OK: return "ok";
    case GOM_E_ARG: return "bad argument";
    case GOM_E_CUDA: return "CUDA error";
    case GOM_E_NOT_SPD: return "free-surface matrix not positive definite";
    case GOM_E_ZERO_PIVOT: return "tridiagonal solver zero pivot";
    case GOM_E_ELM: return "ELM backtracking geometry failure";
    case GOM_E_DRY: return "dry element or boundary where water is required";
    case GOM_E_LAYER: return "impossible elevation or layer";
    case GOM_E_DENSITY: return "density, salinity or temperature out of range";
    case GOM_E_PCG_MAXIT: return "PCG reached max_iteration_pcg";
    case GOM_E_TIMEOUT: return "device wait timed out";
    case GOM_E_NOMEM: return "out of device memory";
    default: return "unknown error";
    }
}

const char *gom_last_message(const gom_ctx *ctx) { return ctx ? ctx->msg.c_str() : ""; }

int gom_field_info(const gom_dims *dims, int field, int64_t *count, int32_t *elem_bytes) {
    if (!dims || field <= 0 || field >= GOM_F_COUNT) return GOM_E_ARG;
    gom_ctx tmp;
    describe_fields(&tmp, tmp.x.s);
    const FieldDesc &f = tmp.fields[field];
    if (f.lo == -2) return GOM_E_ARG;
    if (count) *count = field_count(*dims, f);
    if (elem_bytes) *elem_bytes = f.is_int ? 4 : 8;   // host-side element: int32 or FP64
    return GOM_OK;
}

int gom_create(const gom_dims *dims, const gom_params *params, const gom_geom *g, gom_ctx **out) {
    if (!dims || !params || !g || !out) return GOM_E_ARG;
    *out = nullptr;
    const gom_dims &d = *dims;
    if (d.n_cells <= 0 || d.n_faces <= 0 || d.n_nodes <= 0 || d.n_layers <= 0 || d.n_layers > GOM_MAXL ||
        d.max_nb <= 0 || d.max_nb > GOM_MAXNB || d.n_ob < 0 || d.n_qb < 0 || d.n_cells >= LIST_MAX_ENTITIES ||
        d.n_faces >= LIST_MAX_ENTITIES)
        return GOM_E_ARG;
    if (params->transport_flag && params->is_salt == 0 && params->is_temp == 1) return GOM_E_ARG;
    if (params->transport_solver < 0 || params->transport_solver > 2) return GOM_E_ARG;
    if (params->precision != GOM_PRECISION_FP64 && params->precision != GOM_PRECISION_MIXED) return GOM_E_ARG;
    if (params->turbulence_flag < 0 || params->turbulence_flag > 2) return GOM_E_ARG;
    if (params->transport_flag && params->is_temp && params->heat_option != 1 && params->heat_option != 2)
        return GOM_E_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GOM_E_CUDA;
    gom_ctx *c = new gom_ctx();
    c->d = d;
    c->hp = *params;
    cudaGetDevice(&c->device);
    c->mixed = params->precision == GOM_PRECISION_MIXED;
    if (c->mixed) describe_fields(c, c->xf.s);
    else describe_fields(c, c->x.s);
    auto fail = [&](int code) {
        gom_destroy(c);
        return code;
    };
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, c->device) != cudaSuccess) return fail(GOM_E_CUDA);
    c->x.num_sms = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&c->x.stream, cudaStreamNonBlocking) != cudaSuccess) return fail(GOM_E_CUDA);
    const size_t NC = d.n_cells, NF = d.n_faces, NN = d.n_nodes, NB = d.max_nb, L = d.n_layers;
    Geom &G = c->x.g;
    G.NC = d.n_cells;
    G.NF = d.n_faces;
    G.NN = d.n_nodes;
    G.L = d.n_layers;
    G.NB = d.max_nb;
    G.NOB = d.n_ob;
    G.NQB = d.n_qb;
    cudaError_t e = cudaSuccess;
#define UP(dst, src, n, req) \
    if (e == cudaSuccess) e = upload(c, &G.dst, g->src, n, req)
    UP(x_node, x_node, NN, true);
    UP(y_node, y_node, NN, true);
    UP(h_node, h_node, NN, true);
    UP(adj_cells_at_node, adj_cells_at_node, NN, true);
    UP(adj_cellnum_at_node, adj_cellnum_at_node, NB * NN, true);
    UP(node_count_each_element, node_count_each_element, NB * NN, true);
    UP(adj_nodes_at_node, adj_nodes_at_node, NN, true);
    UP(adj_nodenum_at_node, adj_nodenum_at_node, (NB + 1) * NN, true);
    UP(bottom_node, bottom_layer_at_node, NN, true);
    UP(initial_wetdry_node, initial_wetdry_node, NN, false);
    UP(x_cell, x_cell, NC, true);
    UP(y_cell, y_cell, NC, true);
    UP(h_cell, h_cell, NC, true);
    UP(area, area, NC, true);
    UP(tri_or_quad, tri_or_quad, NC, true);
    UP(nodenum_at_cell, nodenum_at_cell, 4 * NC, true);
    UP(facenum_at_cell, facenum_at_cell, 4 * NC, true);
    UP(adj_cellnum_at_cell, adj_cellnum_at_cell, 4 * NC, true);
    UP(sign_in_outflow, sign_in_outflow, 4 * NC, true);
    UP(bottom_cell, bottom_layer_at_element, NC, true);
    UP(ob_element_flag, ob_element_flag, NC, false);
    UP(qb_element_flag, qb_element_flag, NC, false);
    UP(x_face, x_face, NF, true);
    UP(y_face, y_face, NF, true);
    UP(h_face, h_face, NF, true);
    UP(face_length, face_length, NF, true);
    UP(delta_j, delta_j, NF, true);
    UP(cos_theta, cos_theta, NF, true);
    UP(sin_theta, sin_theta, NF, true);
    UP(cos_theta2, cos_theta2, NF, true);
    UP(sin_theta2, sin_theta2, NF, true);
    UP(coriolis_factor, coriolis_factor, NF, false);
    UP(manning, manning, NF, params->bf_flag == 1);
    UP(bf_height, bf_height, NF, params->bf_flag == 2);
    UP(adj_cellnum_at_face, adj_cellnum_at_face, 2 * NF, true);
    UP(nodenum_at_face, nodenum_at_face, 2 * NF, true);
    UP(bottom_face, bottom_layer_at_face, NF, true);
    UP(boundary_type_of_face, boundary_type_of_face, NF, true);
    UP(isflowside3, isflowside3, NF, false);
    UP(ob_cell_id, ob_cell_id, (size_t)d.n_ob, d.n_ob > 0);
    UP(qb_cell, qb_cell, (size_t)d.n_qb, d.n_qb > 0);
    UP(qb_face, qb_face, (size_t)d.n_qb, d.n_qb > 0);
    UP(z_level, z_level, L + 1, true);
    UP(delta_z, delta_z, L, true);
#undef UP
    // calculate_bottom_friction.f90:25-60 on the host where the result is static (the C library's
    // pow and log, which the reference calls)
    if (e == cudaSuccess && (params->bf_flag == 1 || params->bf_flag == 2)) {
        std::vector<double> cdb(NF, 0.0), arg(NF, -1.0);
        for (size_t j = 0; j < NF; ++j) {
            const double hf = g->h_face[j];
            if (!(hf > params->dry_depth)) continue;
            if (params->bf_flag == 1) {
                const double expo = 1.0 / 6.0;
                const double chezy = std::pow(std::max(1.0, hf), expo) / g->manning[j];
                cdb[j] = params->gravity / (chezy * chezy);
            } else {
                const int b = g->bottom_layer_at_face[j];
                if (b < 1 || b > (int)L) continue;
                arg[j] = g->z_level[b] - (params->msl - hf);
                const double lg = std::log(std::max(0.5, arg[j]) / g->bf_height[j]);
                cdb[j] = params->von_karman * params->von_karman / (lg * lg);
            }
        }
        e = upload(c, &G.cdb_static, (const double *)cdb.data(), NF, true);
        if (e == cudaSuccess) e = upload(c, &G.cdb_arg, (const double *)arg.data(), NF, true);
    }
    G.NR = d.n_runs > 1 ? d.n_runs : 1;
    if (d.n_runs > 1 && e == cudaSuccess) {
        // packed runs: each range starts at 0, never decreases and ends at the entity count
        const int32_t *starts[4] = {g->run_cell_start, g->run_face_start, g->run_node_start, g->run_ob_start};
        const int32_t totals[4] = {d.n_cells, d.n_faces, d.n_nodes, d.n_ob};
        for (int t = 0; t < 4; ++t) {
            const int32_t *v = starts[t];
            if (!v || v[0] != 0 || v[d.n_runs] != totals[t]) return fail(GOM_E_ARG);
            for (int r = 0; r < d.n_runs; ++r)
                if (v[r + 1] < v[r] || (t == 0 && v[r + 1] == v[r])) return fail(GOM_E_ARG);
        }
        const size_t NR1 = (size_t)d.n_runs + 1;
        for (int t = 0; t < 4; ++t) c->run_starts[t].assign(starts[t], starts[t] + NR1);
        e = upload(c, &G.run_cell_start, (const int *)g->run_cell_start, NR1, true);
        if (e == cudaSuccess) e = upload(c, &G.run_face_start, (const int *)g->run_face_start, NR1, true);
        if (e == cudaSuccess) e = upload(c, &G.run_node_start, (const int *)g->run_node_start, NR1, true);
        if (e == cudaSuccess) e = upload(c, &G.run_ob_start, (const int *)g->run_ob_start, NR1, true);
    }
    if (e != cudaSuccess) return fail(e == cudaErrorInvalidValue ? GOM_E_ARG : GOM_E_CUDA);
    // column orders: entity ids (1-based) stably sorted by bottom layer
    {
        auto order = [&](const int32_t *bottom, size_t n, const int **dst) {
            std::vector<int> ids(n);
            std::iota(ids.begin(), ids.end(), 1);
            std::stable_sort(ids.begin(), ids.end(), [&](int a, int b) { return bottom[a - 1] < bottom[b - 1]; });
            return upload(c, dst, (const int *)ids.data(), n, true);
        };
        if (e == cudaSuccess) e = order(g->bottom_layer_at_element, NC, &G.cell_order);
        if (e == cudaSuccess) e = order(g->bottom_layer_at_face, NF, &G.face_order);
        if (e == cudaSuccess) e = order(g->bottom_layer_at_node, NN, &G.node_order);
        if (e != cudaSuccess) return fail(GOM_E_CUDA);
    }
    // state
    for (int f = 1; f < GOM_F_COUNT && e == cudaSuccess; ++f) {
        const FieldDesc &fd = c->fields[f];
        if (fd.lo == -2 || is_forcing_field(f)) continue;
        size_t n = (size_t)field_count(d, fd);
        if (fd.is_int) e = dalloc(c, (int **)fd.dev, n);
        else if (fd.dev_bytes == 4) e = dalloc(c, (float **)fd.dev, n);
        else e = dalloc(c, (double **)fd.dev, n);
    }
    // derived per-cell arrays of the ELM walk (static bottom height; surface height and dry test
    // refreshed at the start of every advection phase)
    {
        double **ztop = c->mixed ? &c->xf.s.ztop_cell : &c->x.s.ztop_cell;
        int **dry = c->mixed ? &c->xf.s.dry_cell : &c->x.s.dry_cell;
        double *zbot = nullptr;
        if (e == cudaSuccess) e = dalloc(c, ztop, NC);
        if (e == cudaSuccess) e = dalloc(c, dry, NC);
        if (e == cudaSuccess) e = dalloc(c, &zbot, NC);
        if (e == cudaSuccess && c->mixed) e = dalloc(c, &c->xf.s.ztop_cell_f, NC);
        if (e == cudaSuccess) e = launch_cell_zbot(G, params->msl, zbot, c->x.stream);
        G.zbot_cell = zbot;
        if (c->mixed) {
            float *zbf = nullptr;
            if (e == cudaSuccess) e = dalloc(c, &zbf, NC);
            if (e == cudaSuccess) e = launch_cell_zbot_f(G, zbot, zbf, c->x.stream);
            G.zbot_cell_f = zbf;
        }
    }
    // forcing
    int nt = params->trans_sub_iter > 0 ? params->trans_sub_iter : 1;
    if (e == cudaSuccess) e = dalloc(c, &c->f_eta_old, (size_t)d.n_ob);
    if (e == cudaSuccess) e = dalloc(c, &c->f_eta_new, (size_t)d.n_ob);
    if (e == cudaSuccess) e = dalloc(c, &c->f_q_add, (size_t)d.n_qb);
    if (e == cudaSuccess) e = dalloc(c, &c->f_wsn, NF);
    if (e == cudaSuccess) e = dalloc(c, &c->f_wst, NF);
    if (e == cudaSuccess) e = dalloc(c, &c->f_gamma_t, NF);
    if (e == cudaSuccess) e = dalloc(c, &c->f_air_p, NN);
    if (e == cudaSuccess) e = dalloc(c, &c->f_con_ob, (size_t)d.n_ob * 2 * nt);
    if (e == cudaSuccess) e = dalloc(c, &c->f_con_qb, (size_t)d.n_qb * 2 * nt);
    if (e == cudaSuccess) e = dalloc(c, &c->f_phi_sw, NC);
    if (e == cudaSuccess) e = dalloc(c, &c->f_phi_sz, L * NC);
    // [elapsed_time, spinup_tide, spinup_baroclinic, -, julian_day, it, -, -]
    if (e == cudaSuccess) e = dalloc(c, &c->f_scal, 8);
    if (e == cudaSuccess) {
        const double one[8] = {0.0, 1.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        e = cudaMemcpy(c->f_scal, one, sizeof(one), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = legacy_done();
    }
    Forcing &F = c->x.f;
    F.scal = c->f_scal;
    F.eta_at_ob_old = c->f_eta_old;
    F.eta_at_ob_new = c->f_eta_new;
    F.q_add = c->f_q_add;
    F.wind_stress_normal = c->f_wsn;
    F.wind_stress_tangnt = c->f_wst;
    F.gamma_t = c->f_gamma_t;
    F.air_p = c->f_air_p;
    F.con_at_ob = c->f_con_ob;
    F.con_at_qb = c->f_con_qb;
    F.phi_sw = c->f_phi_sw;
    F.phi_sz = c->f_phi_sz;
    // work
    Work &W = c->x.w;
    if (e == cudaSuccess) e = dalloc(c, &W.sparsem, 5 * NC);
    if (e == cudaSuccess) e = dalloc(c, &W.rhs, NC);
    if (e == cudaSuccess) e = dalloc(c, &W.minv, NC);
    if (e == cudaSuccess) e = dalloc(c, &W.r, NC);
    if (e == cudaSuccess) e = dalloc(c, &W.s, NC);
    if (e == cudaSuccess) e = dalloc(c, &W.q, NC);
    if (e == cudaSuccess) e = dalloc(c, &W.d0, NC);
    if (e == cudaSuccess) e = dalloc(c, &W.d1, NC);
    if (!c->mixed && d.n_runs <= 1) {
        if (e == cudaSuccess) e = dalloc(c, &W.cg_s1, NC);
        if (e == cudaSuccess) e = dalloc(c, &W.cg_w1, NC);
        if (e == cudaSuccess) e = dalloc(c, &W.cg_xs, NC);
    }
    // grid barrier (count, generation) or one pair per packed run
    if (e == cudaSuccess) e = dalloc(c, &W.barrier, 2 * (size_t)PCG_MAX_RUNS);
    if (e == cudaSuccess) e = dalloc(c, &W.pcg_iters, 1);
    if (e == cudaSuccess) e = dalloc(c, &W.run_block_start, (size_t)G.NR + 1);
    if (e == cudaSuccess) e = dalloc(c, &W.run_iters, (size_t)G.NR);
    if (e == cudaSuccess) e = c->mixed ? alloc_layered_work(c, c->xf.w) : alloc_layered_work(c, W);
    if (e == cudaSuccess) e = dalloc(c, &W.idev, L * NF);
    if (params->advection_flag != 0) {
        if (e == cudaSuccess) e = dalloc(c, &W.fl_list, L * NF);
        if (e == cudaSuccess) e = dalloc(c, &W.fl_off, NF);
        if (e == cudaSuccess) e = dalloc(c, &W.fl_bsum, NF / LIST_BLOCK + 2);
        if (e == cudaSuccess) e = dalloc(c, &W.fl_count, 2);
    }
    if (e == cudaSuccess) e = dalloc(c, &W.node_weight, NN);
    if (!c->mixed && L + 1 <= 64) {
        if (e == cudaSuccess) e = dalloc(c, &W.nl_list, (size_t)(L + 1) * NN);
        if (e == cudaSuccess) e = dalloc(c, &W.nl_off, NN);
        if (e == cudaSuccess) e = dalloc(c, &W.nl_bsum, NN / LIST_BLOCK + 2);
        if (e == cudaSuccess) e = dalloc(c, &W.nl_count, 2);
    }
    if (e == cudaSuccess) e = dalloc(c, &W.fs_sums, 3 * NF);
    if (e == cudaSuccess) e = dalloc(c, &W.cons, 2 + 2 * (size_t)((NC + 255) / 256));
    if (e == cudaSuccess) e = dalloc(c, &c->x.status, 1);
    if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? GOM_E_NOMEM : GOM_E_CUDA);
    // parameters
    Params &P = c->x.p;
    P.gravity = params->gravity;
    P.rho_o = params->rho_o;
    P.msl = params->msl;
    P.dt = params->dt;
    for (int n = 1; n <= GOM_BT_TABLE; ++n) P.bt_dt[n - 1] = params->dt / n;
    P.theta = params->theta;
    P.adv_onoff_depth = params->adv_onoff_depth;
    P.von_karman = params->von_karman;
    P.cd_const = params->cd_const;
    P.dry_depth = params->dry_depth;
    P.smagorinsky = params->smagorinsky;
    P.ah_0 = params->ah_0;
    P.kh_0 = params->kh_0;
    P.error_tolerance = params->error_tolerance;
    P.delta_z_min = params->delta_z_min;
    P.denominator_min_for_matrix = params->denominator_min_for_matrix;
    P.advection_flag = params->advection_flag;
    P.elm_backtrace_flag = params->elm_backtrace_flag;
    P.elm_sub_iter = params->elm_sub_iter;
    P.elm_min_iter = params->elm_min_iter;
    P.elm_max_iter = params->elm_max_iter;
    P.bf_flag = params->bf_flag;
    P.baroclinic_flag = params->baroclinic_flag;
    P.ana_density = params->ana_density;
    P.max_iteration_pcg = params->max_iteration_pcg;
    P.transport_flag = params->transport_flag;
    P.transport_solver = params->transport_solver;
    P.trans_sub_iter = params->trans_sub_iter;
    P.h_flux_limiter = params->h_flux_limiter;
    P.v_flux_limiter = params->v_flux_limiter;
    P.is_salt = params->is_salt;
    P.is_temp = params->is_temp;
    P.heat_option = params->heat_option;
    P.test_barrier_phantom_blocks = params->test_barrier_phantom_blocks;
    P.turbulence_flag = params->turbulence_flag;
    P.pp_h1 = params->pp_h1;
    P.pp_h2 = params->pp_h2;
    P.pp_vdmax1 = params->pp_vdmax1;
    P.pp_vdmax2 = params->pp_vdmax2;
    P.pp_vdmin1 = params->pp_vdmin1;
    P.pp_vdmin2 = params->pp_vdmin2;
    P.pp_tdmin = params->pp_tdmin;
    // pinned host staging
    c->stage_len = std::max<size_t>({NF, NN, NC, (size_t)d.n_ob * 2 * nt, (size_t)d.n_qb * 2 * nt}) * 10 + 64;
    if (cudaMallocHost((void **)&c->h_status, sizeof(gom_status)) != cudaSuccess ||
        cudaMallocHost((void **)&c->h_iters, sizeof(int)) != cudaSuccess ||
        cudaMallocHost((void **)&c->h_cons, 2 * sizeof(double)) != cudaSuccess ||
        cudaMallocHost((void **)&c->h_stage, 2 * c->stage_len * sizeof(double)) != cudaSuccess)
        return fail(GOM_E_NOMEM);
    for (int h = 0; h < 2; ++h)
        if (cudaEventCreateWithFlags(&c->stage_done[h], cudaEventDisableTiming) != cudaSuccess) return fail(GOM_E_CUDA);
    if (cudaEventCreateWithFlags(&c->ev_to_solver, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_from_solver, cudaEventDisableTiming) != cudaSuccess)
        return fail(GOM_E_CUDA);
    std::memset(c->h_status, 0, sizeof(gom_status));
    {
        cudaError_t pe = pcg_configure(c->x, c->device);
        if (pe == cudaErrorInvalidValue) {
            c->msg = "packed runs: more runs than the free-surface solver grid holds";
            return fail(GOM_E_ARG);
        }
        if (pe != cudaSuccess) return fail(GOM_E_CUDA);
    }
    if (launch_node_weights(c->x) != cudaSuccess) return fail(GOM_E_CUDA);
    {
        // two halves: the mixed solvers alternate them with every barrier
        size_t nb = 2 * (size_t)std::max(c->x.w.pcg_blocks, c->x.num_sms);
        if (dalloc(c, &W.partial_dq, nb) != cudaSuccess || dalloc(c, &W.partial_delta, nb) != cudaSuccess)
            return fail(GOM_E_NOMEM);
    }
    if (c->mixed) {
        float *el = nullptr;
        if (dalloc(c, &el, 8 * NC) != cudaSuccess) return fail(GOM_E_NOMEM);
        c->x.g.elem_local = el;
        if (launch_elem_local(c->x.g, el, c->x.stream) != cudaSuccess) return fail(GOM_E_CUDA);
        struct {
            const double *src;
            const float **dst;
            long n;
        } f32[] = {{c->x.g.area, &c->x.g.area_f, NC},
                   {c->x.g.face_length, &c->x.g.face_length_f, NF},
                   {c->x.g.delta_j, &c->x.g.delta_j_f, NF},
                   {c->x.g.cos_theta, &c->x.g.cos_theta_f, NF},
                   {c->x.g.sin_theta, &c->x.g.sin_theta_f, NF},
                   {W.node_weight, &c->x.g.node_weight_f, NN},
                   {c->x.g.z_level, &c->x.g.z_level_f, (long)c->x.g.L + 1}};
        for (auto &cv : f32) {
            float *d = nullptr;
            if (dalloc(c, &d, (size_t)cv.n) != cudaSuccess) return fail(GOM_E_NOMEM);
            if (launch_to_float(cv.src, d, cv.n, c->x.stream) != cudaSuccess) return fail(GOM_E_CUDA);
            *cv.dst = d;
        }
        float *el2 = nullptr;
        if (dalloc(c, &el2, NF) != cudaSuccess) return fail(GOM_E_NOMEM);
        if (launch_edge_len2(c->x.g, el2, c->x.stream) != cudaSuccess) return fail(GOM_E_CUDA);
        c->x.g.edge_len2_f = el2;
        // the FP32 context shares geometry, forcing, parameters, status, stream and the FP64
        // work arrays (free-surface system, PCG vectors, ELM counts, node weights, sums)
        LaunchT<float> &X = c->xf;
        X.g = c->x.g;
        X.f = c->x.f;
        X.p = c->x.p;
        X.status = c->x.status;
        X.stream = c->x.stream;
        X.num_sms = c->x.num_sms;
        X.w.sparsem = W.sparsem;
        X.w.rhs = W.rhs;
        X.w.minv = W.minv;
        X.w.r = W.r;
        X.w.s = W.s;
        X.w.q = W.q;
        X.w.d0 = W.d0;
        X.w.d1 = W.d1;
        X.w.partial_dq = W.partial_dq;
        X.w.partial_delta = W.partial_delta;
        X.w.barrier = W.barrier;
        X.w.pcg_iters = W.pcg_iters;
        X.w.pcg_blocks = W.pcg_blocks;
        X.w.pcg_threads = W.pcg_threads;
        X.w.run_block_start = W.run_block_start;
        X.w.run_iters = W.run_iters;
        X.w.idev = W.idev;
        X.w.fl_list = W.fl_list;
        X.w.fl_off = W.fl_off;
        X.w.fl_bsum = W.fl_bsum;
        X.w.fl_count = W.fl_count;
        X.w.node_weight = W.node_weight;
        X.w.fs_sums = W.fs_sums;
        X.w.cons = W.cons;
        // FP32 copy of the free-surface system for the FP32 inner PCG iterations
        if (dalloc(c, &X.w.sp32, 5 * NC) != cudaSuccess) return fail(GOM_E_NOMEM);
    }
    if (cudaDeviceSynchronize() != cudaSuccess) return fail(GOM_E_CUDA);
    *out = c;
    return GOM_OK;
}

void gom_destroy(gom_ctx *c) {
    if (!c) return;
    if (c->x.stream) cudaStreamSynchronize(c->x.stream);
    drop_graphs(c);
    if (c->ev_to_solver) cudaEventDestroy(c->ev_to_solver);
    if (c->ev_from_solver) cudaEventDestroy(c->ev_from_solver);
    for (void *p : c->allocs) cudaFree(p);
    for (void *p : c->series_allocs) cudaFree(p);
    if (c->h_status) cudaFreeHost(c->h_status);
    if (c->h_iters) cudaFreeHost(c->h_iters);
    if (c->h_cons) cudaFreeHost(c->h_cons);
    if (c->h_stage) cudaFreeHost(c->h_stage);
    for (int h = 0; h < 2; ++h)
        if (c->stage_done[h]) cudaEventDestroy(c->stage_done[h]);
    if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
    if (c->snap_dev) cudaFree(c->snap_dev);
    if (c->ev_snap_staged) cudaEventDestroy(c->ev_snap_staged);
    if (c->ev_snap_done) cudaEventDestroy(c->ev_snap_done);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->st_ids) cudaFree(c->st_ids);
    if (c->st_out) cudaFree(c->st_out);
    if (c->x.stream) cudaStreamDestroy(c->x.stream);
    delete c;
}

int gom_snapshot_begin(gom_ctx *c, int32_t n_fields, const int32_t *fields, void *const *host) {
    if (!c || n_fields < 0 || (n_fields > 0 && (!fields || !host)) || c->snap_pending) return GOM_E_ARG;
    size_t total = 0;
    for (int q = 0; q < n_fields; ++q) {
        if (fields[q] <= 0 || fields[q] >= GOM_F_COUNT || !host[q]) return GOM_E_ARG;
        const FieldDesc &f = c->fields[fields[q]];
        if (f.lo == -2) return GOM_E_ARG;
        total += (size_t)field_count(c->d, f) * (f.is_int ? 4 : 8);
    }
    if (!c->copy_stream) {
        CK(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&c->ev_snap_staged, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&c->ev_snap_done, cudaEventDisableTiming));
    }
    if (total > c->snap_cap) {
        // no snapshot is in flight, so the old area is free once the context stream has passed it
        CK(cudaStreamSynchronize(c->x.stream));
        if (c->snap_dev) {
            cudaFree(c->snap_dev);
            c->bytes -= c->snap_cap;
        }
        c->snap_dev = nullptr;
        c->snap_cap = 0;
        if (cudaMalloc(&c->snap_dev, total) != cudaSuccess) return GOM_E_NOMEM;
        c->snap_cap = total;
        c->bytes += total;
    }
    // stage on the context stream, after the work enqueued so far (FP32 fields widened to FP64)
    size_t off = 0;
    for (int q = 0; q < n_fields; ++q) {
        const FieldDesc &f = c->fields[fields[q]];
        const long n = (long)field_count(c->d, f);
        const size_t nb = (size_t)n * (f.is_int ? 4 : 8);
        if (!f.is_int && f.dev_bytes == 4)
            CK(launch_to_double((const float *)*f.dev, (double *)(c->snap_dev + off), n, c->x.stream));
        else
            CK(cudaMemcpyAsync(c->snap_dev + off, *f.dev, nb, cudaMemcpyDeviceToDevice, c->x.stream));
        off += nb;
    }
    CK(cudaEventRecord(c->ev_snap_staged, c->x.stream));
    // transfer on the copy stream while later steps run on the context stream
    CK(cudaStreamWaitEvent(c->copy_stream, c->ev_snap_staged, 0));
    off = 0;
    for (int q = 0; q < n_fields; ++q) {
        const FieldDesc &f = c->fields[fields[q]];
        const size_t nb = (size_t)field_count(c->d, f) * (f.is_int ? 4 : 8);
        CK(cudaMemcpyAsync(host[q], c->snap_dev + off, nb, cudaMemcpyDeviceToHost, c->copy_stream));
        off += nb;
    }
    CK(cudaEventRecord(c->ev_snap_done, c->copy_stream));
    c->snap_pending = true;
    return GOM_OK;
}

int gom_snapshot_ready(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    if (!c->snap_pending) return 1;
    cudaError_t e = cudaEventQuery(c->ev_snap_done);
    if (e == cudaErrorNotReady) return 0;
    CK(e);
    return 1;
}

int gom_snapshot_wait(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    if (!c->snap_pending) return GOM_OK;
    c->snap_pending = false;
    CK(cudaEventSynchronize(c->ev_snap_done));
    return GOM_OK;
}

int gom_host_alloc(int64_t bytes, void **out) {
    if (!out || bytes <= 0) return GOM_E_ARG;
    *out = nullptr;
    if (cudaHostAlloc(out, (size_t)bytes, cudaHostAllocDefault) != cudaSuccess) return GOM_E_NOMEM;
    return GOM_OK;
}

void gom_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

int gom_set_field(gom_ctx *c, int field, const void *host, int64_t count) {
    if (!c || !host || field <= 0 || field >= GOM_F_COUNT) return GOM_E_ARG;
    const FieldDesc &f = c->fields[field];
    if (f.lo == -2 || count != field_count(c->d, f)) return GOM_E_ARG;
    if (!f.is_int && f.dev_bytes == 4) {
        // FP32 storage: round the FP64 host array to nearest
        std::vector<float> tmp((size_t)count);
        const double *h = (const double *)host;
        for (int64_t k = 0; k < count; ++k) tmp[k] = (float)h[k];
        CK(cudaMemcpyAsync(*f.dev, tmp.data(), (size_t)count * 4, cudaMemcpyHostToDevice, c->x.stream));
        CK(cudaStreamSynchronize(c->x.stream));
        return GOM_OK;
    }
    CK(cudaMemcpyAsync(*f.dev, host, (size_t)count * (f.is_int ? 4 : 8), cudaMemcpyHostToDevice, c->x.stream));
    CK(cudaStreamSynchronize(c->x.stream));
    return GOM_OK;
}

int gom_get_field(gom_ctx *c, int field, void *host, int64_t count) {
    if (!c || !host || field <= 0 || field >= GOM_F_COUNT) return GOM_E_ARG;
    const FieldDesc &f = c->fields[field];
    if (f.lo == -2 || count != field_count(c->d, f)) return GOM_E_ARG;
    if (!f.is_int && f.dev_bytes == 4) {
        std::vector<float> tmp((size_t)count);
        CK(cudaMemcpyAsync(tmp.data(), *f.dev, (size_t)count * 4, cudaMemcpyDeviceToHost, c->x.stream));
        CK(cudaStreamSynchronize(c->x.stream));
        double *h = (double *)host;
        for (int64_t k = 0; k < count; ++k) h[k] = (double)tmp[k];
        return GOM_OK;
    }
    CK(cudaMemcpyAsync(host, *f.dev, (size_t)count * (f.is_int ? 4 : 8), cudaMemcpyDeviceToHost, c->x.stream));
    CK(cudaStreamSynchronize(c->x.stream));
    return GOM_OK;
}

int gom_set_forcing(gom_ctx *c, const gom_forcing *fo) {
    if (!c || !fo) return GOM_E_ARG;
    const gom_dims &d = c->d;
    const double scal[4] = {fo->elapsed_time, fo->spinup_tide, fo->spinup_baroclinic, 0.0};
    int nt = c->hp.trans_sub_iter > 0 ? c->hp.trans_sub_iter : 1;
    struct Item {
        const double *src;
        double *dst;
        size_t n;
    } items[] = {{scal, c->f_scal, 4},
                 {fo->eta_at_ob_old, c->f_eta_old, (size_t)d.n_ob},
                 {fo->eta_at_ob_new, c->f_eta_new, (size_t)d.n_ob},
                 {fo->q_add, c->f_q_add, (size_t)d.n_qb},
                 {fo->wind_stress_normal, c->f_wsn, (size_t)d.n_faces},
                 {fo->wind_stress_tangnt, c->f_wst, (size_t)d.n_faces},
                 {fo->gamma_t, c->f_gamma_t, (size_t)d.n_faces},
                 {fo->air_p, c->f_air_p, (size_t)d.n_nodes},
                 {fo->con_at_ob, c->f_con_ob, (size_t)d.n_ob * 2 * nt},
                 {fo->con_at_qb, c->f_con_qb, (size_t)d.n_qb * 2 * nt},
                 {fo->phi_sw, c->f_phi_sw, (size_t)d.n_cells},
                 {fo->phi_sz, c->f_phi_sz, (size_t)d.n_cells * d.n_layers}};
    // alternate between the two staging halves; wait only until the upload that last used this
    // half has left it (so one step can be in flight while the next step's forcing is staged)
    int h = c->stage_half;
    c->stage_half ^= 1;
    double *stage = c->h_stage + (size_t)h * c->stage_len;
    CK(cudaEventSynchronize(c->stage_done[h]));
    size_t off = 0;
    for (auto &it : items) {
        if (!it.src || it.n == 0) continue;
        if (off + it.n > c->stage_len) {
            // larger than the staging half: copied straight from the caller's buffer (synchronous)
            CK(cudaMemcpyAsync(it.dst, it.src, it.n * 8, cudaMemcpyHostToDevice, c->x.stream));
            CK(cudaStreamSynchronize(c->x.stream));
            continue;
        }
        std::memcpy(stage + off, it.src, it.n * 8);
        CK(cudaMemcpyAsync(it.dst, stage + off, it.n * 8, cudaMemcpyHostToDevice, c->x.stream));
        off += it.n;
    }
    CK(cudaEventRecord(c->stage_done[h], c->x.stream));
    return GOM_OK;
}

int gom_get_status(gom_ctx *c, gom_status *s, int clear) {
    if (!c || !s) return GOM_E_ARG;
    CK(cudaMemcpyAsync(c->h_status, c->x.status, sizeof(gom_status), cudaMemcpyDeviceToHost, c->x.stream));
    CK(cudaStreamSynchronize(c->x.stream));
    *s = *c->h_status;
    s->run = status_run(c, *s);
    if (clear) {
        CK(cudaMemsetAsync(c->x.status, 0, sizeof(gom_status), c->x.stream));
        CK(cudaStreamSynchronize(c->x.stream));
        std::memset(c->h_status, 0, sizeof(gom_status));
    }
    return GOM_OK;
}

int gom_synchronize(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    CK(cudaStreamSynchronize(c->x.stream));
    return GOM_OK;
}

int64_t gom_pcg_iterations_total(gom_ctx *c) { return c ? c->pcg_total : 0; }

int64_t gom_device_bytes(const gom_ctx *c) { return c ? (int64_t)c->bytes : 0; }

void *gom_stream(gom_ctx *c) { return c ? (void *)c->x.stream : nullptr; }

int gom_step_bottom_friction(gom_ctx *c) { return run_phase(c, GOM_PHASE(launch_bottom_friction)); }
int gom_step_boundary_velocity(gom_ctx *c) { return run_phase(c, GOM_PHASE(launch_boundary_velocity)); }
int gom_step_advection(gom_ctx *c) { return run_phase(c, GOM_PHASE(launch_advection)); }
int gom_step_momentum(gom_ctx *c) { return run_phase(c, GOM_PHASE(launch_momentum)); }
int gom_step_velocities(gom_ctx *c) { return run_phase(c, GOM_PHASE(launch_velocities)); }
int gom_step_layers(gom_ctx *c) { return run_phase(c, GOM_PHASE(launch_layers)); }
int gom_step_node_velocity(gom_ctx *c) { return run_phase(c, GOM_PHASE(launch_node_velocity)); }
int gom_step_transport(gom_ctx *c) { return run_phase(c, GOM_PHASE(launch_transport)); }
int gom_step_density(gom_ctx *c) { return run_phase(c, GOM_PHASE(launch_density)); }
int gom_step_turbulence(gom_ctx *c) { return run_phase(c, GOM_PHASE(launch_turbulence)); }

int gom_step_free_surface(gom_ctx *c, int32_t *pcg_iters) {
    if (!c) return GOM_E_ARG;
    CK(c->mixed ? launch_free_surface(c->xf) : launch_free_surface(c->x));
    return finish(c, pcg_iters, true);
}

int gom_step_swap(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    CK(enqueue_swap(c));
    return finish(c, nullptr, false);
}

int gom_step_launch(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    // The timestep is captured once into CUDA graphs and replayed: every kernel argument is a
    // device pointer or a constant of the context, and per-step forcing lives in device memory.
    if (!c->graph && !c->graph_failed) {
        cudaError_t e = capture(c, 0, &c->graph);
        if (e == cudaSuccess) e = capture(c, 1, &c->graph_fs);
        if (e == cudaSuccess) e = capture(c, 2, &c->graph_post);
        if (e != cudaSuccess) {
            cudaGetLastError();
            drop_graphs(c);
            c->graph_failed = true;
            c->msg = std::string("graph capture unavailable: ") + cudaGetErrorString(e);
        }
    }
    cudaStream_t solver = nullptr;
    CK(solver_stream(c->device, &solver));
    if (c->graph) {
        CK(cudaGraphLaunch(c->graph, c->x.stream));
        CK(cudaEventRecord(c->ev_to_solver, c->x.stream));
        CK(cudaStreamWaitEvent(solver, c->ev_to_solver, 0));
        CK(cudaGraphLaunch(c->graph_fs, solver));
        CK(cudaEventRecord(c->ev_from_solver, solver));
        CK(cudaStreamWaitEvent(c->x.stream, c->ev_from_solver, 0));
        CK(cudaGraphLaunch(c->graph_post, c->x.stream));
    } else {
        CK(enqueue_step(c));
    }
    CK(cudaMemcpyAsync(c->h_status, c->x.status, sizeof(gom_status), cudaMemcpyDeviceToHost, c->x.stream));
    CK(cudaMemcpyAsync(c->h_iters, c->x.w.pcg_iters, sizeof(int), cudaMemcpyDeviceToHost, c->x.stream));
    c->step_pending = true;
    return GOM_OK;
}

int gom_step_wait(gom_ctx *c, int32_t *pcg_iters) {
    if (!c) return GOM_E_ARG;
    CK(cudaStreamSynchronize(c->x.stream));
    if (c->step_pending) {
        c->step_pending = false;
        c->pcg_total += *c->h_iters;
        if (pcg_iters) *pcg_iters = *c->h_iters;
    }
    return c->h_status->code;
}

int gom_step_all(gom_ctx *c, int32_t *pcg_iters) {
    int rc = gom_step_launch(c);
    if (rc != GOM_OK) return rc;
    return gom_step_wait(c, pcg_iters);
}

int gom_cold_start(gom_ctx *c, double salt, double temp, double av_0, double kv_0) {
    if (!c) return GOM_E_ARG;
    // every state field starts at zero (setup_cold_start.f90)
    for (int f = 1; f < GOM_F_COUNT; ++f) {
        const FieldDesc &fd = c->fields[f];
        if (fd.lo == -2 || is_forcing_field(f)) continue;
        CK(cudaMemsetAsync(*fd.dev, 0, (size_t)field_count(c->d, fd) * fd.dev_bytes, c->x.stream));
    }
    CK(cudaMemsetAsync(c->x.status, 0, sizeof(gom_status), c->x.stream));
    CK(c->mixed ? launch_cold_start(c->xf, salt, temp, av_0, kv_0) : launch_cold_start(c->x, salt, temp, av_0, kv_0));
    return finish(c, nullptr, false);
}

int gom_profile_kernel(gom_ctx *c, int32_t which, int32_t reps, double *ms_per_launch) {
    if (!c || reps < 1 || !ms_per_launch) return GOM_E_ARG;
    cudaError_t (*run)(gom_ctx *) = nullptr;
    switch (which) {
    case GOM_KERNEL_ELM_WALK: run = GOM_PHASE(launch_elm_walk_only); break;
    case GOM_KERNEL_MOMENTUM: run = GOM_PHASE(launch_momentum_columns_only); break;
    case GOM_KERNEL_TRANSPORT_SOLVE:
        // the TVD solve exists only when the context runs the TVD transport
        if (!c->hp.transport_flag || c->hp.transport_solver == 2) return GOM_E_ARG;
        CK(c->mixed ? launch_transport(c->xf) : launch_transport(c->x));   // coefficients and limiter
        run = GOM_PHASE(launch_tr_solve_only);
        break;
    default: return GOM_E_ARG;
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    cudaError_t e = run(c);
    if (e == cudaSuccess) e = cudaEventRecord(e0, c->x.stream);
    for (int r = 0; r < reps && e == cudaSuccess; ++r) e = run(c);
    if (e == cudaSuccess) e = cudaEventRecord(e1, c->x.stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CK(e);
    *ms_per_launch = (double)ms / reps;
    return finish(c, nullptr, false);
}

int gom_autotune(gom_ctx *c, int32_t reps, int32_t *choice) {
    if (!c || reps < 1) return GOM_E_ARG;
    struct Site {
        int site;
        cudaError_t (*run)(gom_ctx *);
    };
    const Site sites[] = {{TUNE_ELM, GOM_PHASE(launch_advection)},
                          {TUNE_MOMENTUM, GOM_PHASE(launch_momentum)},
                          {TUNE_TR_SOLVE, GOM_PHASE(launch_transport)},
                          {TUNE_TR_LIMITER, GOM_PHASE(launch_transport)}};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    int rc = GOM_OK;
    for (const Site &st : sites) {
        int best = 0;
        float best_ms = 1e30f;
        for (int v = 0; v < TUNE_VARIANTS[st.site] && rc == GOM_OK; ++v) {
            c->x.tune[st.site] = v;
            c->xf.tune[st.site] = v;
            cudaError_t e = st.run(c);                        // warm-up (and first-touch)
            if (e == cudaSuccess) e = cudaEventRecord(e0, c->x.stream);
            for (int r = 0; r < reps && e == cudaSuccess; ++r) e = st.run(c);
            if (e == cudaSuccess) e = cudaEventRecord(e1, c->x.stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float ms = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            if (e != cudaSuccess) {
                rc = set_cuda_error(c, e, "autotune");
                break;
            }
            if (ms < best_ms) {
                best_ms = ms;
                best = v;
            }
        }
        c->x.tune[st.site] = best;
        c->xf.tune[st.site] = best;
        if (choice) choice[st.site] = best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != GOM_OK) return rc;
    drop_graphs(c);   // captured again with the chosen variants
    return finish(c, nullptr, false);
}

int gom_tuning_variants(int32_t counts[GOM_TUNE_SITES]) {
    if (!counts) return GOM_E_ARG;
    for (int k = 0; k < GOM_TUNE_SITES; ++k) counts[k] = TUNE_VARIANTS[k];
    return GOM_OK;
}

int gom_set_tuning(gom_ctx *c, const int32_t choice[GOM_TUNE_SITES]) {
    if (!c || !choice) return GOM_E_ARG;
    for (int k = 0; k < GOM_TUNE_SITES; ++k)
        if (choice[k] < -1 || choice[k] >= TUNE_VARIANTS[k]) return GOM_E_ARG;
    for (int k = 0; k < GOM_TUNE_SITES; ++k)
        if (choice[k] >= 0) {
            c->x.tune[k] = choice[k];
            c->xf.tune[k] = choice[k];
        }
    drop_graphs(c);
    return GOM_OK;
}

int gom_copy_run(gom_ctx *dst, int32_t dst_run, gom_ctx *src, int32_t src_run) {
    gom_ctx *c = dst;
    if (!dst || !src || dst->d.n_layers != src->d.n_layers || dst->mixed != src->mixed || dst->device != src->device)
        return GOM_E_ARG;
    if (dst_run < 0 || dst_run >= dst->x.g.NR || src_run < 0 || src_run >= src->x.g.NR) return GOM_E_ARG;
    // the runs' entity ranges, from the host copies of the run tables
    auto range = [](gom_ctx *k, int run, int kind, int64_t &b, int64_t &n) {
        const gom_dims &d = k->d;
        if (k->x.g.NR <= 1) {
            b = 0;
            n = kind == 0 ? d.n_cells : kind == 1 ? d.n_faces : kind == 2 ? d.n_nodes : kind == 3 ? d.n_qb : d.n_ob;
            return;
        }
        const std::vector<int> &s = k->run_starts[kind == 0 ? 0 : kind == 1 ? 1 : kind == 2 ? 2 : 3];
        b = s[run];
        n = s[run + 1] - s[run];
    };
    CK(cudaStreamSynchronize(src->x.stream));
    for (int f = 1; f < GOM_F_COUNT; ++f) {
        const FieldDesc &fd = dst->fields[f];
        if (fd.lo == -2 || is_forcing_field(f)) continue;
        if (fd.kind == 3) {
            if (dst->d.n_qb == 0 && src->d.n_qb == 0) continue;
            return GOM_E_ARG;   // river cells are not split into runs
        }
        int64_t db, dn, sb, sn;
        range(dst, dst_run, fd.kind, db, dn);
        range(src, src_run, fd.kind, sb, sn);
        if (dn != sn) return GOM_E_ARG;
        const int64_t per = fd.lo < 0 ? 1 : (int64_t)(dst->d.n_layers - fd.lo + 1);
        const size_t eb = (size_t)fd.dev_bytes;
        char *dp = (char *)*fd.dev + (size_t)(db * per) * eb;
        const char *sp = (const char *)*src->fields[f].dev + (size_t)(sb * per) * eb;
        CK(cudaMemcpyAsync(dp, sp, (size_t)(dn * per) * eb, cudaMemcpyDeviceToDevice, dst->x.stream));
    }
    CK(cudaStreamSynchronize(dst->x.stream));
    return GOM_OK;
}

int gom_set_storms(gom_ctx *c, int32_t n_storms, const gom_storm *storms, double elapsed_time) {
    if (!c || !storms || n_storms != c->x.g.NR || c->has_series) return GOM_E_ARG;
    static_assert(sizeof(gom_storm) == 13 * sizeof(double), "gom_storm is 13 doubles");
    for (int r = 0; r < n_storms; ++r) {
        const gom_storm &s = storms[r];
        if (!(s.rmax > 0.0) || !(s.dp >= 0.0) || !(s.b > 0.0) || !(s.tide_period > 0.0) || s.coriolis == 0.0)
            return GOM_E_ARG;
    }
    CK(cudaStreamSynchronize(c->x.stream));
    if (!c->d_storms) {
        CK(dalloc(c, &c->d_storms, (size_t)13 * n_storms));
        CK(dalloc(c, &c->storm_wu, (size_t)c->d.n_nodes));
        CK(dalloc(c, &c->storm_wv, (size_t)c->d.n_nodes));
    }
    CK(cudaMemcpy(c->d_storms, storms, sizeof(gom_storm) * n_storms, cudaMemcpyHostToDevice));
    CK(legacy_done());
    const double scal0[1] = {elapsed_time};
    CK(cudaMemcpy(c->f_scal, scal0, sizeof(double), cudaMemcpyHostToDevice));
    CK(legacy_done());
    c->n_storms = n_storms;
    // the captured step gains the forcing kernels: capture again on the next launch
    drop_graphs(c);
    return GOM_OK;
}

}  // extern "C"

namespace {

template <typename T> cudaError_t series_upload(gom_ctx *c, const T **dst, const T *src, size_t n) {
    T *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)&p, n * sizeof(T));
    if (e != cudaSuccess) return e;
    c->series_allocs.push_back(p);
    c->series_bytes += n * sizeof(T);
    e = src ? cudaMemcpy(p, src, n * sizeof(T), cudaMemcpyHostToDevice) : cudaMemset(p, 0, n * sizeof(T));
    if (e == cudaSuccess) e = legacy_done();
    *dst = p;
    return e;
}

void series_free(gom_ctx *c) {
    for (void *p : c->series_allocs) cudaFree(p);
    c->series_allocs.clear();
    c->bytes -= c->series_bytes;
    c->series_bytes = 0;
    c->has_series = false;
}

// a series set is usable: offsets start at 0 and grow, times never decrease within a series
bool series_ok(const gom_series &s) {
    if (s.n_series < 0) return false;
    if (s.n_series == 0) return true;
    if (!s.start || !s.time || !s.value || s.start[0] != 0) return false;
    for (int k = 0; k < s.n_series; ++k) {
        if (s.start[k + 1] < s.start[k]) return false;
        for (int q = s.start[k] + 1; q < s.start[k + 1]; ++q)
            if (!(s.time[q] >= s.time[q - 1])) return false;
    }
    return true;
}

bool ids_ok(const int32_t *ids, int n, int n_series) {
    if (n > 0 && !ids) return false;
    for (int i = 0; i < n; ++i)
        if (ids[i] < 0 || ids[i] > n_series) return false;
    return true;
}

}  // namespace

extern "C" {

int gom_set_boundary_series(gom_ctx *c, const gom_boundary_series *bs) {
    if (!c || !bs || c->n_storms > 0 || c->d.n_runs > 1) return GOM_E_ARG;
    const int nob = c->d.n_ob, nqb = c->d.n_qb;
    const gom_series *sets[4] = {&bs->eta, &bs->q, &bs->salt, &bs->temp};
    for (const gom_series *sr : sets)
        if (!series_ok(*sr)) return GOM_E_ARG;
    if (bs->n_harmonic < 0 || (bs->n_harmonic > 0 && (!bs->harmonic_start || !bs->amplitude || !bs->period_h ||
                                                       !bs->nodal || !bs->eq_arg || !bs->phase || !bs->phase_shift)))
        return GOM_E_ARG;
    if (bs->n_harmonic > 0 && bs->harmonic_start[0] != 0) return GOM_E_ARG;
    for (int k = 0; k < bs->n_harmonic; ++k)
        if (bs->harmonic_start[k + 1] < bs->harmonic_start[k]) return GOM_E_ARG;
    if (nob > 0 && !bs->ob_eta_type) return GOM_E_ARG;
    for (int i = 0; i < nob; ++i)
        if (bs->ob_eta_type[i] < -1 || bs->ob_eta_type[i] > 3) return GOM_E_ARG;   // read_main_inp.f90:460-464
    if (!ids_ok(bs->ob_harmonic_id, nob, bs->n_harmonic) || !ids_ok(bs->ob_eta_id, nob, bs->eta.n_series) ||
        !ids_ok(bs->ob_salt_id, nob, bs->salt.n_series) || !ids_ok(bs->ob_temp_id, nob, bs->temp.n_series) ||
        !ids_ok(bs->qb_q_id, nqb, bs->q.n_series) || !ids_ok(bs->qb_salt_id, nqb, bs->salt.n_series) ||
        !ids_ok(bs->qb_temp_id, nqb, bs->temp.n_series) || (nqb > 0 && !bs->qb_portion))
        return GOM_E_ARG;
    if (bs->q_interp_method != 1 && bs->q_interp_method != 2) return GOM_E_ARG;
    // station wind: one to three stations, each with u and v series, nodes inside the mesh
    if (bs->wind_flag != 0 && bs->wind_flag != 1) return GOM_E_ARG;
    if (bs->wind_flag == 1) {
        if (bs->wind_formular < 1 || bs->wind_formular > 3 || bs->n_wind < 1 || bs->n_wind > 3 ||
            bs->wind_u.n_series != bs->n_wind || bs->wind_v.n_series != bs->n_wind || !series_ok(bs->wind_u) ||
            !series_ok(bs->wind_v) || !(bs->rho_a > 0.0))
            return GOM_E_ARG;
        if (bs->n_wind > 1) {
            if (!bs->wind_station_node) return GOM_E_ARG;
            for (int k = 0; k < bs->n_wind; ++k)
                if (bs->wind_station_node[k] < 1 || bs->wind_station_node[k] > c->d.n_nodes) return GOM_E_ARG;
        }
    }
    // hurricane node frames: a read interval of at least one step, the three frames, air density
    if (bs->hurricane_flag != 0 && bs->hurricane_flag != 1) return GOM_E_ARG;
    if (bs->hurricane_flag == 1 && (bs->hurricane_read_interval < 1 || !bs->hurricane_frames || !(bs->rho_a > 0.0) ||
                                    bs->hurricane_interp_method < 0 || bs->hurricane_interp_method > 2))
        return GOM_E_ARG;
    // method 2 builds find_neighbour_nodes' lists by brute force over node pairs (as the
    // reference does): bounded to meshes the reference itself can hold
    const bool hur2 = bs->hurricane_flag == 1 && bs->hurricane_interp_method == 2;
    if (hur2 && c->d.n_nodes > (1 << 19)) return GOM_E_ARG;
    // heat balance: heat_term_by_term runs for temperature transport with heat_option 1; the
    // short-wave radiation from the air series (sol_swr 2); the series' times non-decreasing
    if (bs->heat_flag != 0 && bs->heat_flag != 1) return GOM_E_ARG;
    if (bs->heat_flag == 1) {
        if (!c->hp.transport_flag || !c->hp.is_temp || c->hp.heat_option != 1 || (bs->sol_swr != 1 && bs->sol_swr != 2) ||
            bs->n_air < 0 || (bs->sol_swr == 1 && (bs->month < 1 || bs->month > 12)) ||
            (bs->n_air > 0 && (!bs->air_time || !bs->air_values)))
            return GOM_E_ARG;
        for (int t = 1; t < bs->n_air; ++t)
            if (!(bs->air_time[t] >= bs->air_time[t - 1])) return GOM_E_ARG;
    }
    CK(cudaStreamSynchronize(c->x.stream));
    series_free(c);
    SeriesDev &S = c->series;
    S = SeriesDev{};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 4 && e == cudaSuccess; ++k) {
        const gom_series &sr = *sets[k];
        S.n[k] = sr.n_series;
        const size_t len = sr.n_series > 0 ? (size_t)sr.start[sr.n_series] : 0;
        e = series_upload(c, &S.start[k], sr.n_series > 0 ? sr.start : nullptr, (size_t)sr.n_series + 1);
        if (e == cudaSuccess) e = series_upload(c, &S.time[k], sr.n_series > 0 ? sr.time : nullptr, len);
        if (e == cudaSuccess) e = series_upload(c, &S.value[k], sr.n_series > 0 ? sr.value : nullptr, len);
    }
    if (e == cudaSuccess) e = series_upload(c, &S.ob_type, bs->ob_eta_type, (size_t)nob);
    if (e == cudaSuccess) e = series_upload(c, &S.ob_h, bs->ob_harmonic_id, (size_t)nob);
    if (e == cudaSuccess) e = series_upload(c, &S.ob_eta, bs->ob_eta_id, (size_t)nob);
    if (e == cudaSuccess) e = series_upload(c, &S.ob_salt, bs->ob_salt_id, (size_t)nob);
    if (e == cudaSuccess) e = series_upload(c, &S.ob_temp, bs->ob_temp_id, (size_t)nob);
    if (e == cudaSuccess) e = series_upload(c, &S.qb_q, bs->qb_q_id, (size_t)nqb);
    if (e == cudaSuccess) e = series_upload(c, &S.qb_salt, bs->qb_salt_id, (size_t)nqb);
    if (e == cudaSuccess) e = series_upload(c, &S.qb_temp, bs->qb_temp_id, (size_t)nqb);
    if (e == cudaSuccess) e = series_upload(c, &S.qb_portion, bs->qb_portion, (size_t)nqb);
    const int nh = bs->n_harmonic;
    const size_t nc = nh > 0 ? (size_t)bs->harmonic_start[nh] : 0;
    S.n_harm = nh;
    if (e == cudaSuccess) e = series_upload(c, &S.h_start, nh > 0 ? bs->harmonic_start : nullptr, (size_t)nh + 1);
    if (e == cudaSuccess) e = series_upload(c, &S.amp, nh > 0 ? bs->amplitude : nullptr, nc);
    if (e == cudaSuccess) e = series_upload(c, &S.per_h, nh > 0 ? bs->period_h : nullptr, nc);
    if (e == cudaSuccess) e = series_upload(c, &S.nodal, nh > 0 ? bs->nodal : nullptr, nc);
    if (e == cudaSuccess) e = series_upload(c, &S.eq, nh > 0 ? bs->eq_arg : nullptr, nc);
    if (e == cudaSuccess) e = series_upload(c, &S.ph, nh > 0 ? bs->phase : nullptr, nc);
    if (e == cudaSuccess) e = series_upload(c, &S.shift, nh > 0 ? bs->phase_shift : nullptr, (size_t)nh);
    const gom_series *wsets[2] = {&bs->wind_u, &bs->wind_v};
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
        const gom_series &sr = *wsets[k];
        const int ns = bs->wind_flag == 1 ? sr.n_series : 0;
        S.n[4 + k] = ns;
        const size_t len = ns > 0 ? (size_t)sr.start[ns] : 0;
        e = series_upload(c, &S.start[4 + k], ns > 0 ? sr.start : nullptr, (size_t)ns + 1);
        if (e == cudaSuccess) e = series_upload(c, &S.time[4 + k], ns > 0 ? sr.time : nullptr, len);
        if (e == cudaSuccess) e = series_upload(c, &S.value[4 + k], ns > 0 ? sr.value : nullptr, len);
    }
    const int nw = bs->wind_flag == 1 ? bs->n_wind : 0;
    if (e == cudaSuccess) e = series_upload(c, &S.wind_node, nw > 1 ? bs->wind_station_node : nullptr, (size_t)nw);
    if (e == cudaSuccess) {
        const double *ws = nullptr;
        e = series_upload(c, &ws, (const double *)nullptr, 6);
        S.wind_at_station = const_cast<double *>(ws);
    }
    const bool hur = bs->hurricane_flag == 1;
    const size_t nn = (size_t)c->d.n_nodes, nf = (size_t)c->d.n_faces;
    if (e == cudaSuccess && hur) {
        const double *fr = nullptr, *nx = nullptr, *fu = nullptr, *fv = nullptr;
        const int *rd = nullptr;
        e = series_upload(c, &fr, bs->hurricane_frames, 9 * nn);
        if (e == cudaSuccess) e = series_upload(c, &nx, (const double *)nullptr, 3 * nn);
        if (e == cudaSuccess) e = series_upload(c, &rd, (const int *)nullptr, 1);
        if (e == cudaSuccess) e = series_upload(c, &fu, (const double *)nullptr, nf);
        if (e == cudaSuccess) e = series_upload(c, &fv, (const double *)nullptr, nf);
        S.hur_frames = const_cast<double *>(fr);
        S.hur_next = const_cast<double *>(nx);
        S.hur_ready = const_cast<int *>(rd);
        S.face_u = const_cast<double *>(fu);
        S.face_v = const_cast<double *>(fv);
    }
    if (e == cudaSuccess && bs->heat_flag == 1) {
        const double *at = nullptr, *av = nullptr, *hs = nullptr;
        const size_t na = (size_t)bs->n_air;
        e = series_upload(c, &at, na > 0 ? bs->air_time : nullptr, na);
        if (e == cudaSuccess) e = series_upload(c, &av, na > 0 ? bs->air_values : nullptr, 5 * na);
        if (e == cudaSuccess) e = series_upload(c, &hs, (const double *)nullptr, 8);
        const int month_state[2] = {bs->month, 0};
        const int *ms = nullptr;
        if (e == cudaSuccess) e = series_upload(c, &ms, month_state, 2);
        S.heat_month = const_cast<int *>(ms);
        S.sol_swr = bs->sol_swr;
        S.year = bs->year;
        S.lon = bs->lon;
        S.lat = bs->lat;
        S.air_time = at;
        S.air_values = av;
        S.heat_scal = const_cast<double *>(hs);
        S.heat_flag = 1;
        S.n_air = bs->n_air;
        S.fwz_a = bs->fwz_a;
        S.fwz_b = bs->fwz_b;
        S.fwz_c = bs->fwz_c;
        S.wind_height = bs->wind_height;
        S.light_extinction = bs->light_extinction;
        S.sol_absorb = bs->sol_absorb;
        S.sed_water_exchange = bs->sed_water_exchange;
        S.t_sed = bs->t_sed;
        S.sed_temp_coeff = bs->sed_temp_coeff;
    }
    if (e == cudaSuccess && hur2) {
        double track[12] = {0};
        for (int k = 0; k < 6; ++k) track[k] = bs->hurricane_track[k];
        const double *tk = nullptr, *wn = nullptr;
        const int *tr = nullptr, *cnt = nullptr;
        e = series_upload(c, &tk, (const double *)track, 12);
        if (e == cudaSuccess) e = series_upload(c, &tr, (const int *)nullptr, 1);
        if (e == cudaSuccess) e = series_upload(c, &wn, (const double *)nullptr, 3 * nn);
        if (e == cudaSuccess) e = series_upload(c, &cnt, (const int *)nullptr, nn);
        S.hur_track = const_cast<double *>(tk);
        S.hur_track_ready = const_cast<int *>(tr);
        S.hur_w1n = const_cast<double *>(wn);
        // the lists: counts on the device, offsets on the host, then the ids
        std::vector<int> h_count(nn);
        std::vector<long long> h_start(nn + 1, 0);
        if (e == cudaSuccess) e = hurricane_neighbour_counts(c->x.g, const_cast<int *>(cnt), c->x.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->x.stream);
        if (e == cudaSuccess) e = cudaMemcpy(h_count.data(), cnt, nn * sizeof(int), cudaMemcpyDeviceToHost);
        bool empty = false;
        for (size_t i = 0; i < nn && e == cudaSuccess; ++i) {
            h_start[i + 1] = h_start[i] + h_count[i];
            empty = empty || h_count[i] == 0;
        }
        if (e == cudaSuccess && empty) {
            series_free(c);
            return GOM_E_ARG;   // a node with no neighbour in range: IDW_5 would read outside its list
        }
        const long long *st = nullptr;
        const int *nodes = nullptr;
        if (e == cudaSuccess) e = series_upload(c, &st, (const long long *)h_start.data(), nn + 1);
        if (e == cudaSuccess) e = series_upload(c, &nodes, (const int *)nullptr, (size_t)h_start[nn]);
        if (e == cudaSuccess) e = hurricane_neighbour_fill(c->x.g, st, const_cast<int *>(nodes), c->x.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->x.stream);
        S.search_start = st;
        S.search_nodes = nodes;
    }
    if (e != cudaSuccess) {
        series_free(c);
        return set_cuda_error(c, e, "gom_set_boundary_series");
    }
    c->bytes += c->series_bytes;
    // reference_diff_days * 86400.0: an integer times a default-REAL constant, in single precision
    S.rdd_s = (double)((float)bs->reference_diff_days * 86400.0f);
    S.tide_per_s = bs->tide_spinup == 1 ? bs->tide_spinup_period * 86400.0 : 0.0;
    S.bc_per_s = (bs->baroclinic_spinup == 1 && c->hp.baroclinic_flag == 1) ? bs->baroclinic_spinup_period * 86400.0
                                                                                : 0.0;
    S.q_method = bs->q_interp_method;
    S.wind_flag = bs->wind_flag;
    S.wind_formular = bs->wind_formular;
    S.n_wind = nw;
    S.wind_per_s = (bs->wind_flag == 1 && bs->wind_spinup == 1) ? bs->wind_spinup_period * 86400.0 : 0.0;
    S.rho_ratio = (bs->wind_flag == 1 || hur) ? bs->rho_a / c->hp.rho_o : 0.0;
    S.hur_flag = hur ? 1 : 0;
    S.hur_interval = hur ? bs->hurricane_read_interval : 1;
    S.hur_start = bs->hurricane_start_jday;
    S.hur_end = bs->hurricane_end_jday;
    S.hur_cda_max = (double)0.003f;
    S.hur_method = hur2 ? 2 : 1;
    // calculate_wind_stress.f90:20-33: the bounds are default-REAL expressions scaled in double
    const float lo[3] = {0.75f + 0.067f * 4.0f, 0.61f + 0.063f * 6.0f, 0.80f + 0.065f * 1.0f};
    const float hi[3] = {0.75f + 0.067f * 50.0f, 0.61f + 0.063f * 50.0f, 0.80f + 0.065f * 50.0f};
    const int fi = bs->wind_formular >= 1 && bs->wind_formular <= 3 ? bs->wind_formular - 1 : 1;
    S.cda_min = 0.001 * (double)lo[fi];
    S.cda_max = 0.001 * (double)hi[fi];
    // the device clock: elapsed time and spin-up of the last step, its julian day and step number
    const double scal[8] = {bs->step * c->hp.dt, 1.0, 1.0, 0.0, bs->julian_day, (double)bs->step, 1.0, 0.0};
    CK(cudaMemcpy(c->f_scal, scal, sizeof(scal), cudaMemcpyHostToDevice));
    CK(legacy_done());
    c->has_series = true;
    drop_graphs(c);   // the captured step gains the series kernels
    return GOM_OK;
}

int gom_push_hurricane_frame(gom_ctx *c, const double *frame) {
    if (!c || !frame || !c->has_series || c->series.hur_flag != 1) return GOM_E_ARG;
    const size_t bytes = 3 * (size_t)c->d.n_nodes * sizeof(double);
    // on the context's stream: after every step already launched, before every later one
    cudaError_t e = cudaMemcpyAsync(c->series.hur_next, frame, bytes, cudaMemcpyHostToDevice, c->x.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->series.hur_ready, 1, sizeof(int), c->x.stream);
    if (e != cudaSuccess) return set_cuda_error(c, e, "gom_push_hurricane_frame");
    return GOM_OK;
}

int gom_push_hurricane_center(gom_ctx *c, double x, double y, double julian_day) {
    if (!c || !c->has_series || c->series.hur_flag != 1 || c->series.hur_method != 2) return GOM_E_ARG;
    const double rec[3] = {x, y, julian_day};
    // pageable source: staged before the call returns; ordered after every step already launched
    cudaError_t e = cudaMemcpyAsync(c->series.hur_track + 6, rec, sizeof(rec), cudaMemcpyHostToDevice, c->x.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->series.hur_track_ready, 1, sizeof(int), c->x.stream);
    if (e != cudaSuccess) return set_cuda_error(c, e, "gom_push_hurricane_center");
    return GOM_OK;
}

int gom_set_stations(gom_ctx *c, int32_t hloc, int32_t n_stations, const int32_t *station_cell,
                     const int32_t *station_node) {
    if (!c || (hloc != 1 && hloc != 2) || n_stations < 0) return GOM_E_ARG;
    const int32_t *ids = hloc == 1 ? station_cell : station_node;
    const int limit = hloc == 1 ? c->d.n_cells : c->d.n_nodes;
    if (n_stations > 0 && !ids) return GOM_E_ARG;
    for (int q = 0; q < n_stations; ++q)
        if (ids[q] < 1 || ids[q] > limit) return GOM_E_ARG;
    CK(cudaStreamSynchronize(c->x.stream));
    if (c->st_ids) cudaFree(c->st_ids);
    if (c->st_out) cudaFree(c->st_out);
    if (c->st_n > 0) c->bytes -= (size_t)c->st_n * (4 + 8 * (7 + 4 * (size_t)c->d.n_layers));
    c->st_ids = nullptr;
    c->st_out = nullptr;
    c->st_n = 0;
    c->st_hloc = hloc;
    if (n_stations == 0) return GOM_OK;
    const size_t rec = 7 + 4 * (size_t)c->d.n_layers;
    if (cudaMalloc(&c->st_ids, sizeof(int) * n_stations) != cudaSuccess ||
        cudaMalloc(&c->st_out, sizeof(double) * rec * n_stations) != cudaSuccess)
        return GOM_E_NOMEM;
    CK(cudaMemcpy(c->st_ids, ids, sizeof(int) * n_stations, cudaMemcpyHostToDevice));
    CK(legacy_done());
    c->st_n = n_stations;
    c->bytes += (size_t)n_stations * (4 + 8 * rec);
    return GOM_OK;
}

int gom_station_series(gom_ctx *c, double *out) {
    if (!c || (c->st_n > 0 && !out)) return GOM_E_ARG;
    if (c->st_n == 0) return GOM_OK;
    const size_t rec = 7 + 4 * (size_t)c->d.n_layers;
    CK(c->mixed ? launch_station_series(c->xf, c->st_hloc, c->st_n, c->st_ids, c->st_out)
                : launch_station_series(c->x, c->st_hloc, c->st_n, c->st_ids, c->st_out));
    CK(cudaMemcpyAsync(out, c->st_out, sizeof(double) * rec * c->st_n, cudaMemcpyDeviceToHost, c->x.stream));
    CK(cudaStreamSynchronize(c->x.stream));
    return GOM_OK;
}

int gom_conservation(gom_ctx *c, double *volume, double *salt_mass) {
    if (!c) return GOM_E_ARG;
    CK(c->mixed ? launch_conservation(c->xf) : launch_conservation(c->x));
    CK(cudaMemcpyAsync(c->h_cons, c->x.w.cons, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->x.stream));
    CK(cudaStreamSynchronize(c->x.stream));
    if (volume) *volume = c->h_cons[0];
    if (salt_mass) *salt_mass = c->h_cons[1];
    return GOM_OK;
}

}  // extern "C"
