// gom_launch.h -- host-side launch interface between the ABI layer (gom_core.cu) and the kernel
// files.  Every launcher enqueues work on the context stream and returns a cudaError_t.
#pragma once

#include "gom_device.cuh"

namespace gom {

// device work buffers owned by a context (R: storage type of the layered state)
template <typename R> struct WorkT {
    // free surface / PCG (the system, its right-hand side and the solution are always FP64)
    double *sparsem = nullptr;   // (0:4, NC)
    double *rhs = nullptr;       // (NC)
    double *minv = nullptr, *r = nullptr, *s = nullptr, *q = nullptr, *d0 = nullptr, *d1 = nullptr;
    // single-run FP64 solver: second buffers of s and w, scaled solution x'
    double *cg_s1 = nullptr, *cg_w1 = nullptr, *cg_xs = nullptr;
    double *partial_dq = nullptr, *partial_delta = nullptr;   // (2 x max_blocks)
    unsigned *barrier = nullptr;                               // [count, generation]
    int *pcg_iters = nullptr;                                  // device: iterations of the last solve
    int pcg_blocks = 0, pcg_threads = 256;
    int *run_block_start = nullptr;   // packed runs: first PCG block of each run (NR + 1), device
    int *run_iters = nullptr;         // packed runs: PCG iterations of each run's last solve, device
    float *sp32 = nullptr;       // mixed precision: FP32 copy of the system (0:4, NC)
    // transport
    R *con = nullptr, *con2 = nullptr;        // (0:L+1, NC, 2)
    R *qj = nullptr, *dj = nullptr, *phij = nullptr;            // (L, NF)
    R *qi = nullptr, *di = nullptr, *phii = nullptr;            // (0:L, NC)
    R *psij = nullptr;                                          // (L, NF, 2)
    R *psii = nullptr;                                          // (0:L, NC, 2)
    R *sa1 = nullptr, *sa2 = nullptr;                           // (L, NC, 2) limiter sums per layer
    R *obk = nullptr, *qbk = nullptr;                           // (L, NOB, 2), (L, NQB, 2)
    // ELM: INT(dev/0.1) per (layer, face) edge
    int *idev = nullptr;
    // ELM: compact list of the face-layers the walk visits (gom_scan.cuh); fl_count = [length,
    // work-queue counter]; null when the mesh has too many faces for the list encoding
    int *fl_list = nullptr, *fl_off = nullptr, *fl_bsum = nullptr, *fl_count = nullptr;
    // node velocities: face-level velocity / face length (0:L, NF), static node weights (NN)
    R *uflf = nullptr, *vflf = nullptr;
    double *node_weight = nullptr;
    // FP64 node velocities: static list of the (node, level + 1) pairs from the lowest level any
    // face or cell of the node reaches (gom_scan.cuh); null when L + 1 exceeds the list encoding
    int *nl_list = nullptr, *nl_off = nullptr, *nl_bsum = nullptr, *nl_count = nullptr;
    // turbulence closure: face diffusivity per interface (0:L, NF)
    R *kvf = nullptr;
    // mixed-precision transport: rows of the vertical systems (L, NC) and right-hand sides
    // (L, NC, 2); top-layer horizontal sums of the limiter (2, NC, 2)
    R *tr_a = nullptr, *tr_b = nullptr, *tr_c = nullptr, *tr_rhs = nullptr, *tr_last = nullptr;
    // mixed-precision transport: compact list of the wet (cell, layer) pairs and its scan arrays
    int *cl_list = nullptr, *cl_off = nullptr, *cl_bsum = nullptr, *cl_count = nullptr;
    // conservation
    double *cons = nullptr;                                     // [volume, salt]
    double *fs_sums = nullptr;                                  // free-surface column sums (3, NF)
};
using Work = WorkT<double>;

// Tunable launches: each picks one of a few compiled variants (block size, minimum resident
// blocks per SM); gom_autotune times the variants on the context's state and keeps the fastest.
enum TuneSite { TUNE_ELM = 0, TUNE_MOMENTUM, TUNE_TR_SOLVE, TUNE_TR_LIMITER, TUNE_COUNT };
// TUNE_TR_SOLVE: FP64 column solve with 128 / 64 / 256 threads, or (3) rows per listed wet
// cell-layer then one thread per column (the FP32 path's form); TUNE_TR_LIMITER: column kernels
// with 128 / 64 / 256 threads, or (3) the per-(entity, layer) list kernels (the only form of the
// FP32 path), or the two mixed: (4) cell sums per listed wet cell-layer with the face limiter per
// face, (5) cell sums per column (64 threads) with the face limiter per face-layer, (6) variant 1
// with the face coefficients per face-layer.  Variants 3-6 change nothing in an FP32 context.
constexpr int TUNE_VARIANTS[TUNE_COUNT] = {7, 4, 4, 7};

// packed runs a free-surface solve holds (one barrier pair and one state per run)
constexpr int PCG_MAX_RUNS = 256;

template <typename R> struct LaunchT {
    int tune[TUNE_COUNT] = {0, 0, 0, 0};
    Geom g;
    StateT<R> s;
    Forcing f;
    Params p;
    WorkT<R> w;
    gom_status *status = nullptr;   // device
    cudaStream_t stream = nullptr;
    int num_sms = 0;
};
using Launch = LaunchT<double>;

template <typename R> cudaError_t launch_bottom_friction(const LaunchT<R> &x);
template <typename R> cudaError_t launch_boundary_velocity(const LaunchT<R> &x);
template <typename R> cudaError_t launch_advection(const LaunchT<R> &x);
template <typename R> cudaError_t launch_momentum(const LaunchT<R> &x);
template <typename R> cudaError_t launch_free_surface(const LaunchT<R> &x);
template <typename R> cudaError_t launch_velocities(const LaunchT<R> &x);
template <typename R> cudaError_t launch_transport_elm(const LaunchT<R> &x);
template <typename R> cudaError_t launch_layers(const LaunchT<R> &x);
template <typename R> cudaError_t launch_node_velocity(const LaunchT<R> &x);
template <typename R> cudaError_t launch_transport(const LaunchT<R> &x);
template <typename R> cudaError_t launch_density(const LaunchT<R> &x);
template <typename R> cudaError_t launch_turbulence(const LaunchT<R> &x);
template <typename R> cudaError_t launch_conservation(const LaunchT<R> &x);
// station records of write_tser_out_files.f90 (7 + 4 L doubles per station) into out
template <typename R>
cudaError_t launch_station_series(const LaunchT<R> &x, int hloc, int n, const int *ids, double *out);

// cooperative PCG set-up (grid size from occupancy); called once per context
template <typename R> cudaError_t pcg_configure(LaunchT<R> &x, int device);
// static per-node weights of calculate_velocity_at_node.f90:103; called once per context
template <typename R> cudaError_t launch_node_weights(const LaunchT<R> &x);

// one kernel of a phase alone, on the current state (for timing): the ELM walk, the momentum
// columns, the transport column solve of one subcycle (the transport phase must have run)
template <typename R> cudaError_t launch_elm_walk_only(const LaunchT<R> &x);
template <typename R> cudaError_t launch_momentum_columns_only(const LaunchT<R> &x);
template <typename R> cudaError_t launch_tr_solve_only(const LaunchT<R> &x);

// FP32 element node offsets (8 per element) for the mixed-precision ELM, once per context
cudaError_t launch_elem_local(const Geom &g, float *out, cudaStream_t stream);
cudaError_t launch_edge_len2(const Geom &g, float *out, cudaStream_t stream);
cudaError_t launch_cell_zbot(const Geom &g, double msl, double *out, cudaStream_t stream);
cudaError_t launch_cell_zbot_f(const Geom &g, const double *zbot, float *out, cudaStream_t stream);
// FP64 copy of an FP32 array (n elements)
cudaError_t launch_to_double(const float *in, double *out, long n, cudaStream_t stream);
// FP32 copy of an FP64 array (n elements)
cudaError_t launch_to_float(const double *in, float *out, long n, cudaStream_t stream);

// cold start on the device (all state fields must have been cleared first)
template <typename R>
cudaError_t launch_cold_start(const LaunchT<R> &x, double salt, double temp, double av0, double kv0);

// per-step storm-surge forcing on the device (k_forcing.cu): advances the elapsed time by dt and
// writes the forcing arrays of f from the runs' storms (12 doubles each, gom_storm order)
cudaError_t launch_storm_forcing(const Geom &g, const Forcing &f, const Params &p, cudaStream_t stream,
                                 const double *storms, double *wu, double *wv);

// device copies of a gom_boundary_series (k_forcing.cu evaluates them at the start of every step)
struct SeriesDev {
    int n[6];                              // series per kind: 0 eta, 1 Q, 2 salinity, 3 temperature,
                                           // 4 station wind u, 5 station wind v
    const int *start[6];                   // (n + 1) offsets per kind
    const double *time[6], *value[6];
    const int *ob_type, *ob_h, *ob_eta, *ob_salt, *ob_temp;   // (NOB)
    const int *qb_q, *qb_salt, *qb_temp;                      // (NQB)
    const double *qb_portion;                                 // (NQB)
    int n_harm;
    const int *h_start;                    // (n_harm + 1)
    const double *amp, *per_h, *nodal, *eq, *ph, *shift;
    double rdd_s;                          // reference_diff_days x 86400.0 (single precision, widened)
    double tide_per_s, bc_per_s;           // spin-up periods in seconds, 0 = no ramp
    int q_method;
    // station wind (get_windp_at_face.f90, IDW_windp_ser.f90, calculate_wind_stress.f90)
    int wind_flag, wind_formular, n_wind;
    double wind_per_s;                     // wind spin-up period in seconds, 0 = no ramp
    double rho_ratio, cda_min, cda_max;    // rho_a / rho_o and the drag-coefficient bounds
    const int *wind_node;                  // (n_wind) station nodes
    double *wind_at_station;               // (2 n_wind) work: u, v of each station this step
    // hurricane node frames (read_hurricane_ser_1.f90, calculate_wind_stress.f90:105-137)
    int hur_flag, hur_interval;
    double hur_start, hur_end;             // julian-day window
    double *hur_frames;                    // (NN, 3, 3): frames 0, 1, 2 of (u, v, air_p)
    double *hur_next;                      // (NN, 3) the record pushed for the next read step
    int *hur_ready;                        // nonzero once a record is pushed, cleared when taken
    double *face_u, *face_v;               // (NF) wind_u_at_face / wind_v_at_face, kept between steps
    double hur_cda_max;                    // MIN(0.003, Cda): the default-REAL 0.003 widened
    // method 2 (read_hurricane_ser_2.f90, IDW_5.f90): the track [x1, y1, t1, x2, y2, t2], the
    // pushed centre [6..8], this step's time ratio and centre shift [9..11]; find_neighbour_nodes'
    // lists (CSR); the blended frame 1 of the step
    int hur_method;
    double *hur_track;
    int *hur_track_ready;
    const long long *search_start;         // (NN + 1)
    const int *search_nodes;
    double *hur_w1n;                       // (NN, 3)
    // heat balance (heat_term_by_term.f90, sol_swr 2): the air series, card C7_3 / C7_4 values and
    // this step's scalar terms [Ta, phi_sn, phi_an, fWz, ea]
    int heat_flag, n_air, sol_swr, year;
    int *heat_month;                       // julian_to_localtime's state: [month, table set]
    double lon, lat;
    const double *air_time, *air_values;   // (n_air), (n_air, 5)
    double fwz_a, fwz_b, fwz_c, wind_height, light_extinction, sol_absorb, sed_water_exchange, t_sed,
        sed_temp_coeff;
    double *heat_scal;
};

// per-step boundary forcing from the series (k_forcing.cu): advances the device clock in f.scal
// ([0] elapsed_time, [1] spin-up tide, [2] spin-up baroclinic, [4] julian_day, [5] it, [6] spin-up
// wind), forms the station wind stress when wind_flag is 1 (the hurricane drag law on the hurricane
// or station face winds when hur_flag is 1, with air_p from the node frames), then
// writes eta_at_ob_old/new (type -1 from eta_cell; an isolated cell records GOM_E_ARG in
// status), q_add and the boundary concentrations of every subcycle
cudaError_t launch_series_forcing(const Geom &g, const Forcing &f, const Params &p, const SeriesDev &s,
                                  const double *eta_cell, gom_status *status, cudaStream_t stream);
// heat_term_by_term.f90 (sol_swr 2) before the transport: the air series at julian_day, then
// phi_sz and phi_sw of every wet column from its top and bottom temperatures (R: the state type)
template <typename R>
cudaError_t launch_heat_terms(const Geom &g, const Forcing &f, const StateT<R> &s, const SeriesDev &S,
                              cudaStream_t stream);

// find_neighbour_nodes.f90 on the device (hurricane method 2): per node the count of its
// neighbours in range, then (start: NN + 1 offsets) their 1-based ids in node order
cudaError_t hurricane_neighbour_counts(const Geom &g, int *count, cudaStream_t stream);
cudaError_t hurricane_neighbour_fill(const Geom &g, const long long *start, int *nodes, cudaStream_t stream);

// explicit instantiations live in the kernel files
#define GOM_INSTANTIATE_LAUNCH(fn)                              \
    template cudaError_t fn<double>(const LaunchT<double> &x); \
    template cudaError_t fn<float>(const LaunchT<float> &x);

}  // namespace gom
