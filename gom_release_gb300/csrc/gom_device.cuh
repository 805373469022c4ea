// gom_device.cuh -- device-side data views and helpers shared by the GOM core kernels.
//
// Memory layout is that of the Fortran module arrays (include/gom_core.h): every cell, face and
// node column is contiguous over its layers, so one warp staging a batch of columns reads
// contiguous bytes.  Entity indices stay 1-based as in the reference connectivity.
//
// Floating point: the library is compiled with -fmad=false and IEEE division/square root, so
// each expression below rounds exactly like the serial FP64 restatement of the reference.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/gom_core.h"

#define GOM_MAXL 64          // largest n_layers a context accepts
#define GOM_BT_TABLE 32      // ELM substep counts with a precomputed dt / n
#define GOM_MAXNB 16         // largest max_no_neighbor_node a context accepts

namespace gom {

__host__ __device__ inline double F(float x) { return (double)x; }

// -------------------------------------------------------------------- static geometry (device)
struct Geom {
    int NC, NF, NN, L, NB, NOB, NQB;
    // nodes
    const double *x_node, *y_node, *h_node;
    const int *adj_cells_at_node, *adj_cellnum_at_node, *node_count_each_element;
    const int *adj_nodes_at_node, *adj_nodenum_at_node, *bottom_node, *initial_wetdry_node;
    // cells
    const double *x_cell, *y_cell, *h_cell, *area;
    const int *tri_or_quad, *nodenum_at_cell, *facenum_at_cell, *adj_cellnum_at_cell, *sign_in_outflow;
    const int *bottom_cell, *ob_element_flag, *qb_element_flag;
    // faces
    const double *x_face, *y_face, *h_face, *face_length, *delta_j, *cos_theta, *sin_theta, *cos_theta2,
        *sin_theta2, *coriolis_factor, *manning, *bf_height;
    const int *adj_cellnum_at_face, *nodenum_at_face, *bottom_face, *boundary_type_of_face, *isflowside3;
    // bottom drag coefficients formed on the host with the C library's pow / log (the functions
    // the reference calls): bf_flag 1 Manning Cdb per face; bf_flag 2 the log-law Cdb of the
    // static bottom half-thickness (z_level(b) - (MSL - h) of a column with more than one layer)
    // and that half-thickness; null otherwise
    const double *cdb_static, *cdb_arg;
    // boundaries / vertical grid
    const int *ob_cell_id, *qb_cell, *qb_face;
    const double *z_level, *delta_z;
    // entity ids sorted by bottom layer: column kernels take their entity from these so that the
    // 32 lanes of a warp walk columns of nearly equal height (results do not depend on the order)
    const int *cell_order, *face_order, *node_order;
    // element node offsets from the element centre in FP32, (8, NC): x1..x4, y1..y4 (mixed path)
    const float *elem_local;
    // FP32 copies of per-entity geometry and of the static node weights for the mixed path (null
    // in FP64 contexts): a conversion from FP64 runs on the FP64 pipe, so FP32 kernels read these
    const float *area_f, *face_length_f, *delta_j_f, *cos_theta_f, *sin_theta_f, *node_weight_f;
    const float *edge_len2_f;   // squared node-to-node length of each face
    const float *z_level_f;     // the L + 1 level heights
    const double *zbot_cell;    // MSL - h of each cell
    const float *zbot_cell_f;   // its FP32 copy (mixed contexts), kept above z_level[0] where it is
    // packed runs (NR > 1): 0-based first cell / face / node / open-boundary cell of each run
    int NR;
    const int *run_cell_start, *run_face_start, *run_node_start, *run_ob_start;

    // 1-based accessors of the (m, N) connectivity arrays
    __device__ __forceinline__ int cell_node(int l, int i) const { return nodenum_at_cell[(i - 1) * 4 + l - 1]; }
    __device__ __forceinline__ int cell_face(int l, int i) const { return facenum_at_cell[(i - 1) * 4 + l - 1]; }
    __device__ __forceinline__ int cell_adj(int l, int i) const { return adj_cellnum_at_cell[(i - 1) * 4 + l - 1]; }
    __device__ __forceinline__ int cell_sign(int l, int i) const { return sign_in_outflow[(i - 1) * 4 + l - 1]; }
    __device__ __forceinline__ int face_cell(int l, int j) const { return adj_cellnum_at_face[(j - 1) * 2 + l - 1]; }
    __device__ __forceinline__ int face_node(int l, int j) const { return nodenum_at_face[(j - 1) * 2 + l - 1]; }
    __device__ __forceinline__ int node_cell(int l, int i) const { return adj_cellnum_at_node[(i - 1) * NB + l - 1]; }
    __device__ __forceinline__ int node_count(int l, int i) const { return node_count_each_element[(i - 1) * NB + l - 1]; }
    __device__ __forceinline__ int node_nb(int l, int i) const { return adj_nodenum_at_node[(i - 1) * (NB + 1) + l]; }
};

// -------------------------------------------------------------------- state (device)
// R is the storage type of the layered state: double for the FP64 path (bit-for-bit with the
// reference restatement), float for the mixed-precision path.  Elevations (the free-surface
// solution), densities and the river boundary velocity stay double in both.
template <typename R> struct StateT {
    double *eta_cell, *eta_cell_new, *eta_node;
    int *wetdry_node;
    R *un_face, *vn_face, *un_face_new, *vn_face_new, *un_elm, *vn_elm;
    R *wn_cell, *wn_cell_new, *u_node, *v_node, *w_node, *u_face_level, *v_face_level;
    R *dz_cell, *dz_cell_new, *dzhalf_cell, *dzhalf_cell_new;
    R *dz_face, *dz_face_new, *dzhalf_face, *dzhalf_face_new;
    R *dz_node, *dz_node_new, *dzhalf_node, *dzhalf_node_new;
    int *top_cell, *top_face, *top_node;
    R *ainvg1, *ainvg2, *ainvdz1, *ainvdz2, *kh, *av, *kv;
    R *salt_cell, *salt_cell_new, *temp_cell, *temp_cell_new, *salt_node, *temp_node, *salt_face, *temp_face;
    double *rho_cell, *rho_node, *rho_face;   // FP64 in both: baroclinic terms difference them
    int *num_sub_elm;
    R *cdb, *gamma_b;
    double *qu_boundary;
    int *elm_foot, *elm_near_edge;
    // derived at the start of each ELM step (not fields): MSL + eta and the ELM dry test per cell
    double *ztop_cell;
    float *ztop_cell_f;   // FP32 copy of ztop_cell (mixed contexts only)
    int *dry_cell;
};
using State = StateT<double>;

// per-step forcing (device copies)
struct Forcing {
    const double *scal;   // [elapsed_time, spinup_tide, spinup_baroclinic] in device memory
    const double *eta_at_ob_old, *eta_at_ob_new, *q_add, *wind_stress_normal, *wind_stress_tangnt, *gamma_t, *air_p,
        *con_at_ob, *con_at_qb, *phi_sw;
    const double *phi_sz;   // (L, NC) heat source per layer (heat_option 1, ELM transport)
};

// scalar parameters
struct Params {
    double gravity, rho_o, msl, dt, theta, adv_onoff_depth, von_karman, cd_const, dry_depth, smagorinsky, ah_0,
        kh_0, error_tolerance, delta_z_min, denominator_min_for_matrix;
    int advection_flag, elm_backtrace_flag, elm_sub_iter, elm_min_iter, elm_max_iter, bf_flag, baroclinic_flag,
        ana_density, max_iteration_pcg, transport_flag, trans_sub_iter, h_flux_limiter, v_flux_limiter, is_salt,
        is_temp, heat_option, test_barrier_phantom_blocks, turbulence_flag, transport_solver;
    double pp_h1, pp_h2, pp_vdmax1, pp_vdmax2, pp_vdmin1, pp_vdmin2, pp_tdmin;
    double bt_dt[GOM_BT_TABLE];   // dt / n for ELM substep counts n = 1..GOM_BT_TABLE
};

// -------------------------------------------------------------------- layer indexing
// (1:L, N) arrays
__device__ __forceinline__ long ix(int k, int e, int L) { return (long)(e - 1) * L + (k - 1); }
// (0:L, N) arrays
__device__ __forceinline__ long ix0(int k, int e, int L) { return (long)(e - 1) * (L + 1) + k; }

// Column kernels take their entity from a bottom-layer-sorted order in the FP64 path (the 32
// columns of a warp have nearly equal heights, which keeps the FP64 pipe busy); the FP32 path
// takes entities in natural order, where neighbouring lanes work on neighbouring columns of the
// (layer, entity) arrays and share their memory sectors.
template <typename R> __device__ __forceinline__ int column_entity(const int *order, unsigned tid) {
    if constexpr (sizeof(R) == sizeof(float)) return (int)tid + 1;
    else return order[tid];
}

// an entity's geometry value in the layered-state type: the FP64 array for R = double, its FP32
// copy for R = float
template <typename R> __device__ __forceinline__ R geo(const double *d, const float *f, int i) {
    if constexpr (sizeof(R) == sizeof(float)) return f[i];
    else return d[i];
}

// -------------------------------------------------------------------- error status
// The first failure wins; kind is the GOM_ENTITY_* that entity indexes (the host maps it to a
// packed run).
__device__ inline void record_error(gom_status *st, int code, int site, int entity, int layer, double value,
                                    int kind) {
    if (atomicCAS(&st->code, 0, code) == 0) {
        st->site = site;
        st->entity = entity;
        st->layer = layer;
        st->value = value;
        st->entity_kind = kind;
    }
}

__device__ __forceinline__ bool failed(const gom_status *st) { return *(volatile const int *)&st->code != 0; }

// -------------------------------------------------------------------- geometry helpers
// mod_function_library.f90:49-60 (x/2 == x*0.5 exactly)
__device__ __forceinline__ double calculate_area(double x1, double x2, double x3, double y1, double y2, double y3) {
    return fabs((x1 - x3) * (y2 - y3) - (x2 - x3) * (y1 - y3)) * 0.5;
}
template <typename T>
__device__ __forceinline__ T calculate_area_t(T x1, T x2, T x3, T y1, T y2, T y3) {
    return fabs((x1 - x3) * (y2 - y3) - (x2 - x3) * (y1 - y3)) * T(0.5);
}

// Comparisons on the bit patterns (integer pipe).  GB300's FP64 pipe issues a warp instruction in
// about 80 cycles per SM sub-partition, comparisons included, so the sign and size tests of the
// hot kernels run as integer compares; each gives the FP64 comparison's result for every input
// the caller can pass, NaN and signed zeros included:
//   is_zero(x)            x == 0
//   pos_finite_or_inf(x)  x > 0
//   gt_nonneg(x, y)       x > y    for y >= +0 or NaN (never -0)
//   lt_of_nonneg(x, y)    x < y    for x with its sign bit clear (+0, positive, +inf, +NaN)
// Non-negative doubles (floats) are ordered as their bit patterns; an infinity's pattern is the
// largest of them and a NaN's lies above it (sign clear) or below zero (sign set).
__device__ __forceinline__ long long fbits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ int fbits(float x) { return __float_as_int(x); }
__device__ __forceinline__ long long inf_bits(double) { return 0x7ff0000000000000LL; }
__device__ __forceinline__ int inf_bits(float) { return 0x7f800000; }
__device__ __forceinline__ bool is_zero(double x) { return ((unsigned long long)fbits(x) << 1) == 0ull; }
__device__ __forceinline__ bool is_zero(float x) { return ((unsigned)fbits(x) << 1) == 0u; }
template <typename R> __device__ __forceinline__ bool pos_finite_or_inf(R x) {
    const auto b = fbits(x);
    return b > 0 && b <= inf_bits(x);
}
template <typename R> __device__ __forceinline__ bool gt_nonneg(R x, R y) {
    const auto xb = fbits(x), yb = fbits(y);
    return yb >= 0 && yb <= inf_bits(x) && xb > yb && xb <= inf_bits(x);
}
__device__ __forceinline__ bool nan_bits(double x) {
    return (__double_as_longlong(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
}
__device__ __forceinline__ bool nan_bits(float x) { return (__float_as_int(x) & 0x7fffffff) > 0x7f800000; }
template <typename R> __device__ __forceinline__ bool lt_of_nonneg(R x, R y) {
    const auto yb = fbits(y);
    return yb <= inf_bits(x) && fbits(x) < yb;
}

// Exact decisions about a rounded quotient fl(num/den) (num >= 0, den > 0) against a constant c,
// deciding from num and c*den when they are more than 1e-9 apart (far beyond every rounding
// error involved) and dividing only otherwise.  Same outcome as the division, fewer FP64 ops;
// the comparisons on the bit patterns (num >= 0 and c den > 0).
__device__ __forceinline__ bool quotient_gt(double num, double den, double c) {
    double t = c * den;
    if (gt_nonneg(num, t * (1.0 + 1e-9))) return true;
    if (lt_of_nonneg(num, t * (1.0 - 1e-9))) return false;
    return gt_nonneg(num / den, c);
}
__device__ __forceinline__ bool quotient_lt(double num, double den, double c) {
    double t = c * den;
    if (lt_of_nonneg(num, t * (1.0 - 1e-9))) return true;
    if (gt_nonneg(num, t * (1.0 + 1e-9))) return false;
    return lt_of_nonneg(num / den, c);
}

// set_geometry_1.f90:48-63
__device__ __forceinline__ int start_end_node(int k, int i, int j) {
    int v = i + j;
    return v > k ? v - k : v;
}

// tridiagonal_solver.f90:15-61, NRHS right-hand sides held in registers/local memory.
// Returns false on a zero pivot.
template <int NRHS, typename R>
__device__ inline bool thomas(int n, const R *a, const R *b, const R *c, R (*rhs)[NRHS], R *gam) {
    if (b[0] == R(0)) return false;
    R den = b[0];
#pragma unroll
    for (int r = 0; r < NRHS; ++r) rhs[0][r] = rhs[0][r] / den;
    for (int j = 1; j < n; ++j) {
        gam[j] = c[j - 1] / den;
        den = b[j] - a[j] * gam[j];
        if (den == R(0)) return false;
#pragma unroll
        for (int r = 0; r < NRHS; ++r) rhs[j][r] = (rhs[j][r] - a[j] * rhs[j - 1][r]) / den;
    }
    for (int j = n - 2; j >= 0; --j) {
#pragma unroll
        for (int r = 0; r < NRHS; ++r) rhs[j][r] = rhs[j][r] - gam[j + 1] * rhs[j + 1][r];
    }
    return true;
}

// -------------------------------------------------------------------- flat thread indices
// Flat (entity, layer) thread indices stay in 32 bits: a 64-bit integer division is emulated
// partly on the FP64 pipe, the scarcest unit of this GPU, while the 32-bit one is not.
__device__ __forceinline__ unsigned flat_tid() { return blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ void split_index(unsigned t, unsigned n, int &e0, int &k0) {
    unsigned q = t / n;
    e0 = (int)q;
    k0 = (int)(t - q * n);
}

// -------------------------------------------------------------------- launch helpers
inline int blocks_for(long n, int threads) { return (int)((n + threads - 1) / threads); }

}  // namespace gom
