// gom_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A serial FP64 CPU restatement of GOM's per-timestep core (GOM_Rv1.1.0/source), used by the
// tests, smoke() and bench.py's CPU-baseline leg as the checker of the CUDA library.  It is
// never linked into, loaded by or called from the product path (libgomcore.so).
//
// It exports the C ABI of include/gom_core.h.  Every routine follows the Fortran file and lines
// cited beside it, in the same loop order and the same floating-point operation order, with
// these rules:
//   * compiled with -O2 -ffp-contract=off (no fused multiply-add), like gfortran -O2 on x86-64;
//   * default-REAL (single precision) literals of the Fortran source are written F(x) =
//     (double)(float)x, because gfortran promotes them from single precision;
//   * x**2 is x*x; x**3 = (x*x)*x; x**4 = (x*x)*(x*x); x**5 = ((x*x)*x)*(x*x), GCC's powi
//     expansion for constant exponents;
//   * loops run serially in index order, so order-dependent reference behaviour (the stale
//     rtemp0 of solve_momentum_equation.f90:503, the last-writer r_jk of
//     solve_transport_equation_v19.f90:789-796) is that of a single-threaded run;
//   * entries of the reference's automatic work arrays that the reference reads without ever
//     assigning them in the call (solve_transport_equation_v19.f90:738,809,806,1130,1136) are
//     defined as 0 (no flux).
//
// Parity is unpinned: the reference has no tests or golden vectors and cannot be compiled in
// this environment (no Fortran compiler), so this file is checked against known-answer tests
// derived from the mathematics (tests/test_oracle_kat.py) and the CUDA library against it.
//
// Built a second time with -fopenmp -DGOM_ORACLE_OMP (oracle/Makefile, libgomoracle_omp.so) as
// the multithreaded CPU timing baseline: the entity loops the reference runs as OpenMP parallel
// do (every hot subroutine) become parallel for loops, the dot products become reductions, and
// the reference's serial parts (the CSR pack of solve_free_surface_equation.f90:235-258, the
// boundary-cell loops) stay serial.  That build is for timing only: the order-dependent values
// above (stale rtemp0, last-writer r_jk) and the PCG sums then depend on the thread split, as
// they do in the reference's own OpenMP build.  Without GOM_ORACLE_OMP the pragmas vanish and
// the loops run serially in index order.

#include "../include/gom_core.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#ifdef GOM_ORACLE_OMP
#include <omp.h>
#endif

#define GOM_PRAGMA(x) _Pragma(#x)
#ifdef GOM_ORACLE_OMP
#define OMP_FOR GOM_PRAGMA(omp parallel for schedule(dynamic, 256))
#define OMP_FOR_SUM(v) GOM_PRAGMA(omp parallel for reduction(+ : v) schedule(static))
#define OMP_FOR_FIRSTPRIVATE(v) GOM_PRAGMA(omp parallel for firstprivate(v) schedule(static))
#define OMP_CRITICAL GOM_PRAGMA(omp critical(gom_err))
#else
#define OMP_FOR
#define OMP_FOR_SUM(v)
#define OMP_FOR_FIRSTPRIVATE(v)
#define OMP_CRITICAL
#endif

namespace {

inline double F(float x) { return (double)x; }

constexpr int GOM_ORACLE_MAXL = 64;   // largest n_layers gom_create accepts

// 1-D array with 1-based index
template <typename T> struct A1 {
    T *p = nullptr;
    T &operator()(long i) const { return p[i - 1]; }
};
// 2-D Fortran array (lo:hi, 1:N): element (k, e)
template <typename T> struct A2 {
    T *p = nullptr;
    int lo = 1, n = 0;
    T &operator()(long k, long e) const { return p[(e - 1) * (long)n + (k - lo)]; }
};

struct Err {
    int code = 0, site = 0, entity = 0, layer = 0;
    double value = 0;
    int kind = 0;   // GOM_ENTITY_* of entity
};

}  // namespace

struct gom_ctx {
    gom_dims d{};
    gom_params p{};
    int L = 0, NC = 0, NF = 0, NN = 0, NB = 0, NOB = 0, NQB = 0;
    bool snap_pending = false;
    Err err;
    std::string msg;
    long long pcg_total = 0;
    int pending_rc = 0;
    int32_t pending_iters = 0;

    // ---------------- geometry storage
    std::vector<double> g_x_node, g_y_node, g_h_node, g_x_cell, g_y_cell, g_h_cell, g_area;
    std::vector<double> g_x_face, g_y_face, g_h_face, g_face_length, g_delta_j, g_cos_theta, g_sin_theta,
        g_cos_theta2, g_sin_theta2, g_coriolis, g_manning, g_bf_height, g_z_level, g_delta_z;
    std::vector<int32_t> g_adj_cells_at_node, g_adj_cellnum_at_node, g_node_count_each_element,
        g_adj_nodes_at_node, g_adj_nodenum_at_node, g_bottom_node, g_initial_wetdry_node, g_tri_or_quad,
        g_nodenum_at_cell, g_facenum_at_cell, g_adj_cellnum_at_cell, g_sign_in_outflow, g_bottom_cell,
        g_ob_element_flag, g_qb_element_flag, g_adj_cellnum_at_face, g_nodenum_at_face, g_bottom_face,
        g_boundary_type_of_face, g_isflowside3, g_ob_cell_id, g_qb_cell, g_qb_face;
    std::vector<int32_t> run_cell_start;   // packed runs: first cell of each run (0-based), n_runs + 1
    std::vector<int32_t> run_face_start;   // packed runs: first face of each run (0-based), n_runs + 1
    std::vector<int32_t> run_node_start;   // packed runs: first node of each run (0-based), n_runs + 1
    // time-series stations (gom_set_stations): tser_hloc and the station cells or nodes
    int tser_hloc = 0;
    std::vector<int32_t> tser_station;

    // ---------------- state storage, indexed by gom_field
    std::vector<double> fd[GOM_F_COUNT];
    std::vector<int32_t> fi[GOM_F_COUNT];

    // ---------------- forcing
    double elapsed_time = 0, spinup_tide = 1, spinup_baroclinic = 1;
    // boundary series (gom_set_boundary_series), evaluated at the start of gom_step_all
    bool has_series = false;
    double jday = 0, rdd_s = 0, tide_per_s = 0, bc_per_s = 0;
    int step_no = 0, q_method = 1, n_harm = 0;
    std::vector<int32_t> sr_start[6];   // eta, Q, salinity, temperature, station wind u, v
    std::vector<double> sr_time[6], sr_value[6];
    int wind_flag = 0, wind_formular = 1, n_wind = 0;
    double wind_per_s = 0, rho_ratio = 0, cda_min = 0, cda_max = 0;
    std::vector<int32_t> wind_node;
    // hurricane node frames (read_hurricane_ser_0/1.f90): wind_u0.. / wind_u1.. / wind_u2.. as
    // (NN, 3, 3), the pushed record, wind_u_at_face / wind_v_at_face
    int hur_flag = 0, hur_interval = 1, hur_method = 1;
    bool hur_ready = false, track_ready = false;
    double hur_start = 0, hur_end = 0;
    std::vector<double> hur_frames, hur_next, face_u, face_v;
    // method 2 (read_hurricane_ser_2.f90): hurric_x_1, hurric_y_1, hurricane_time_1, hurric_x_2,
    // hurric_y_2, hurricane_time_2, the pushed centre, and find_neighbour_nodes' lists (CSR)
    double track[6] = {0, 0, 0, 0, 0, 0}, track_next[3] = {0, 0, 0};
    std::vector<int64_t> search_start;
    std::vector<int32_t> search_nodes;
    // heat balance (heat_term_by_term.f90, sol_swr 2): air series and card values
    int heat_flag = 0, sol_swr = 2, year = 2001, month = 1, month_table_set = 0;
    double lon = 0, lat = 0;
    std::vector<double> air_time, air_values;
    double fwz_a = 0, fwz_b = 0, fwz_c = 0, wind_height = 0, light_extinction = 0, sol_absorb = 0,
           sed_water_exchange = 0, t_sed = 0, sed_temp_coeff = 0;
    std::vector<int32_t> ob_type, ob_h, ob_eta, ob_salt, ob_temp, qb_q, qb_salt, qb_temp, h_start;
    std::vector<double> qb_portion, h_amp, h_per, h_nodal, h_eq, h_ph, h_shift;
    std::vector<double> eta_at_ob_old, eta_at_ob_new, q_add, wind_stress_normal, wind_stress_tangnt, gamma_t,
        air_p, con_at_ob, con_at_qb, phi_sw, phi_sz;

    // ---------------- accessors (geometry)
    A1<double> x_node, y_node, h_node, x_cell, y_cell, h_cell, area, x_face, y_face, h_face, face_length, delta_j,
        cos_theta, sin_theta, cos_theta2, sin_theta2, coriolis_factor, manning, bf_height, delta_z;
    A2<double> z_level;  // (0:L, 1) used as z_level(k, 1)
    A1<int32_t> adj_cells_at_node, adj_nodes_at_node, bottom_layer_at_node, initial_wetdry_node, tri_or_quad,
        bottom_layer_at_element, ob_element_flag, Qb_element_flag, bottom_layer_at_face, boundary_type_of_face,
        isflowside3, ob_cell_id, qb_cell, qb_face;
    A2<int32_t> adj_cellnum_at_node, node_count_each_element, adj_nodenum_at_node, nodenum_at_cell,
        facenum_at_cell, adj_cellnum_at_cell, sign_in_outflow, adj_cellnum_at_face, nodenum_at_face;

    double zl(int k) const { return g_z_level[k]; }
};

namespace {

struct FieldShape {
    int lo;       // lower layer bound, or -1 for a 1-D entity array
    int kind;     // 0 cells, 1 faces, 2 nodes, 3 qb
    int is_int;
    int extra;    // 0: hi = L ; 1: hi = L
};

FieldShape field_shape(int f) {
    switch (f) {
    case GOM_F_ETA_CELL: case GOM_F_ETA_CELL_NEW: return {-1, 0, 0, 0};
    case GOM_F_ETA_NODE: return {-1, 2, 0, 0};
    case GOM_F_WETDRY_NODE: return {-1, 2, 1, 0};
    case GOM_F_UN_FACE: case GOM_F_VN_FACE: case GOM_F_UN_FACE_NEW: case GOM_F_VN_FACE_NEW:
    case GOM_F_UN_ELM: case GOM_F_VN_ELM: case GOM_F_DZ_FACE: case GOM_F_DZ_FACE_NEW:
    case GOM_F_AINVG1: case GOM_F_AINVG2: case GOM_F_AINVDZ1: case GOM_F_AINVDZ2: case GOM_F_KH:
    case GOM_F_SALT_FACE: case GOM_F_TEMP_FACE: case GOM_F_RHO_FACE:
        return {1, 1, 0, 0};
    case GOM_F_ELM_FOOT: case GOM_F_ELM_NEAR_EDGE: return {1, 1, 1, 0};
    case GOM_F_WN_CELL: case GOM_F_WN_CELL_NEW: case GOM_F_DZHALF_CELL: case GOM_F_DZHALF_CELL_NEW:
    case GOM_F_KV:
        return {0, 0, 0, 0};
    case GOM_F_U_NODE: case GOM_F_V_NODE: case GOM_F_W_NODE: case GOM_F_DZHALF_NODE: case GOM_F_DZHALF_NODE_NEW:
        return {0, 2, 0, 0};
    case GOM_F_U_FACE_LEVEL: case GOM_F_V_FACE_LEVEL: case GOM_F_DZHALF_FACE: case GOM_F_DZHALF_FACE_NEW:
    case GOM_F_AV:
        return {0, 1, 0, 0};
    case GOM_F_DZ_CELL: case GOM_F_DZ_CELL_NEW: case GOM_F_SALT_CELL: case GOM_F_SALT_CELL_NEW:
    case GOM_F_TEMP_CELL: case GOM_F_TEMP_CELL_NEW: case GOM_F_RHO_CELL:
        return {1, 0, 0, 0};
    case GOM_F_DZ_NODE: case GOM_F_DZ_NODE_NEW: case GOM_F_SALT_NODE: case GOM_F_TEMP_NODE: case GOM_F_RHO_NODE:
        return {1, 2, 0, 0};
    case GOM_F_NUM_SUB_ELM: return {1, 2, 1, 0};
    case GOM_F_TOP_LAYER_CELL: return {-1, 0, 1, 0};
    case GOM_F_TOP_LAYER_FACE: return {-1, 1, 1, 0};
    case GOM_F_TOP_LAYER_NODE: return {-1, 2, 1, 0};
    case GOM_F_CDB: case GOM_F_GAMMA_B: return {-1, 1, 0, 0};
    case GOM_F_QU_BOUNDARY: return {-1, 3, 0, 0};
    case GOM_F_WIND_STRESS_NORMAL: case GOM_F_WIND_STRESS_TANGNT: case GOM_F_GAMMA_T: return {-1, 1, 0, 0};
    case GOM_F_AIR_P: return {-1, 2, 0, 0};
    case GOM_F_ETA_AT_OB_OLD: case GOM_F_ETA_AT_OB_NEW: return {-1, 4, 0, 0};
    case GOM_F_Q_ADD: return {-1, 3, 0, 0};
    case GOM_F_PHI_SW: return {-1, 0, 0, 0};
    case GOM_F_PHI_SZ: return {1, 0, 0, 0};
    default: return {-2, 0, 0, 0};
    }
}

int64_t field_count(const gom_dims &d, int f, int32_t *eb) {
    FieldShape s = field_shape(f);
    if (s.lo == -2) return -1;
    int64_t n = s.kind == 0 ? d.n_cells : s.kind == 1 ? d.n_faces : s.kind == 2 ? d.n_nodes : s.kind == 3 ? d.n_qb : d.n_ob;
    if (eb) *eb = s.is_int ? 4 : 8;
    if (s.lo == -1) return n;
    return n * (int64_t)(d.n_layers - s.lo + 1);
}

void set_err(gom_ctx *c, int code, int site, int entity, int layer, double value, int kind) {
    OMP_CRITICAL
    if (c->err.code == 0) {
        c->err.code = code;
        c->err.site = site;
        c->err.entity = entity;
        c->err.layer = layer;
        c->err.value = value;
        c->err.kind = kind;
    }
}

// field accessors
A2<double> FD(gom_ctx *c, int f) {
    FieldShape s = field_shape(f);
    return A2<double>{c->fd[f].data(), s.lo, c->L - s.lo + 1};
}
A2<int32_t> FI(gom_ctx *c, int f) {
    FieldShape s = field_shape(f);
    return A2<int32_t>{c->fi[f].data(), s.lo, c->L - s.lo + 1};
}
A1<double> FD1(gom_ctx *c, int f) { return A1<double>{c->fd[f].data()}; }
A1<int32_t> FI1(gom_ctx *c, int f) { return A1<int32_t>{c->fi[f].data()}; }

template <typename T> void copy_in(std::vector<T> &dst, const T *src, size_t n) {
    if (src) dst.assign(src, src + n);
    else dst.assign(n, T(0));
}

// mod_function_library.f90:49-60
inline double calculate_area(double x1, double x2, double x3, double y1, double y2, double y3) {
    return std::fabs((x1 - x3) * (y2 - y3) - (x2 - x3) * (y1 - y3)) / 2.0;
}

// set_geometry_1.f90:48-63
inline int start_end_node(int k, int i, int j) {
    int v = i + j;
    if (v > k) v -= k;
    return v;
}

// tridiagonal_solver.f90:15-61; solution/rhs are (nmax, nc) column-major
bool tridiagonal_solver(int nmax, int n, int nc, const double *a, const double *b, const double *cu,
                        const double *rhs, double *sol, double *gam) {
    if (b[0] == 0.0) return false;
    double den = b[0];
    for (int i = 0; i < nc; ++i) sol[i * nmax + 0] = rhs[i * nmax + 0] / den;
    for (int j = 2; j <= n; ++j) {
        gam[j - 1] = cu[j - 2] / den;
        den = b[j - 1] - a[j - 1] * gam[j - 1];
        if (den == 0.0) return false;
        for (int i = 0; i < nc; ++i)
            sol[i * nmax + j - 1] = (rhs[i * nmax + j - 1] - a[j - 1] * sol[i * nmax + j - 2]) / den;
    }
    for (int j = n - 1; j >= 1; --j)
        for (int i = 0; i < nc; ++i) sol[i * nmax + j - 1] = sol[i * nmax + j - 1] - gam[j] * sol[i * nmax + j];
    return true;
}

// check_intersection.f90:14-50
inline void check_intersection(double x1, double x2, double x3, double x4, double y1, double y2, double y3,
                               double y4, int &iflag, double &xin, double &yin) {
    const double small2 = 0.0;
    iflag = 0;
    double delta = (x2 - x1) * (y3 - y4) - (y2 - y1) * (x3 - x4);
    double delta1 = (x3 - x1) * (y3 - y4) - (y3 - y1) * (x3 - x4);
    double delta2 = (x2 - x1) * (y3 - y1) - (y2 - y1) * (x3 - x1);
    if (delta != 0.0) {
        double tt1 = delta1 / delta;
        double tt2 = delta2 / delta;
        if (tt1 >= -small2 && tt1 <= 1 + small2 && tt2 >= -small2 && tt2 <= 1 + small2) {
            iflag = 1;
            xin = x1 + (x2 - x1) * tt1;
            yin = y1 + (y2 - y1) * tt1;
        }
    }
}

// bilinear_interpolation.f90:8-121; returns 0 or GOM_ELM_BILINEAR
int bilinear_interpolation(double x1, double x2, double x3, double x4, double y1, double y2, double y3,
                           double y4, double x, double y, double &xi, double &eta, double shapef[4]) {
    const double small3 = F(1.e-5f);
    const double small_06 = F(1.e-6f);
    const double b11 = F(1.1f);
    double axi[2], aet[2], bxy[2], root_xi[2], root_et[2];
    double x0 = (x1 + x2 + x3 + x4) / 4.0;
    double y0 = (y1 + y2 + y3 + y4) / 4.0;
    axi[0] = x2 - x1 + x3 - x4;
    axi[1] = y2 - y1 + y3 - y4;
    aet[0] = x3 + x4 - x1 - x2;
    aet[1] = y3 + y4 - y1 - y2;
    bxy[0] = x1 - x2 + x3 - x4;
    bxy[1] = y1 - y2 + y3 - y4;
    double dxi = 2.0 * ((x3 - x4) * (y1 - y2) - (y3 - y4) * (x1 - x2));
    double deta = 2.0 * ((x4 - x1) * (y3 - y2) - (y4 - y1) * (x3 - x2));
    if ((std::fabs(bxy[0]) < small3 && std::fabs(bxy[1]) < small3) ||
        (std::fabs(dxi) < small3 && std::fabs(deta) < small3)) {
        double dd = axi[0] * aet[1] - axi[1] * aet[0];
        if (dd == 0.0) return GOM_ELM_BILINEAR;
        xi = 4.0 * (aet[1] * (x - x0) - aet[0] * (y - y0)) / dd;
        eta = 4.0 * (axi[0] * (y - y0) - axi[1] * (x - x0)) / dd;
    } else if (std::fabs(dxi) < small3 && std::fabs(deta) >= small3) {
        eta = 4.0 * (bxy[1] * (x - x0) - bxy[0] * (y - y0)) / deta;
        double t1 = axi[0] + eta * bxy[0], t2 = axi[1] + eta * bxy[1];
        double dd = t1 * t1 + t2 * t2;
        if (dd == 0.0) return GOM_ELM_BILINEAR;
        xi = ((4.0 * (x - x0) - eta * aet[0]) * (axi[0] + eta * bxy[0]) +
              (4.0 * (y - y0) - eta * aet[1]) * (axi[1] + eta * bxy[1])) / dd;
    } else if (std::fabs(dxi) >= small3 && std::fabs(deta) < small3) {
        xi = 4.0 * (bxy[1] * (x - x0) - bxy[0] * (y - y0)) / dxi;
        double t1 = aet[0] + xi * bxy[0], t2 = aet[1] + xi * bxy[1];
        double dd = t1 * t1 + t2 * t2;
        if (dd == 0.0) return GOM_ELM_BILINEAR;
        eta = ((4.0 * (x - x0) - xi * axi[0]) * (aet[0] + xi * bxy[0]) +
               (4.0 * (y - y0) - xi * axi[1]) * (aet[1] + xi * bxy[1])) / dd;
    } else {
        double beta = aet[1] * axi[0] - aet[0] * axi[1] - 4 * (bxy[1] * (x - x0) - bxy[0] * (y - y0));
        double gamma = 4.0 * (aet[0] * (y - y0) - aet[1] * (x - x0));
        double delta = beta * beta - 4 * gamma * dxi;
        if (delta == 0.0) {
            xi = -beta / 2 / dxi;
            eta = (4.0 * (bxy[1] * (x - x0) - bxy[0] * (y - y0)) - xi * dxi) / deta;
        } else if (delta > 0) {
            root_xi[0] = (-beta + std::sqrt(delta)) / 2 / dxi;
            root_xi[1] = (-beta - std::sqrt(delta)) / 2 / dxi;
            int icount = 0;
            for (int i = 0; i < 2; ++i) {
                root_et[i] = (4 * (bxy[1] * (x - x0) - bxy[0] * (y - y0)) - root_xi[i] * dxi) / deta;
                if (std::fabs(root_xi[i]) <= b11 && std::fabs(root_et[i]) <= b11) {
                    xi = root_xi[i];
                    eta = root_et[i];
                    icount = icount + 1;
                }
            }
            if (icount == 2 && std::fabs(root_xi[0] - root_xi[1]) < small_06) {
                // two equal roots: keep the last one
            } else if (icount != 1) {
                return GOM_ELM_BILINEAR;
            }
        } else {
            return GOM_ELM_BILINEAR;
        }
    }
    if (std::fabs(xi) > b11 || std::fabs(eta) > b11) return GOM_ELM_BILINEAR;
    xi = std::min(1.0, std::max(xi, -1.0));
    eta = std::min(1.0, std::max(eta, -1.0));
    shapef[0] = (1 - xi) * (1 - eta) / 4;
    shapef[1] = (1 + xi) * (1 - eta) / 4;
    shapef[2] = (1 + xi) * (1 + eta) / 4;
    shapef[3] = (1 - xi) * (1 + eta) / 4;
    return 0;
}

// diagnostic for foot parity: (x, y) lies within 1e-12 m of an edge line of element nel, tested
// as cross^2 < (1e-12)^2 * |edge|^2 (cross = edge x (point - edge start))
bool near_edge_line(gom_ctx *c, int nel, double x, double y) {
    int tq = c->tri_or_quad(nel);
    for (int l = 1; l <= tq; ++l) {
        int a = c->nodenum_at_cell(l, nel);
        int b = c->nodenum_at_cell(start_end_node(tq, l, 1), nel);
        double ex = c->x_node(b) - c->x_node(a), ey = c->y_node(b) - c->y_node(a);
        double cr = ex * (y - c->y_node(a)) - ey * (x - c->x_node(a));
        if (cr * cr < 1e-24 * (ex * ex + ey * ey)) return true;
    }
    return false;
}

// ============================================================================================
// search_straight_line.f90:15-399 (i_which_backtrack = 1).  Returns 0 or a GOM_ELM_* site.
int search_straight_line(gom_ctx *c, int &nnel, int &jlev, double time, double x0, double y0, double z0,
                         double &xt, double &yt, double &zt, int &nfl) {
    const double small_06 = F(1.e-6f);
    A1<double> eta_cell = FD1(c, GOM_F_ETA_CELL);
    A1<int32_t> top = FI1(c, GOM_F_TOP_LAYER_CELL);
    auto top_el = [&](int e) { return e == 0 ? 0 : top(e); };
    const double MSL = c->p.msl;
    int L = c->L;
    if (top_el(nnel) == 0 || MSL - c->h_cell(nnel) > MSL + eta_cell(nnel)) return GOM_ELM_START_DRY;
    nfl = 0;
    double trm = time;
    int nel = nnel;
    double area1 = 0.0, area2 = 0.0;
    int tq = c->tri_or_quad(nel);
    for (int l = 1; l <= tq; ++l) {
        int node1 = c->nodenum_at_cell(l, nel);
        int node2 = c->nodenum_at_cell(start_end_node(tq, l, 1), nel);
        area1 = area1 + std::fabs(calculate_area(c->x_node(node1), c->x_node(node2), x0, c->y_node(node1),
                                                 c->y_node(node2), y0));
        area2 = area2 + std::fabs(calculate_area(c->x_node(node1), c->x_node(node2), xt, c->y_node(node1),
                                                 c->y_node(node2), yt));
    }
    double ae = std::fabs(area1 - c->area(nel)) / c->area(nel);
    if (ae > small_06) return GOM_ELM_START_OUTSIDE;
    ae = std::fabs(area2 - c->area(nel)) / c->area(nel);
    if (ae < small_06) {
        nnel = nel;
    } else {
        const double c1 = 1.0 - 1.0e-4;
        double xcg = c1 * x0 + 1.0e-4 * c->x_cell(nel);
        double ycg = c1 * y0 + 1.0e-4 * c->y_cell(nel);
        double pathl = std::sqrt((xt - xcg) * (xt - xcg) + (yt - ycg) * (yt - ycg));
        if ((xcg == xt && ycg == yt) || pathl == 0.0) return GOM_ELM_ZERO_PATH;
        int iflag = 0, nel_j = 0;
        double xin = 0, yin = 0;
        for (int l = 1; l <= tq; ++l) {
            int jd1 = c->nodenum_at_cell(start_end_node(tq, l, 1), nel);
            int jd2 = c->nodenum_at_cell(start_end_node(tq, l, 2), nel);
            check_intersection(xcg, xt, c->x_node(jd1), c->x_node(jd2), ycg, yt, c->y_node(jd1), c->y_node(jd2),
                               iflag, xin, yin);
            if (iflag == 1) {
                nel_j = l;
                break;
            }
        }
        if (iflag == 0) return GOM_ELM_NO_FIRST_EDGE;
        double zin = z0;
        int iteration = 0;
        for (;;) {
            iteration = iteration + 1;
            if (iteration > 1000) {
                nfl = 1;
                xt = xin;
                yt = yin;
                zt = zin;
                nnel = nel;
                break;
            }
            int tqn = c->tri_or_quad(nel);
            int md1 = c->nodenum_at_cell(start_end_node(tqn, nel_j, 1), nel);
            int md2 = c->nodenum_at_cell(start_end_node(tqn, nel_j, 2), nel);
            double dist = std::sqrt((xin - xt) * (xin - xt) + (yin - yt) * (yin - yt));
            if (dist / pathl > 1.0 + 1.0e-4) return GOM_ELM_OVERSHOOT;
            zin = zt - dist / pathl * (zt - zin);
            trm = trm * dist / pathl;
            pathl = std::sqrt((xin - xt) * (xin - xt) + (yin - yt) * (yin - yt));
            if (pathl == 0.0 || trm == 0.0) return GOM_ELM_ZERO_REMAIN;
            int iter_temp = 0;
            int adjc = c->adj_cellnum_at_cell(nel_j, nel);
            if (adjc == 0 || top_el(adjc) == 0) {
                iter_temp = 1;
                int isd = c->facenum_at_cell(nel_j, nel);
                if (c->nodenum_at_face(1, isd) + c->nodenum_at_face(2, isd) != md1 + md2) return GOM_ELM_FACE_MISMATCH;
                xin = c1 * xin + 1.0e-4 * c->x_cell(nel);
                yin = c1 * yin + 1.0e-4 * c->y_cell(nel);
                nfl = 1;
                xt = xin;
                yt = yin;
                zt = zin;
                nnel = nel;
                break;
            }
            if (iter_temp == 0) nel = adjc;
            area1 = 0.0;
            tqn = c->tri_or_quad(nel);
            for (int l = 1; l <= tqn; ++l) {
                int k1 = c->nodenum_at_cell(l, nel);
                int k2 = c->nodenum_at_cell(start_end_node(tqn, l, 1), nel);
                area1 = area1 + std::fabs(calculate_area(c->x_node(k1), c->x_node(k2), xt, c->y_node(k1),
                                                         c->y_node(k2), yt));
            }
            ae = std::fabs(area1 - c->area(nel)) / c->area(nel);
            if (ae < small_06) {
                nnel = nel;
                break;
            }
            bool found = false;
            for (int l = 1; l <= tqn; ++l) {
                int jd1 = c->nodenum_at_cell(start_end_node(tqn, l, 1), nel);
                int jd2 = c->nodenum_at_cell(start_end_node(tqn, l, 2), nel);
                if ((jd1 == md1 && jd2 == md2) || (jd2 == md1 && jd1 == md2)) continue;
                check_intersection(xcg, xt, c->x_node(jd1), c->x_node(jd2), ycg, yt, c->y_node(jd1),
                                   c->y_node(jd2), iflag, xin, yin);
                if (iflag == 1) {
                    nel_j = l;
                    found = true;
                    break;
                }
            }
            if (found) continue;
            if (iflag == 0) return GOM_ELM_NO_NEXT_EDGE;
        }
    }
    if (top_el(nnel) == 0 || MSL - c->h_cell(nnel) > MSL + eta_cell(nnel)) return GOM_ELM_END_DRY;
    zt = std::min(std::max(zt, MSL - c->h_cell(nnel)), MSL + eta_cell(nnel));
    if (zt <= c->zl(0)) return GOM_ELM_Z_RANGE;
    if (zt > c->zl(L)) return GOM_ELM_Z_RANGE;
    for (int k = 0; k <= L - 1; ++k) {
        if (zt > c->zl(k) && zt <= c->zl(k + 1)) {
            jlev = k + 1;
            break;
        }
    }
    jlev = std::min(std::max(jlev, (int)c->bottom_layer_at_element(nnel)), (int)top_el(nnel));
    return 0;
}

// ELM_backtrace_v1.f90:15-200 (i_which_backtrack = 1).  Returns 0 or a GOM_ELM_* site.
// the last substep's foot, surface or level height above it and interpolation weights, which the
// transport mode of ELM_backtrace_v1.f90:216-473 interpolates the tracers with
struct ElmFinal {
    double xt = 0.0, yt = 0.0, zt = 0.0, zup = 0.0;
    double staint[4] = {0.0, 0.0, 0.0, 0.0};
};

int elm_backtrace(gom_ctx *c, int bt_step, double bt_dt, double &uuint, double &vvint, double &wwint,
                  double &x0, double &y0, double &z0, int &nnel, int &jlev, int &near_edge, ElmFinal *fin = nullptr) {
    const double small_06 = F(1.e-6f);
    A2<double> u_node = FD(c, GOM_F_U_NODE), v_node = FD(c, GOM_F_V_NODE), w_node = FD(c, GOM_F_W_NODE);
    A2<double> dz_cell = FD(c, GOM_F_DZ_CELL);
    A1<double> eta_cell = FD1(c, GOM_F_ETA_CELL);
    A1<int32_t> top = FI1(c, GOM_F_TOP_LAYER_CELL);
    double xt = 0, yt = 0, zt = 0;
    double vxl[4][2], vyl[4][2], vzl[4][2], vxn[4], vyn[4], vzn[4], staint[4];
    for (int idt = 1; idt <= bt_step; ++idt) {
        xt = x0 - bt_dt * uuint;
        yt = y0 - bt_dt * vvint;
        zt = z0 - bt_dt * wwint;
        int nfl = 0;
        int e = search_straight_line(c, nnel, jlev, bt_dt, x0, y0, z0, xt, yt, zt, nfl);
        if (e) return e;
        int tq = c->tri_or_quad(nnel);
        for (int l = 1; l <= tq; ++l) {
            int nd = c->nodenum_at_cell(l, nnel);
            for (int k2 = 1; k2 <= 2; ++k2) {
                int lev = jlev + k2 - 2;
                vxl[l - 1][k2 - 1] = u_node(lev, nd);
                vyl[l - 1][k2 - 1] = v_node(lev, nd);
                vzl[l - 1][k2 - 1] = w_node(lev, nd);
            }
        }
        double zup = (jlev == top(nnel)) ? c->p.msl + eta_cell(nnel) : c->zl(jlev);
        if (zt > zup) return GOM_ELM_Z_ABOVE;
        double zrat = (zup - zt) / dz_cell(jlev, nnel);
        for (int l = 1; l <= tq; ++l) {
            vxn[l - 1] = vxl[l - 1][1] * (1 - zrat) + vxl[l - 1][0] * zrat;
            vyn[l - 1] = vyl[l - 1][1] * (1 - zrat) + vyl[l - 1][0] * zrat;
            vzn[l - 1] = vzl[l - 1][1] * (1 - zrat) + vzl[l - 1][0] * zrat;
        }
        int node1 = c->nodenum_at_cell(1, nnel), node2 = c->nodenum_at_cell(2, nnel),
            node3 = c->nodenum_at_cell(3, nnel);
        if (tq == 3) {
            double ar = c->area(nnel);
            staint[0] = calculate_area(xt, c->x_node(node2), c->x_node(node3), yt, c->y_node(node2), c->y_node(node3)) / ar;
            staint[1] = calculate_area(c->x_node(node1), xt, c->x_node(node3), c->y_node(node1), yt, c->y_node(node3)) / ar;
            staint[2] = calculate_area(c->x_node(node1), c->x_node(node2), xt, c->y_node(node1), c->y_node(node2), yt) / ar;
            staint[0] = std::max(0.0, std::min(1.0, staint[0]));
            staint[1] = std::max(0.0, std::min(1.0, staint[1]));
            if (staint[0] + staint[1] > 1) {
                staint[2] = 0;
                staint[1] = 1.0 - staint[0];
            } else {
                staint[2] = 1.0 - staint[0] - staint[1];
            }
        } else {
            int node4 = c->nodenum_at_cell(4, nnel);
            double aa1 = calculate_area(c->x_node(node1), c->x_node(node2), xt, c->y_node(node1), c->y_node(node2), yt);
            double aa2 = calculate_area(c->x_node(node2), c->x_node(node3), xt, c->y_node(node2), c->y_node(node3), yt);
            double aa3 = calculate_area(c->x_node(node3), c->x_node(node4), xt, c->y_node(node3), c->y_node(node4), yt);
            double aa4 = calculate_area(c->x_node(node4), c->x_node(node1), xt, c->y_node(node4), c->y_node(node1), yt);
            double aa = std::fabs(aa1) + std::fabs(aa2) + std::fabs(aa3) + std::fabs(aa4);
            if (std::fabs(aa - c->area(nnel)) / c->area(nnel) > small_06) return GOM_ELM_QUAD_OUTSIDE;
            double csi, etta;
            int b = bilinear_interpolation(c->x_node(node1), c->x_node(node2), c->x_node(node3), c->x_node(node4),
                                           c->y_node(node1), c->y_node(node2), c->y_node(node3), c->y_node(node4), xt,
                                           yt, csi, etta, staint);
            if (b) return b;
        }
        uuint = 0.0;
        vvint = 0.0;
        wwint = 0.0;
        for (int j = 1; j <= tq; ++j) {
            uuint = uuint + vxn[j - 1] * staint[j - 1];
            vvint = vvint + vyn[j - 1] * staint[j - 1];
            wwint = wwint + vzn[j - 1] * staint[j - 1];
        }
        if (near_edge_line(c, nnel, xt, yt)) near_edge = 1;
        if (fin) {
            fin->xt = xt;
            fin->yt = yt;
            fin->zt = zt;
            fin->zup = zup;
            for (int l = 0; l < 4; ++l) fin->staint[l] = staint[l];
        }
        if (nfl == 1) break;
        x0 = xt;
        y0 = yt;
        z0 = zt;
    }
    return 0;
}

// ELM_backtrace_v1.f90:216-473 (i_which_backtrack = 2): temperature and salinity at the foot.
// Open-boundary and river cells take the boundary concentrations; otherwise a vertical anchor
// at the layer middle picks two levels of node and face values, and the foot is located in the
// element's sub-elements (triangles: three corner triangles and the central one of the face
// midpoints; quads: four quads of a node, two face midpoints and the cell centre) for an
// interpolation of node and face values; with a dry node the mean of the wet nodes stands.
// Returns 0 or a GOM_ELM_* site.
int elm_tracer_at_foot(gom_ctx *c, const ElmFinal &fin, int nnel, int jlev, double &ttint, double &ssint) {
    const double small_06 = F(1.e-6f);
    A2<double> dz_cell = FD(c, GOM_F_DZ_CELL), dzh_c = FD(c, GOM_F_DZHALF_CELL);
    A2<double> salt_node = FD(c, GOM_F_SALT_NODE), temp_node = FD(c, GOM_F_TEMP_NODE),
               salt_face = FD(c, GOM_F_SALT_FACE), temp_face = FD(c, GOM_F_TEMP_FACE);
    A1<int32_t> top = FI1(c, GOM_F_TOP_LAYER_CELL), top_n = FI1(c, GOM_F_TOP_LAYER_NODE),
                top_f = FI1(c, GOM_F_TOP_LAYER_FACE);
    const double xt = fin.xt, yt = fin.yt, zt = fin.zt, zup = fin.zup;
    const int ibnd1 = c->ob_element_flag(nnel), ibnd2 = c->Qb_element_flag(nnel);
    ttint = 0.0;
    ssint = 0.0;
    if (ibnd1 > 0) {
        // salt_at_obck(jlev, ibnd1): the boundary concentration, the same in every layer
        ssint = c->con_at_ob[(size_t)0 * c->NOB + (ibnd1 - 1)];
        ttint = c->con_at_ob[(size_t)1 * c->NOB + (ibnd1 - 1)];
        return 0;
    }
    if (ibnd2 > 0) {
        ssint = c->con_at_qb[(size_t)0 * c->NQB + (ibnd2 - 1)];
        ttint = c->con_at_qb[(size_t)1 * c->NQB + (ibnd2 - 1)];
        return 0;
    }
    const double zanchor = zup - dz_cell(jlev, nnel) * 0.5;
    int k1, k2;
    double zrat2;
    if (jlev == top(nnel) && zt > zanchor) {
        k1 = jlev;
        k2 = jlev;
        zrat2 = 0.5;
    } else if (zt > zanchor) {
        k1 = jlev;
        k2 = jlev + 1;
        zrat2 = (zt - zanchor) / dzh_c(jlev, nnel);
    } else {
        k1 = std::max(jlev - 1, (int)c->bottom_layer_at_element(nnel));
        k2 = jlev;
        zrat2 = 1.0 - (zanchor - zt) / dzh_c(k1, nnel);
    }
    zrat2 = std::max(0.0, std::min(1.0, zrat2));
    const int tq = c->tri_or_quad(nnel);
    int icount = 0;
    double ta = 0.0, sa = 0.0, t_xi[4] = {0, 0, 0, 0}, s_xi[4] = {0, 0, 0, 0};
    for (int l = 1; l <= tq; ++l) {
        int nd = c->nodenum_at_cell(l, nnel);
        if (top_n(nd) != 0) {
            icount = icount + 1;
            t_xi[l - 1] = temp_node(k1, nd) * (1 - zrat2) + temp_node(k2, nd) * zrat2;
            s_xi[l - 1] = salt_node(k1, nd) * (1 - zrat2) + salt_node(k2, nd) * zrat2;
            ta = ta + t_xi[l - 1];
            sa = sa + s_xi[l - 1];
        }
    }
    if (icount == 0) return GOM_ELM_ALL_DRY;
    if (icount != tq) {
        ta = ta / icount;
        sa = sa / icount;
        ttint = ta;
        ssint = sa;
    } else {
        ta = ta / icount;
        sa = sa / icount;
        ttint = 0.0;
        ssint = 0.0;
        for (int l = 1; l <= tq; ++l) {
            ttint = ttint + t_xi[l - 1] * fin.staint[l - 1];
            ssint = ssint + s_xi[l - 1] * fin.staint[l - 1];
        }
    }
    auto lev = [&](const A2<double> &a, int e) { return a(k1, e) * (1 - zrat2) + a(k2, e) * zrat2; };
    const double ar = c->area(nnel);
    int index_1 = 0;
    if (tq == 3) {
        for (int l = 1; l <= 4; ++l) {
            double aa1, aa2, aa3;
            int n1 = 0, f1 = 0, f2, f3;
            if (l <= 3) {
                n1 = c->nodenum_at_cell(l, nnel);
                f2 = c->facenum_at_cell(start_end_node(tq, l, 2), nnel);
                f3 = c->facenum_at_cell(start_end_node(tq, l, 1), nnel);
                aa1 = calculate_area(xt, c->x_face(f2), c->x_face(f3), yt, c->y_face(f2), c->y_face(f3));
                aa2 = calculate_area(c->x_node(n1), xt, c->x_face(f3), c->y_node(n1), yt, c->y_face(f3));
                aa3 = calculate_area(c->x_node(n1), c->x_face(f2), xt, c->y_node(n1), c->y_face(f2), yt);
            } else {
                f1 = c->facenum_at_cell(1, nnel);
                f2 = c->facenum_at_cell(2, nnel);
                f3 = c->facenum_at_cell(3, nnel);
                aa1 = calculate_area(xt, c->x_face(f2), c->x_face(f3), yt, c->y_face(f2), c->y_face(f3));
                aa2 = calculate_area(c->x_face(f1), xt, c->x_face(f3), c->y_face(f1), yt, c->y_face(f3));
                aa3 = calculate_area(c->x_face(f1), c->x_face(f2), xt, c->y_face(f1), c->y_face(f2), yt);
            }
            double aa = std::fabs(aa1) + std::fabs(aa2) + std::fabs(aa3);
            double subrat = std::fabs(aa - ar / 4) * 4 / ar;
            if (subrat < 100 * small_06) {
                index_1 = 1;
                double sig[3];
                sig[0] = aa1 * 4 / ar;
                sig[1] = aa2 * 4 / ar;
                sig[0] = std::max(0.0, std::min(1.0, sig[0]));
                sig[1] = std::max(0.0, std::min(1.0, sig[1]));
                if (sig[0] + sig[1] > 1) {
                    sig[2] = 0;
                    sig[1] = 1 - sig[0];
                } else {
                    sig[2] = 1 - sig[0] - sig[1];
                }
                bool wet = l <= 3 ? (top_n(n1) != 0 && top_f(f2) != 0 && top_f(f3) != 0)
                                  : (top_f(f1) != 0 && top_f(f2) != 0 && top_f(f3) != 0);
                if (wet) {
                    double tx[3], sx[3];
                    tx[0] = l <= 3 ? lev(temp_node, n1) : lev(temp_face, f1);
                    sx[0] = l <= 3 ? lev(salt_node, n1) : lev(salt_face, f1);
                    tx[1] = lev(temp_face, f2);
                    tx[2] = lev(temp_face, f3);
                    sx[1] = lev(salt_face, f2);
                    sx[2] = lev(salt_face, f3);
                    ttint = tx[0] * sig[0] + tx[1] * sig[1] + tx[2] * sig[2];
                    ssint = sx[0] * sig[0] + sx[1] * sig[1] + sx[2] * sig[2];
                    break;
                }
            }
        }
    } else {
        for (int l = 1; l <= 4; ++l) {
            int n1 = c->nodenum_at_cell(l, nnel);
            int f2 = c->facenum_at_cell(start_end_node(tq, l, 3), nnel);
            int f4 = c->facenum_at_cell(start_end_node(tq, l, 2), nnel);
            const double xc = c->x_cell(nnel), yc = c->y_cell(nnel);
            double aa1 = calculate_area(c->x_node(n1), c->x_face(f2), xt, c->y_node(n1), c->y_face(f2), yt);
            double aa2 = calculate_area(c->x_face(f2), xc, xt, c->y_face(f2), yc, yt);
            double aa3 = calculate_area(xc, c->x_face(f4), xt, yc, c->y_face(f4), yt);
            double aa4 = calculate_area(c->x_face(f4), c->x_node(n1), xt, c->y_face(f4), c->y_node(n1), yt);
            double bb1 = calculate_area(c->x_node(n1), c->x_face(f2), c->x_face(f4), c->y_node(n1), c->y_face(f2),
                                        c->y_face(f4));
            double bb2 = calculate_area(c->x_face(f2), xc, c->x_face(f4), c->y_face(f2), yc, c->y_face(f4));
            if (bb1 <= 0 || bb2 <= 0) return GOM_ELM_NEG_SUBELEMENT;
            double bb = bb1 + bb2;
            double aa = std::fabs(aa1) + std::fabs(aa2) + std::fabs(aa3) + std::fabs(aa4);
            double subrat = std::fabs(aa - bb) / bb;
            if (subrat < 4.0 * small_06) {
                index_1 = 1;
                double csi, etta, st4[4];
                int b = bilinear_interpolation(c->x_node(n1), c->x_face(f2), xc, c->x_face(f4), c->y_node(n1),
                                               c->y_face(f2), yc, c->y_face(f4), xt, yt, csi, etta, st4);
                if (b) return b;
                if (top_n(n1) != 0 && top_f(f2) != 0 && top_f(f4) != 0) {
                    double tx[4] = {lev(temp_node, n1), lev(temp_face, f2), ta, lev(temp_face, f4)};
                    double sx[4] = {lev(salt_node, n1), lev(salt_face, f2), sa, lev(salt_face, f4)};
                    ttint = 0.0;
                    ssint = 0.0;
                    for (int j = 0; j < 4; ++j) {
                        ttint = ttint + tx[j] * st4[j];
                        ssint = ssint + sx[j] * st4[j];
                    }
                }
            }
        }
    }
    if (index_1 == 0) return GOM_ELM_NO_SUBELEMENT;
    return 0;
}

}  // namespace

// ============================================================================================
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
    if (!dims) return GOM_E_ARG;
    int32_t eb = 0;
    int64_t n = field_count(*dims, field, &eb);
    if (n < 0) return GOM_E_ARG;
    if (count) *count = n;
    if (elem_bytes) *elem_bytes = eb;
    return GOM_OK;
}

int gom_create(const gom_dims *dims, const gom_params *params, const gom_geom *g, gom_ctx **out) {
    if (!dims || !params || !g || !out) return GOM_E_ARG;
    const gom_dims &d = *dims;
    if (d.n_cells <= 0 || d.n_faces <= 0 || d.n_nodes <= 0 || d.n_layers <= 0 || d.n_layers > GOM_ORACLE_MAXL ||
        d.max_nb <= 0 || d.n_ob < 0 || d.n_qb < 0)
        return GOM_E_ARG;
    if (params->transport_flag && params->is_salt == 0 && params->is_temp == 1) return GOM_E_ARG;
    if (params->transport_solver < 0 || params->transport_solver > 2) return GOM_E_ARG;
    gom_ctx *c = new gom_ctx();
    c->d = d;
    c->p = *params;
    c->L = d.n_layers;
    c->NC = d.n_cells;
    c->NF = d.n_faces;
    c->NN = d.n_nodes;
    c->NB = d.max_nb;
    c->NOB = d.n_ob;
    c->NQB = d.n_qb;
    size_t NC = d.n_cells, NF = d.n_faces, NN = d.n_nodes, NB = d.max_nb, L = d.n_layers;
    copy_in(c->g_x_node, g->x_node, NN);
    copy_in(c->g_y_node, g->y_node, NN);
    copy_in(c->g_h_node, g->h_node, NN);
    copy_in(c->g_adj_cells_at_node, g->adj_cells_at_node, NN);
    copy_in(c->g_adj_cellnum_at_node, g->adj_cellnum_at_node, NB * NN);
    copy_in(c->g_node_count_each_element, g->node_count_each_element, NB * NN);
    copy_in(c->g_adj_nodes_at_node, g->adj_nodes_at_node, NN);
    copy_in(c->g_adj_nodenum_at_node, g->adj_nodenum_at_node, (NB + 1) * NN);
    copy_in(c->g_bottom_node, g->bottom_layer_at_node, NN);
    copy_in(c->g_initial_wetdry_node, g->initial_wetdry_node, NN);
    copy_in(c->g_x_cell, g->x_cell, NC);
    copy_in(c->g_y_cell, g->y_cell, NC);
    copy_in(c->g_h_cell, g->h_cell, NC);
    copy_in(c->g_area, g->area, NC);
    copy_in(c->g_tri_or_quad, g->tri_or_quad, NC);
    copy_in(c->g_nodenum_at_cell, g->nodenum_at_cell, 4 * NC);
    copy_in(c->g_facenum_at_cell, g->facenum_at_cell, 4 * NC);
    copy_in(c->g_adj_cellnum_at_cell, g->adj_cellnum_at_cell, 4 * NC);
    copy_in(c->g_sign_in_outflow, g->sign_in_outflow, 4 * NC);
    copy_in(c->g_bottom_cell, g->bottom_layer_at_element, NC);
    copy_in(c->g_ob_element_flag, g->ob_element_flag, NC);
    copy_in(c->g_qb_element_flag, g->qb_element_flag, NC);
    copy_in(c->g_x_face, g->x_face, NF);
    copy_in(c->g_y_face, g->y_face, NF);
    copy_in(c->g_h_face, g->h_face, NF);
    copy_in(c->g_face_length, g->face_length, NF);
    copy_in(c->g_delta_j, g->delta_j, NF);
    copy_in(c->g_cos_theta, g->cos_theta, NF);
    copy_in(c->g_sin_theta, g->sin_theta, NF);
    copy_in(c->g_cos_theta2, g->cos_theta2, NF);
    copy_in(c->g_sin_theta2, g->sin_theta2, NF);
    copy_in(c->g_adj_cellnum_at_face, g->adj_cellnum_at_face, 2 * NF);
    copy_in(c->g_nodenum_at_face, g->nodenum_at_face, 2 * NF);
    copy_in(c->g_bottom_face, g->bottom_layer_at_face, NF);
    copy_in(c->g_boundary_type_of_face, g->boundary_type_of_face, NF);
    copy_in(c->g_isflowside3, g->isflowside3, NF);
    copy_in(c->g_coriolis, g->coriolis_factor, NF);
    copy_in(c->g_manning, g->manning, NF);
    copy_in(c->g_bf_height, g->bf_height, NF);
    copy_in(c->g_ob_cell_id, g->ob_cell_id, (size_t)d.n_ob);
    copy_in(c->g_qb_cell, g->qb_cell, (size_t)d.n_qb);
    copy_in(c->g_qb_face, g->qb_face, (size_t)d.n_qb);
    copy_in(c->g_z_level, g->z_level, L + 1);
    copy_in(c->g_delta_z, g->delta_z, L);
    if (d.n_runs > 1) {
        if (!g->run_cell_start) {
            delete c;
            return GOM_E_ARG;
        }
        copy_in(c->run_cell_start, g->run_cell_start, (size_t)d.n_runs + 1);
        if (!g->run_face_start) {
            delete c;
            return GOM_E_ARG;
        }
        copy_in(c->run_face_start, g->run_face_start, (size_t)d.n_runs + 1);
        if (g->run_node_start) copy_in(c->run_node_start, g->run_node_start, (size_t)d.n_runs + 1);
        else c->run_node_start = {0, d.n_nodes};
    } else {
        c->run_cell_start = {0, d.n_cells};
        c->run_face_start = {0, d.n_faces};
        c->run_node_start = {0, d.n_nodes};
    }

    c->x_node.p = c->g_x_node.data();
    c->y_node.p = c->g_y_node.data();
    c->h_node.p = c->g_h_node.data();
    c->x_cell.p = c->g_x_cell.data();
    c->y_cell.p = c->g_y_cell.data();
    c->h_cell.p = c->g_h_cell.data();
    c->area.p = c->g_area.data();
    c->x_face.p = c->g_x_face.data();
    c->y_face.p = c->g_y_face.data();
    c->h_face.p = c->g_h_face.data();
    c->face_length.p = c->g_face_length.data();
    c->delta_j.p = c->g_delta_j.data();
    c->cos_theta.p = c->g_cos_theta.data();
    c->sin_theta.p = c->g_sin_theta.data();
    c->cos_theta2.p = c->g_cos_theta2.data();
    c->sin_theta2.p = c->g_sin_theta2.data();
    c->coriolis_factor.p = c->g_coriolis.data();
    c->manning.p = c->g_manning.data();
    c->bf_height.p = c->g_bf_height.data();
    c->delta_z.p = c->g_delta_z.data();
    c->adj_cells_at_node.p = c->g_adj_cells_at_node.data();
    c->adj_nodes_at_node.p = c->g_adj_nodes_at_node.data();
    c->bottom_layer_at_node.p = c->g_bottom_node.data();
    c->initial_wetdry_node.p = c->g_initial_wetdry_node.data();
    c->tri_or_quad.p = c->g_tri_or_quad.data();
    c->bottom_layer_at_element.p = c->g_bottom_cell.data();
    c->ob_element_flag.p = c->g_ob_element_flag.data();
    c->Qb_element_flag.p = c->g_qb_element_flag.data();
    c->bottom_layer_at_face.p = c->g_bottom_face.data();
    c->boundary_type_of_face.p = c->g_boundary_type_of_face.data();
    c->isflowside3.p = c->g_isflowside3.data();
    c->ob_cell_id.p = c->g_ob_cell_id.data();
    c->qb_cell.p = c->g_qb_cell.data();
    c->qb_face.p = c->g_qb_face.data();
    c->adj_cellnum_at_node = A2<int32_t>{c->g_adj_cellnum_at_node.data(), 1, (int)NB};
    c->node_count_each_element = A2<int32_t>{c->g_node_count_each_element.data(), 1, (int)NB};
    c->adj_nodenum_at_node = A2<int32_t>{c->g_adj_nodenum_at_node.data(), 0, (int)NB + 1};
    c->nodenum_at_cell = A2<int32_t>{c->g_nodenum_at_cell.data(), 1, 4};
    c->facenum_at_cell = A2<int32_t>{c->g_facenum_at_cell.data(), 1, 4};
    c->adj_cellnum_at_cell = A2<int32_t>{c->g_adj_cellnum_at_cell.data(), 1, 4};
    c->sign_in_outflow = A2<int32_t>{c->g_sign_in_outflow.data(), 1, 4};
    c->adj_cellnum_at_face = A2<int32_t>{c->g_adj_cellnum_at_face.data(), 1, 2};
    c->nodenum_at_face = A2<int32_t>{c->g_nodenum_at_face.data(), 1, 2};

    for (int f = 1; f < GOM_F_COUNT; ++f) {
        int32_t eb = 0;
        int64_t n = field_count(d, f, &eb);
        if (n < 0) continue;
        if (eb == 4) c->fi[f].assign((size_t)n, 0);
        else c->fd[f].assign((size_t)n, 0.0);
    }
    c->eta_at_ob_old.assign(d.n_ob, 0.0);
    c->eta_at_ob_new.assign(d.n_ob, 0.0);
    c->q_add.assign(d.n_qb, 0.0);
    c->wind_stress_normal.assign(NF, 0.0);
    c->wind_stress_tangnt.assign(NF, 0.0);
    c->gamma_t.assign(NF, 0.0);
    c->air_p.assign(NN, 0.0);
    int nt = std::max(1, params->trans_sub_iter);
    c->con_at_ob.assign((size_t)d.n_ob * 2 * nt, 0.0);
    c->con_at_qb.assign((size_t)d.n_qb * 2 * nt, 0.0);
    c->phi_sw.assign(NC, 0.0);
    c->phi_sz.assign((size_t)L * NC, 0.0);
    *out = c;
    return GOM_OK;
}

void gom_destroy(gom_ctx *ctx) { delete ctx; }

// forcing arrays exposed as fields
std::vector<double> *forcing_field(gom_ctx *c, int field) {
    switch (field) {
    case GOM_F_WIND_STRESS_NORMAL: return &c->wind_stress_normal;
    case GOM_F_WIND_STRESS_TANGNT: return &c->wind_stress_tangnt;
    case GOM_F_GAMMA_T: return &c->gamma_t;
    case GOM_F_AIR_P: return &c->air_p;
    case GOM_F_ETA_AT_OB_OLD: return &c->eta_at_ob_old;
    case GOM_F_ETA_AT_OB_NEW: return &c->eta_at_ob_new;
    case GOM_F_Q_ADD: return &c->q_add;
    case GOM_F_PHI_SW: return &c->phi_sw;
    case GOM_F_PHI_SZ: return &c->phi_sz;
    default: return nullptr;
    }
}

int gom_set_field(gom_ctx *c, int field, const void *host, int64_t count) {
    if (!c || !host) return GOM_E_ARG;
    int32_t eb = 0;
    int64_t n = field_count(c->d, field, &eb);
    if (n < 0 || n != count) return GOM_E_ARG;
    if (std::vector<double> *v = forcing_field(c, field)) {
        std::memcpy(v->data(), host, (size_t)n * 8);
        return GOM_OK;
    }
    if (eb == 4) std::memcpy(c->fi[field].data(), host, (size_t)n * 4);
    else std::memcpy(c->fd[field].data(), host, (size_t)n * 8);
    return GOM_OK;
}

int gom_get_field(gom_ctx *c, int field, void *host, int64_t count) {
    if (!c || !host) return GOM_E_ARG;
    int32_t eb = 0;
    int64_t n = field_count(c->d, field, &eb);
    if (n < 0 || n != count) return GOM_E_ARG;
    if (std::vector<double> *v = forcing_field(c, field)) {
        std::memcpy(host, v->data(), (size_t)n * 8);
        return GOM_OK;
    }
    if (eb == 4) std::memcpy(host, c->fi[field].data(), (size_t)n * 4);
    else std::memcpy(host, c->fd[field].data(), (size_t)n * 8);
    return GOM_OK;
}

int gom_set_forcing(gom_ctx *c, const gom_forcing *f) {
    if (!c || !f) return GOM_E_ARG;
    c->elapsed_time = f->elapsed_time;
    c->spinup_tide = f->spinup_tide;
    c->spinup_baroclinic = f->spinup_baroclinic;
    int nt = std::max(1, c->p.trans_sub_iter);
    auto up = [](std::vector<double> &v, const double *s) {
        if (s) std::memcpy(v.data(), s, v.size() * sizeof(double));
    };
    up(c->eta_at_ob_old, f->eta_at_ob_old);
    up(c->eta_at_ob_new, f->eta_at_ob_new);
    up(c->q_add, f->q_add);
    up(c->wind_stress_normal, f->wind_stress_normal);
    up(c->wind_stress_tangnt, f->wind_stress_tangnt);
    up(c->gamma_t, f->gamma_t);
    up(c->air_p, f->air_p);
    up(c->con_at_ob, f->con_at_ob);
    up(c->con_at_qb, f->con_at_qb);
    up(c->phi_sw, f->phi_sw);
    up(c->phi_sz, f->phi_sz);
    (void)nt;
    return GOM_OK;
}

// the CPU restatement takes all forcing from the host, and its initial state from the host
int gom_set_storms(gom_ctx *c, int32_t, const gom_storm *, double) { return c ? GOM_E_ARG : GOM_E_ARG; }

// ---------------------------------------------------------------------------- boundary series
// compute_boundary_eta.f90:22-125 (types 1 and 2), calculate_Q.f90:21-75, setup_spinup.f90:12-31 and
// the boundary concentrations of solve_transport_equation_v19.f90:229-382, with a time outside a
// series keeping that entry's previous value (the reference's value there is undefined)
namespace {
bool find_neighbour_nodes(gom_ctx *c);   // hurricane method 2 (defined with the series forcing)
}  // namespace

int gom_set_boundary_series(gom_ctx *c, const gom_boundary_series *bs) {
    if (!c || !bs || c->d.n_runs > 1) return GOM_E_ARG;
    const gom_series *sets[4] = {&bs->eta, &bs->q, &bs->salt, &bs->temp};
    // the argument rules: series starts from 0 and never decrease, times never decrease within a
    // series, ids within 0..n (0 = none), eta types -1..3, Q method 1 or 2
    for (const gom_series *sr : sets) {
        if (sr->n_series < 0) return GOM_E_ARG;
        if (sr->n_series == 0) continue;
        if (!sr->start || !sr->time || !sr->value || sr->start[0] != 0) return GOM_E_ARG;
        for (int k = 0; k < sr->n_series; ++k) {
            if (sr->start[k + 1] < sr->start[k]) return GOM_E_ARG;
            for (int q = sr->start[k] + 1; q < sr->start[k + 1]; ++q)
                if (!(sr->time[q] >= sr->time[q - 1])) return GOM_E_ARG;
        }
    }
    const int nh = bs->n_harmonic;
    if (nh < 0 || (nh > 0 && (!bs->harmonic_start || !bs->amplitude || !bs->period_h || !bs->nodal || !bs->eq_arg ||
                              !bs->phase || !bs->phase_shift || bs->harmonic_start[0] != 0)))
        return GOM_E_ARG;
    for (int k = 0; k < nh; ++k)
        if (bs->harmonic_start[k + 1] < bs->harmonic_start[k]) return GOM_E_ARG;
    auto ids_ok = [](const int32_t *ids, int n, int limit) {
        if (n > 0 && !ids) return false;
        for (int i = 0; i < n; ++i)
            if (ids[i] < 0 || ids[i] > limit) return false;
        return true;
    };
    if (c->NOB > 0 && !bs->ob_eta_type) return GOM_E_ARG;
    for (int i = 0; i < c->NOB; ++i)
        if (bs->ob_eta_type[i] < -1 || bs->ob_eta_type[i] > 3) return GOM_E_ARG;   // read_main_inp.f90:460-464
    if (!ids_ok(bs->ob_harmonic_id, c->NOB, nh) ||
        !ids_ok(bs->ob_eta_id, c->NOB, bs->eta.n_series) || !ids_ok(bs->ob_salt_id, c->NOB, bs->salt.n_series) ||
        !ids_ok(bs->ob_temp_id, c->NOB, bs->temp.n_series) || !ids_ok(bs->qb_q_id, c->NQB, bs->q.n_series) ||
        !ids_ok(bs->qb_salt_id, c->NQB, bs->salt.n_series) || !ids_ok(bs->qb_temp_id, c->NQB, bs->temp.n_series) ||
        (c->NQB > 0 && !bs->qb_portion))
        return GOM_E_ARG;
    if (bs->q_interp_method != 1 && bs->q_interp_method != 2) return GOM_E_ARG;
    if (bs->hurricane_flag != 0 && bs->hurricane_flag != 1) return GOM_E_ARG;
    if (bs->hurricane_flag == 1 && (bs->hurricane_read_interval < 1 || !bs->hurricane_frames || !(bs->rho_a > 0.0) ||
                                    bs->hurricane_interp_method < 0 || bs->hurricane_interp_method > 2))
        return GOM_E_ARG;
    if (bs->heat_flag != 0 && bs->heat_flag != 1) return GOM_E_ARG;
    if (bs->heat_flag == 1) {
        if (!c->p.transport_flag || !c->p.is_temp || c->p.heat_option != 1 || (bs->sol_swr != 1 && bs->sol_swr != 2) ||
            bs->n_air < 0 || (bs->sol_swr == 1 && (bs->month < 1 || bs->month > 12)) ||
            (bs->n_air > 0 && (!bs->air_time || !bs->air_values)))
            return GOM_E_ARG;
        for (int t = 1; t < bs->n_air; ++t)
            if (!(bs->air_time[t] >= bs->air_time[t - 1])) return GOM_E_ARG;
    }
    if (bs->wind_flag != 0 && bs->wind_flag != 1) return GOM_E_ARG;
    if (bs->wind_flag == 1) {
        if (bs->wind_formular < 1 || bs->wind_formular > 3 || bs->n_wind < 1 || bs->n_wind > 3 ||
            bs->wind_u.n_series != bs->n_wind || bs->wind_v.n_series != bs->n_wind || !(bs->rho_a > 0.0))
            return GOM_E_ARG;
        for (const gom_series *sr : {&bs->wind_u, &bs->wind_v}) {
            if (!sr->start || !sr->time || !sr->value || sr->start[0] != 0) return GOM_E_ARG;
            for (int k = 0; k < sr->n_series; ++k) {
                if (sr->start[k + 1] < sr->start[k]) return GOM_E_ARG;
                for (int q = sr->start[k] + 1; q < sr->start[k + 1]; ++q)
                    if (!(sr->time[q] >= sr->time[q - 1])) return GOM_E_ARG;
            }
        }
        if (bs->n_wind > 1) {
            if (!bs->wind_station_node) return GOM_E_ARG;
            for (int k = 0; k < bs->n_wind; ++k)
                if (bs->wind_station_node[k] < 1 || bs->wind_station_node[k] > c->NN) return GOM_E_ARG;
        }
    }
    for (int k = 0; k < 4; ++k) {
        const gom_series &sr = *sets[k];
        c->sr_start[k].assign(1, 0);
        c->sr_time[k].clear();
        c->sr_value[k].clear();
        if (sr.n_series > 0) {
            c->sr_start[k].assign(sr.start, sr.start + sr.n_series + 1);
            c->sr_time[k].assign(sr.time, sr.time + sr.start[sr.n_series]);
            c->sr_value[k].assign(sr.value, sr.value + sr.start[sr.n_series]);
        }
    }
    auto ids = [](std::vector<int32_t> &v, const int32_t *src, int n) {
        v.assign((size_t)n, 0);
        if (src) v.assign(src, src + n);
    };
    ids(c->ob_type, bs->ob_eta_type, c->NOB);
    ids(c->ob_h, bs->ob_harmonic_id, c->NOB);
    ids(c->ob_eta, bs->ob_eta_id, c->NOB);
    ids(c->ob_salt, bs->ob_salt_id, c->NOB);
    ids(c->ob_temp, bs->ob_temp_id, c->NOB);
    ids(c->qb_q, bs->qb_q_id, c->NQB);
    ids(c->qb_salt, bs->qb_salt_id, c->NQB);
    ids(c->qb_temp, bs->qb_temp_id, c->NQB);
    c->qb_portion.assign((size_t)c->NQB, 0.0);
    if (bs->qb_portion) c->qb_portion.assign(bs->qb_portion, bs->qb_portion + c->NQB);
    c->n_harm = bs->n_harmonic;
    c->h_start.assign(1, 0);
    c->h_amp.clear(), c->h_per.clear(), c->h_nodal.clear(), c->h_eq.clear(), c->h_ph.clear(), c->h_shift.clear();
    if (bs->n_harmonic > 0) {
        const int nh = bs->n_harmonic, nc = bs->harmonic_start[nh];
        c->h_start.assign(bs->harmonic_start, bs->harmonic_start + nh + 1);
        c->h_amp.assign(bs->amplitude, bs->amplitude + nc);
        c->h_per.assign(bs->period_h, bs->period_h + nc);
        c->h_nodal.assign(bs->nodal, bs->nodal + nc);
        c->h_eq.assign(bs->eq_arg, bs->eq_arg + nc);
        c->h_ph.assign(bs->phase, bs->phase + nc);
        c->h_shift.assign(bs->phase_shift, bs->phase_shift + nh);
    }
    // reference_diff_days * 86400.0: an integer times a default-REAL constant, in single precision
    c->rdd_s = (double)((float)bs->reference_diff_days * 86400.0f);
    c->tide_per_s = bs->tide_spinup == 1 ? bs->tide_spinup_period * 86400.0 : 0.0;
    c->bc_per_s = (bs->baroclinic_spinup == 1 && c->p.baroclinic_flag == 1) ? bs->baroclinic_spinup_period * 86400.0
                                                                              : 0.0;
    c->q_method = bs->q_interp_method;
    // station wind: the series as kinds 4 (u) and 5 (v), calculate_wind_stress.f90:20-33 bounds
    // (default-REAL expressions scaled in double)
    c->wind_flag = bs->wind_flag;
    c->n_wind = bs->wind_flag == 1 ? bs->n_wind : 0;
    c->wind_formular = bs->wind_formular;
    const gom_series *wsets[2] = {&bs->wind_u, &bs->wind_v};
    for (int k = 0; k < 2; ++k) {
        const gom_series &sr = *wsets[k];
        c->sr_start[4 + k].assign(1, 0);
        c->sr_time[4 + k].clear();
        c->sr_value[4 + k].clear();
        if (c->n_wind > 0) {
            c->sr_start[4 + k].assign(sr.start, sr.start + sr.n_series + 1);
            c->sr_time[4 + k].assign(sr.time, sr.time + sr.start[sr.n_series]);
            c->sr_value[4 + k].assign(sr.value, sr.value + sr.start[sr.n_series]);
        }
    }
    c->wind_node.assign(c->n_wind, 0);
    if (c->n_wind > 1) c->wind_node.assign(bs->wind_station_node, bs->wind_station_node + c->n_wind);
    c->wind_per_s = (bs->wind_flag == 1 && bs->wind_spinup == 1) ? bs->wind_spinup_period * 86400.0 : 0.0;
    c->hur_flag = bs->hurricane_flag;
    c->rho_ratio = (bs->wind_flag == 1 || c->hur_flag == 1) ? bs->rho_a / c->p.rho_o : 0.0;
    c->hur_interval = c->hur_flag == 1 ? bs->hurricane_read_interval : 1;
    c->hur_start = bs->hurricane_start_jday;
    c->hur_end = bs->hurricane_end_jday;
    c->hur_ready = false;
    c->hur_frames.clear();
    if (c->hur_flag == 1) c->hur_frames.assign(bs->hurricane_frames, bs->hurricane_frames + 9 * (size_t)c->NN);
    c->hur_next.assign(c->hur_flag == 1 ? 3 * (size_t)c->NN : 0, 0.0);
    c->face_u.assign(c->NF, 0.0);
    c->face_v.assign(c->NF, 0.0);
    c->heat_flag = bs->heat_flag;
    c->sol_swr = bs->sol_swr;
    c->year = bs->year;
    c->month = bs->month;
    c->month_table_set = 0;
    c->lon = bs->lon;
    c->lat = bs->lat;
    c->air_time.clear();
    c->air_values.clear();
    if (bs->heat_flag == 1 && bs->n_air > 0) {
        c->air_time.assign(bs->air_time, bs->air_time + bs->n_air);
        c->air_values.assign(bs->air_values, bs->air_values + 5 * (size_t)bs->n_air);
    }
    c->fwz_a = bs->fwz_a;
    c->fwz_b = bs->fwz_b;
    c->fwz_c = bs->fwz_c;
    c->wind_height = bs->wind_height;
    c->light_extinction = bs->light_extinction;
    c->sol_absorb = bs->sol_absorb;
    c->sed_water_exchange = bs->sed_water_exchange;
    c->t_sed = bs->t_sed;
    c->sed_temp_coeff = bs->sed_temp_coeff;
    c->hur_method = (c->hur_flag == 1 && bs->hurricane_interp_method == 2) ? 2 : 1;
    c->track_ready = false;
    c->search_start.clear();
    c->search_nodes.clear();
    if (c->hur_flag == 1 && c->hur_method == 2) {
        for (int k = 0; k < 6; ++k) c->track[k] = bs->hurricane_track[k];
        if (!find_neighbour_nodes(c)) {
            c->hur_flag = 0;
            c->has_series = false;
            return GOM_E_ARG;   // a node with no neighbour in range: IDW_5 would read outside its list
        }
    }
    {
        const float lo[3] = {0.75f + 0.067f * 4.0f, 0.61f + 0.063f * 6.0f, 0.80f + 0.065f * 1.0f};
        const float hi[3] = {0.75f + 0.067f * 50.0f, 0.61f + 0.063f * 50.0f, 0.80f + 0.065f * 50.0f};
        const int fi = bs->wind_formular >= 1 && bs->wind_formular <= 3 ? bs->wind_formular - 1 : 1;
        c->cda_min = 0.001 * (double)lo[fi];
        c->cda_max = 0.001 * (double)hi[fi];
    }
    c->jday = bs->julian_day;
    c->step_no = bs->step;
    c->has_series = true;
    return GOM_OK;
}

namespace {

// first interval t2 of the reference's search with u1 <= u2 <= u3 (times minus the offset)
bool series_value(const gom_ctx *c, int kind, int id, double u2, double &v) {
    if (id < 1 || id + 1 > (int)c->sr_start[kind].size()) return false;
    const int s0 = c->sr_start[kind][id - 1], s1 = c->sr_start[kind][id];
    for (int t2 = s0 + 1; t2 < s1; ++t2) {
        const double u1 = c->sr_time[kind][t2 - 1] - c->rdd_s;
        const double u3 = c->sr_time[kind][t2] - c->rdd_s;
        if (u2 >= u1 && u2 <= u3) {
            const double v1 = c->sr_value[kind][t2 - 1], v3 = c->sr_value[kind][t2];
            v = (u2 - u1) * (v3 - v1) / (u3 - u1) + v1;
            return true;
        }
    }
    return false;
}

double q_lagrange(const gom_ctx *c, int id, double u2) {
    const int s0 = c->sr_start[1][id - 1], n = c->sr_start[1][id] - s0;
    const double *t = c->sr_time[1].data() + s0, *val = c->sr_value[1].data() + s0;
    int min_index = 0;
    double best = 0.0;
    for (int k = 0; k < n; ++k) {
        const double d = t[k] - u2;
        if (d >= 0.0 && (min_index == 0 || d < best)) {
            best = d;
            min_index = k + 1;
        }
    }
    if (min_index == 0) min_index = n;
    if (min_index == 1) min_index = min_index + 1;
    min_index = min_index - 1;
    const int shift = (min_index + 2) - n;
    if (shift > 0) min_index = min_index - shift;
    if (min_index < 1) min_index = 1;
    double total = 0.0;
    for (int ii = 0; ii <= 2; ++ii) {
        double prod = val[min_index - 1 + ii];
        for (int jj = 0; jj <= 2; ++jj)
            if (jj != ii) prod = prod * (u2 - t[min_index - 1 + jj]) / (t[min_index - 1 + ii] - t[min_index - 1 + jj]);
        total = total + prod;
    }
    return total;
}

// setup_spinup.f90:44-54, get_windp_at_face.f90:18-48, IDW_windp_ser.f90:27-118 and
// calculate_wind_stress.f90:41-65 (heat_model_flag 0)
void station_wind(gom_ctx *c, double elapsed, double u2) {
    const double spin_w = (c->wind_per_s > 0.0 && elapsed < c->wind_per_s) ? std::tanh(2.0 * elapsed / c->wind_per_s)
                                                                               : 1.0;
    double st[3][2] = {{0, 0}, {0, 0}, {0, 0}};
    for (int k = 1; k <= c->n_wind; ++k) {
        double v12 = 0.0, v22 = 0.0;
        for (int comp = 0; comp < 2; ++comp) {
            const std::vector<int32_t> &sta = c->sr_start[4 + comp];
            const double *t = c->sr_time[4 + comp].data() + sta[k - 1];
            const double *v = c->sr_value[4 + comp].data() + sta[k - 1];
            const int n = sta[k] - sta[k - 1];
            for (int q = 2; q <= n; ++q) {
                const double u1 = t[q - 2] - c->rdd_s, u3 = t[q - 1] - c->rdd_s;
                if (u2 >= u1 && u2 <= u3) {
                    const double r = (v[q - 1] - v[q - 2]) / (u3 - u1) * (u2 - u1) + v[q - 2];
                    if (comp == 0) v12 = r;
                    else v22 = r;
                    break;
                }
            }
        }
        st[k - 1][0] = v12;
        st[k - 1][1] = v22;
    }
    auto idw = [&](int node, double &u, double &v) {
        const double x = c->x_node(node), y = c->y_node(node);
        double dist[3];
        for (int k = 1; k <= c->n_wind; ++k) {
            const double x1 = c->x_node(c->wind_node[k - 1]), y1 = c->y_node(c->wind_node[k - 1]);
            dist[k - 1] = std::sqrt((x - x1) * (x - x1) + (y - y1) * (y - y1));
        }
        if (c->n_wind == 2) {
            const double r1 = dist[1], r2 = dist[0];
            u = (r1 * st[0][0] + r2 * st[1][0]) / (r1 + r2);
            v = (r1 * st[0][1] + r2 * st[1][1]) / (r1 + r2);
        } else {
            const double r1 = dist[1] * dist[2], r2 = dist[0] * dist[2], r3 = dist[0] * dist[1];
            u = (r1 * st[0][0] + r2 * st[1][0] + r3 * st[2][0]) / (r1 + r2 + r3);
            v = (r1 * st[0][1] + r2 * st[1][1] + r3 * st[2][1]) / (r1 + r2 + r3);
        }
    };
    for (int j = 1; j <= c->NF; ++j) {
        double u, v;
        if (c->n_wind == 1) {
            u = st[0][0];
            v = st[0][1];
        } else {
            double u1, v1, u2n, v2n;
            idw(c->nodenum_at_face(1, j), u1, v1);
            idw(c->nodenum_at_face(2, j), u2n, v2n);
            u = (u1 + u2n) * 0.5;
            v = (v1 + v2n) * 0.5;
        }
        c->face_u[j - 1] = u;
        c->face_v[j - 1] = v;
        if (c->hur_flag == 1) continue;   // the hurricane branch below overwrites the stresses
        const double speed = std::sqrt(u * u + v * v);
        const double normal = u * c->cos_theta(j) + v * c->sin_theta(j);
        const double tangent = -u * c->sin_theta(j) + v * c->cos_theta(j);
        double cda;
        if (c->wind_formular == 1) cda = 0.001 * (0.75 + 0.067 * speed);
        else if (c->wind_formular == 2) cda = 0.001 * (0.61 + 0.063 * speed);
        else cda = 0.001 * (0.80 + 0.065 * speed);
        cda = std::min(std::max(cda, c->cda_min), c->cda_max);
        const double gamma_t = cda * c->rho_ratio * speed;
        c->gamma_t[j - 1] = gamma_t;
        c->wind_stress_normal[j - 1] = gamma_t * normal * spin_w;
        c->wind_stress_tangnt[j - 1] = gamma_t * tangent * spin_w;
    }
}

// IDW_5.f90:36-80 at the point (xn, yn) over node i's neighbour list: the three nearest (minloc:
// the first of equal distances; a taken entry becomes the default-REAL 1.0e15), weighted by the
// products of the other two distances (power 1)
void idw5(const gom_ctx *c, int i, double xn, double yn, const double *v, size_t nn, double out[3]) {
    const double far = (double)1.0e15f;
    const int64_t s0 = c->search_start[i - 1], cnt = c->search_start[i] - s0;
    std::vector<double> dist(cnt);
    for (int64_t k = 0; k < cnt; ++k) {
        const int nd = c->search_nodes[s0 + k];
        const double dx = xn - c->x_node(nd), dy = yn - c->y_node(nd);
        dist[k] = std::sqrt(dx * dx + dy * dy);
    }
    int nsel[3];
    double md[3];
    for (int q = 0; q < 3; ++q) {
        int64_t ii = 0;
        for (int64_t k = 1; k < cnt; ++k)
            if (dist[k] < dist[ii]) ii = k;
        nsel[q] = c->search_nodes[s0 + ii];
        md[q] = dist[ii];
        dist[ii] = far;
    }
    const double r1 = md[1] * md[2], r2 = md[0] * md[2], r3 = md[0] * md[1];
    for (int comp = 0; comp < 3; ++comp) {
        const double *w = v + comp * nn;
        out[comp] = (r1 * w[nsel[0] - 1] + r2 * w[nsel[1] - 1] + r3 * w[nsel[2] - 1]) / (r1 + r2 + r3);
    }
}

// find_neighbour_nodes.f90:19-45: every node within 20 km of a node (when its nearest neighbour is
// nearer than 5 km) or within four times that nearest distance, in node order; false when a node
// has none (IDW_5 would then read outside its list)
bool find_neighbour_nodes(gom_ctx *c) {
    const double far = (double)1.0e15f;
    const int nn = c->NN;
    c->search_start.assign(nn + 1, 0);
    std::vector<double> dist(nn);
    for (int i = 1; i <= nn; ++i) {
        double min_dist = far;
        for (int ii = 1; ii <= nn; ++ii) {
            if (ii == i) {
                dist[ii - 1] = far;
            } else {
                const double dx = c->x_node(i) - c->x_node(ii), dy = c->y_node(i) - c->y_node(ii);
                dist[ii - 1] = std::sqrt(dx * dx + dy * dy);
            }
            if (dist[ii - 1] < min_dist) min_dist = dist[ii - 1];
        }
        const double range = min_dist < 5000 ? (double)(20 * 1000.0f) : min_dist * 4;
        for (int ii = 1; ii <= nn; ++ii)
            if (dist[ii - 1] <= range) c->search_nodes.push_back(ii);
        c->search_start[i] = (int64_t)c->search_nodes.size();
        if (c->search_start[i] == c->search_start[i - 1]) return false;
    }
    return true;
}

// main.f90:115-127 with read_hurricane_ser_1.f90:20-86 or read_hurricane_ser_2.f90:19-146 (julian_day
// inside the window), then the hurricane branch of calculate_wind_stress.f90:105-137 on every face
void hurricane_wind(gom_ctx *c, double spin_w) {
    const size_t nn = (size_t)c->NN;
    double *w0 = c->hur_frames.data(), *w1 = w0 + 3 * nn, *w2 = w0 + 6 * nn;
    const bool window = c->jday >= c->hur_start && c->jday <= c->hur_end;
    if (window) {
        const int read_count = c->step_no % c->hur_interval;
        if (read_count == 0) {
            for (size_t q = 0; q < 3 * nn; ++q) {
                w0[q] = w2[q];
                w1[q] = w2[q];
            }
            if (c->hur_method == 2) {
                // read_hurricane_ser_2.f90:35-45: the centre moves on to the next record
                c->track[0] = c->track[3];
                c->track[1] = c->track[4];
                if (!c->track_ready) {
                    set_err(c, GOM_E_ARG, 38, 0, 0, (double)c->step_no, GOM_ENTITY_OTHER);
                } else {
                    c->track[3] = c->track_next[0];
                    c->track[4] = c->track_next[1];
                    c->track[5] = c->track_next[2];
                }
                c->track_ready = false;
            }
            // the record of :34-46 (pushed by the driver)
            if (!c->hur_ready) set_err(c, GOM_E_ARG, 34, 0, 0, (double)c->step_no, GOM_ENTITY_OTHER);
            else std::copy(c->hur_next.begin(), c->hur_next.end(), w2);
            c->hur_ready = false;
        } else if (c->hur_method == 2) {
            // read_hurricane_ser_2.f90:73-134: both frames moved with the centre and blended
            const double tr = (c->jday - c->track[2]) / (c->track[5] - c->track[2]);
            const double dxc = c->track[3] - c->track[0], dyc = c->track[4] - c->track[1];
            const double cx = c->track[0] + dxc * tr, cy = c->track[1] + dyc * tr;
            c->track[0] = cx;
            c->track[1] = cy;
            c->track[2] = c->track[2] + c->p.dt / 86400.0;
            std::vector<double> w1n(3 * nn), w2n(3 * nn);
            for (size_t i = 1; i <= nn; ++i) {
                double o[3];
                idw5(c, (int)i, c->x_node((int)i) - dxc * tr, c->y_node((int)i) - dyc * tr, w1, nn, o);
                for (int comp = 0; comp < 3; ++comp) w1n[comp * nn + i - 1] = o[comp];
                idw5(c, (int)i, c->x_node((int)i) + dxc * (1.0 - tr), c->y_node((int)i) + dyc * (1.0 - tr), w2, nn, o);
                for (int comp = 0; comp < 3; ++comp) w2n[comp * nn + i - 1] = o[comp];
            }
            for (size_t q = 0; q < 3 * nn; ++q) w1[q] = (1.0 - tr) * w1n[q] + tr * w2n[q];
        } else {
            const double den = (double)(float)c->hur_interval;   // real(hurricane_read_interval)
            for (size_t q = 0; q < 3 * nn; ++q) {
                const double inc = (w2[q] - w0[q]) / den;
                w1[q] = w1[q] + inc;
            }
        }
        for (size_t i = 0; i < nn; ++i) c->air_p[i] = w1[2 * nn + i];
        for (int j = 1; j <= c->NF; ++j) {
            const int n1 = c->nodenum_at_face(1, j) - 1, n2 = c->nodenum_at_face(2, j) - 1;
            c->face_u[j - 1] = (w1[n1] + w1[n2]) * 0.5;
            c->face_v[j - 1] = (w1[nn + n1] + w1[nn + n2]) * 0.5;
        }
    }
    const double cda_max = (double)0.003f;   // MIN(0.003, Cda): a default-REAL constant
    for (int j = 1; j <= c->NF; ++j) {
        const double u = c->face_u[j - 1], v = c->face_v[j - 1];
        const double speed = std::sqrt(u * u + v * v);
        const double normal = u * c->cos_theta(j) + v * c->sin_theta(j);
        const double tangent = -u * c->sin_theta(j) + v * c->cos_theta(j);
        double cda;
        if (c->wind_formular == 1) cda = 0.001 * (0.75 + 0.067 * speed);
        else if (c->wind_formular == 2) cda = 0.001 * (0.61 + 0.063 * speed);
        else if (c->wind_formular == 3) cda = 0.001 * (0.80 + 0.065 * speed);
        else cda = 0.001 * (0.61 + 0.063 * speed);
        cda = std::min(cda_max, cda);
        const double gamma_t = cda * c->rho_ratio * speed;
        c->gamma_t[j - 1] = gamma_t;
        c->wind_stress_normal[j - 1] = gamma_t * normal * spin_w;
        c->wind_stress_tangnt[j - 1] = gamma_t * tangent * spin_w;
    }
}

void series_forcing(gom_ctx *c) {
    const double dt = c->p.dt;
    c->step_no += 1;
    const double elapsed = (double)c->step_no * dt;
    c->elapsed_time = elapsed;
    c->jday = c->jday + dt / 86400.0;
    c->spinup_tide = (c->tide_per_s > 0.0 && elapsed < c->tide_per_s) ? std::tanh(2.0 * elapsed / c->tide_per_s) : 1.0;
    c->spinup_baroclinic = (c->bc_per_s > 0.0 && elapsed < c->bc_per_s) ? std::tanh(2.0 * elapsed / c->bc_per_s) : 1.0;
    const double spin = c->spinup_tide, spin_bc = c->spinup_baroclinic, jd_s = c->jday * 86400.0;
    A1<double> eta_cell = FD1(c, GOM_F_ETA_CELL);
    if (c->wind_flag == 1) station_wind(c, elapsed, jd_s);
    if (c->hur_flag == 1)
        hurricane_wind(c, (c->wind_per_s > 0.0 && elapsed < c->wind_per_s) ? std::tanh(2.0 * elapsed / c->wind_per_s)
                                                                            : 1.0);
    const double deg2rad = 3.141592653589793 / 180.0;
    for (int i = 0; i < c->NOB; ++i) {
        if (c->ob_type[i] == -1) {
            // compute_boundary_eta.f90:45-70: the mean elevation of the interior cells around the
            // open-boundary cell's nodes (each counted once per node it shares), old level only
            const int cell = c->ob_cell_id(i + 1);
            double sum0 = 0.0;
            int icount = 0;
            for (int l = 1; l <= c->tri_or_quad(cell); ++l) {
                const int nd = c->nodenum_at_cell(l, cell);
                for (int i2 = 1; i2 <= c->adj_cells_at_node(nd); ++i2) {
                    const int ie = c->adj_cellnum_at_node(i2, nd);
                    if (c->ob_element_flag(ie) == 0) {
                        icount = icount + 1;
                        sum0 = sum0 + eta_cell(ie);
                    }
                }
            }
            if (icount == 0) set_err(c, GOM_E_ARG, 0, i + 1, 0, 0.0, GOM_ENTITY_OTHER);
            else c->eta_at_ob_old[i] = sum0 / icount;
        } else if (c->ob_type[i] == 1) {
            const int h = c->ob_h[i];
            double o = 0.0, nw = 0.0;
            if (h >= 1 && h <= c->n_harm) {
                for (int j = c->h_start[h - 1]; j < c->h_start[h]; ++j) {
                    const double w = 2.0 * 3.141592653589793 / (c->h_per[j] * 3600.0);
                    const double a = spin * c->h_amp[j] * c->h_nodal[j];
                    o = o + a * std::cos(w * (elapsed - dt) + c->h_eq[j] * deg2rad - c->h_ph[j] * deg2rad -
                                         c->h_shift[h - 1] * deg2rad);
                    nw = nw + a * std::cos(w * elapsed + c->h_eq[j] * deg2rad - c->h_ph[j] * deg2rad -
                                           c->h_shift[h - 1] * deg2rad);
                }
            }
            c->eta_at_ob_old[i] = o;
            c->eta_at_ob_new[i] = nw;
        } else if (c->ob_type[i] == 2) {
            double v;
            if (series_value(c, 0, c->ob_eta[i], jd_s - dt, v)) c->eta_at_ob_old[i] = spin * v;
            if (series_value(c, 0, c->ob_eta[i], jd_s, v)) c->eta_at_ob_new[i] = spin * v;
        }
    }
    for (int i = 0; i < c->NQB; ++i) {
        const int q = c->qb_q[i];
        double v;
        if (q >= 1) {   // ids were checked against the series count when they were set
            if (c->q_method == 2) c->q_add[i] = q_lagrange(c, q, jd_s) * c->qb_portion[i];
            else if (series_value(c, 1, q, jd_s, v)) c->q_add[i] = v * c->qb_portion[i];
        }
    }
    const int nt = std::max(1, c->p.trans_sub_iter);
    const bool salt = c->p.transport_flag && c->p.is_salt, temp = c->p.transport_flag && c->p.is_temp;
    const double dt2 = dt / nt;
    for (int sub = 0; sub < nt; ++sub) {
        const double u2 = (jd_s - dt) + (sub + 1) * dt2;
        double v;
        for (int i = 0; i < c->NOB; ++i) {
            if (salt) {
                double &x = c->con_at_ob[((size_t)sub * 2 + 0) * c->NOB + i];
                if (c->ob_salt[i] <= 0) x = 0.0;
                else if (series_value(c, 2, c->ob_salt[i], u2, v)) x = spin_bc * v;
            }
            if (temp) {
                double &x = c->con_at_ob[((size_t)sub * 2 + 1) * c->NOB + i];
                if (c->ob_temp[i] <= 0) x = 0.0;
                else if (series_value(c, 3, c->ob_temp[i], u2, v)) x = spin_bc * v;
            }
        }
        for (int i = 0; i < c->NQB; ++i) {
            if (salt) {
                double &x = c->con_at_qb[((size_t)sub * 2 + 0) * c->NQB + i];
                if (c->qb_salt[i] <= 0) x = 0.0;
                else if (series_value(c, 2, c->qb_salt[i], u2, v)) x = spin_bc * v;
            }
            if (temp) {
                double &x = c->con_at_qb[((size_t)sub * 2 + 1) * c->NQB + i];
                if (c->qb_temp[i] <= 0) x = 0.0;
                else if (series_value(c, 3, c->qb_temp[i], u2, v)) x = spin_bc * v;
            }
        }
    }
}

}  // namespace
int gom_cold_start(gom_ctx *c, double, double, double, double) { return c ? GOM_E_ARG : GOM_E_ARG; }
// nothing to tune on the CPU
int gom_autotune(gom_ctx *c, int32_t, int32_t *choice) {
    if (!c) return GOM_E_ARG;
    if (choice)
        for (int k = 0; k < GOM_TUNE_SITES; ++k) choice[k] = 0;
    return GOM_OK;
}

// snapshots are taken synchronously on the CPU
int gom_snapshot_begin(gom_ctx *c, int32_t n_fields, const int32_t *fields, void *const *host) {
    if (!c || n_fields < 0 || (n_fields > 0 && (!fields || !host)) || c->snap_pending) return GOM_E_ARG;
    for (int q = 0; q < n_fields; ++q) {
        int32_t eb = 0;
        const int64_t n = (fields[q] > 0 && fields[q] < GOM_F_COUNT) ? field_count(c->d, fields[q], &eb) : -1;
        if (n < 0 || !host[q]) return GOM_E_ARG;
        int rc = gom_get_field(c, fields[q], host[q], n);
        if (rc != GOM_OK) return rc;
    }
    c->snap_pending = true;
    return GOM_OK;
}
int gom_snapshot_ready(gom_ctx *c) { return c ? 1 : GOM_E_ARG; }
int gom_snapshot_wait(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    c->snap_pending = false;
    return GOM_OK;
}
int gom_host_alloc(int64_t bytes, void **out) {
    if (!out || bytes <= 0) return GOM_E_ARG;
    *out = std::malloc((size_t)bytes);
    return *out ? GOM_OK : GOM_E_NOMEM;
}
void gom_host_free(void *p) { std::free(p); }

int gom_tuning_variants(int32_t counts[GOM_TUNE_SITES]) {
    if (!counts) return GOM_E_ARG;
    for (int k = 0; k < GOM_TUNE_SITES; ++k) counts[k] = 1;
    return GOM_OK;
}

int gom_set_tuning(gom_ctx *c, const int32_t choice[GOM_TUNE_SITES]) {
    if (!c || !choice) return GOM_E_ARG;
    for (int k = 0; k < GOM_TUNE_SITES; ++k)
        if (choice[k] < -1 || choice[k] > 0) return GOM_E_ARG;
    return GOM_OK;
}

int gom_get_status(gom_ctx *c, gom_status *s, int clear) {
    if (!c || !s) return GOM_E_ARG;
    s->code = c->err.code;
    s->site = c->err.site;
    s->entity = c->err.entity;
    s->layer = c->err.layer;
    s->value = c->err.value;
    s->entity_kind = c->err.kind;
    s->run = -1;
    if (s->code != 0 && s->entity >= 1 && s->entity_kind >= GOM_ENTITY_CELL && s->entity_kind <= GOM_ENTITY_NODE) {
        if (c->d.n_runs <= 1) {
            s->run = 0;
        } else {
            const std::vector<int32_t> &v = s->entity_kind == GOM_ENTITY_CELL   ? c->run_cell_start
                                            : s->entity_kind == GOM_ENTITY_FACE ? c->run_face_start
                                                                                : c->run_node_start;
            for (int r = 0; r + 1 < (int)v.size(); ++r)
                if (s->entity - 1 >= v[r] && s->entity - 1 < v[r + 1]) s->run = r;
        }
    }
    if (clear) c->err = Err();
    return GOM_OK;
}

int gom_synchronize(gom_ctx *c) { return c ? GOM_OK : GOM_E_ARG; }

// GPU measurements: nothing to measure on the CPU
int gom_measure_fp64_peak(double *gflops) {
    if (gflops) *gflops = 0.0;
    return GOM_E_ARG;
}
int gom_measure_fp64_issue(int32_t, double *warp_instr_per_s) {
    if (warp_instr_per_s) *warp_instr_per_s = 0.0;
    return GOM_E_ARG;
}
int gom_selftest_compares(int64_t *checked, int64_t *mismatches) {
    if (checked) *checked = 0;
    if (mismatches) *mismatches = 0;
    return GOM_E_ARG;
}

int64_t gom_pcg_iterations_total(gom_ctx *c) { return c ? c->pcg_total : 0; }

int64_t gom_device_bytes(const gom_ctx *) { return 0; }
int gom_profile_kernel(gom_ctx *c, int32_t, int32_t, double *) { return c ? GOM_E_ARG : GOM_E_ARG; }
int gom_copy_run(gom_ctx *dst, int32_t, gom_ctx *, int32_t) { return dst ? GOM_E_ARG : GOM_E_ARG; }

void *gom_stream(gom_ctx *c) {
    (void)c;
    return nullptr;
}

// ============================================================================================
// calculate_bottom_friction.f90:9-73 (bf_flag 3 = constant Cd, an extension for quadratic drag)
int gom_step_bottom_friction(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    A1<double> Cdb = FD1(c, GOM_F_CDB), Gamma_B = FD1(c, GOM_F_GAMMA_B);
    A2<double> un_face = FD(c, GOM_F_UN_FACE), vn_face = FD(c, GOM_F_VN_FACE), dzhalf_face = FD(c, GOM_F_DZHALF_FACE);
    const gom_params &p = c->p;
    for (int j = 1; j <= c->NF; ++j) {
        Cdb(j) = 0.0;
        Gamma_B(j) = 0.0;
    }
    if (p.bf_flag == 1) {
        double expo = 1.0 / 6.0;
        for (int j = 1; j <= c->NF; ++j) {
            if (c->h_face(j) > p.dry_depth) {
                double hydraulic_radius = std::max(1.0, c->h_face(j));
                double chezy_coef = std::pow(hydraulic_radius, expo) / c->manning(j);
                double rtemp = p.gravity / (chezy_coef * chezy_coef);
                Cdb(j) = rtemp;
                int k = c->bottom_layer_at_face(j);
                Gamma_B(j) = Cdb(j) * std::sqrt(un_face(k, j) * un_face(k, j) + vn_face(k, j) * vn_face(k, j));
            }
        }
    } else if (p.bf_flag == 2) {
        for (int j = 1; j <= c->NF; ++j) {
            if (c->h_face(j) > p.dry_depth) {
                int k = c->bottom_layer_at_face(j);
                double lg = std::log(std::max(0.5, dzhalf_face(k - 1, j)) / c->bf_height(j));
                double rtemp = p.von_karman * p.von_karman / (lg * lg);
                Cdb(j) = rtemp;
                Gamma_B(j) = Cdb(j) * std::sqrt(un_face(k, j) * un_face(k, j) + vn_face(k, j) * vn_face(k, j));
            }
        }
    } else if (p.bf_flag == 3) {
        for (int j = 1; j <= c->NF; ++j) {
            if (c->h_face(j) > p.dry_depth) {
                int k = c->bottom_layer_at_face(j);
                Cdb(j) = p.cd_const;
                Gamma_B(j) = Cdb(j) * std::sqrt(un_face(k, j) * un_face(k, j) + vn_face(k, j) * vn_face(k, j));
            }
        }
    }
    return GOM_OK;
}

// compute_boundary_velocity.f90:60-94 (river faces; Q_add comes from the host's calculate_Q)
int gom_step_boundary_velocity(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    A1<double> Qu = FD1(c, GOM_F_QU_BOUNDARY), eta_node = FD1(c, GOM_F_ETA_NODE);
    for (int i = 1; i <= c->NQB; ++i) {
        int j = c->qb_face(i);
        double channel_width = c->face_length(j);
        int n1 = c->nodenum_at_face(1, j), n2 = c->nodenum_at_face(2, j);
        double temp_depth = c->h_face(j) + (eta_node(n1) + eta_node(n2)) * 0.5;
        if (temp_depth < c->p.dry_depth) {
            set_err(c, GOM_E_DRY, 80, i, 0, temp_depth, GOM_ENTITY_OTHER);
            return GOM_E_DRY;
        }
        Qu(i) = -c->q_add[i - 1] / (channel_width * temp_depth);
    }
    return GOM_OK;
}

// main.f90:167-177 and solve_nonlinear_advection.f90:14-204
int gom_step_advection(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    const gom_params &p = c->p;
    int L = c->L;
    A2<double> un_ELM = FD(c, GOM_F_UN_ELM), vn_ELM = FD(c, GOM_F_VN_ELM), un_face = FD(c, GOM_F_UN_FACE),
               vn_face = FD(c, GOM_F_VN_FACE);
    A2<int32_t> foot = FI(c, GOM_F_ELM_FOOT), near = FI(c, GOM_F_ELM_NEAR_EDGE);
    std::fill(c->fi[GOM_F_ELM_FOOT].begin(), c->fi[GOM_F_ELM_FOOT].end(), 0);
    std::fill(c->fi[GOM_F_ELM_NEAR_EDGE].begin(), c->fi[GOM_F_ELM_NEAR_EDGE].end(), 0);
    if (p.advection_flag == 0) {
        for (int j = 1; j <= c->NF; ++j)
            for (int k = 1; k <= L; ++k) {
                un_ELM(k, j) = un_face(k, j);
                vn_ELM(k, j) = vn_face(k, j);
            }
        return GOM_OK;
    }
    A2<double> u_node = FD(c, GOM_F_U_NODE), v_node = FD(c, GOM_F_V_NODE), w_node = FD(c, GOM_F_W_NODE),
               dz_cell = FD(c, GOM_F_DZ_CELL);
    A2<int32_t> nsub = FI(c, GOM_F_NUM_SUB_ELM);
    A1<double> eta_cell = FD1(c, GOM_F_ETA_CELL);
    A1<int32_t> top_el = FI1(c, GOM_F_TOP_LAYER_CELL), top_f = FI1(c, GOM_F_TOP_LAYER_FACE);
    std::fill(c->fd[GOM_F_UN_ELM].begin(), c->fd[GOM_F_UN_ELM].end(), 0.0);
    std::fill(c->fd[GOM_F_VN_ELM].begin(), c->fd[GOM_F_VN_ELM].end(), 0.0);
    // :52-87 adaptive substep count
    if (p.elm_backtrace_flag == 1) {
        double dt = p.dt;
        OMP_FOR
        for (int i = 1; i <= c->NN; ++i) {
            for (int k = 1; k <= L; ++k) {
                double summ = 0.0;
                int nadj = c->adj_cells_at_node(i);
                for (int j = 1; j <= nadj; ++j) {
                    int ie = c->adj_cellnum_at_node(j, i);
                    int id = c->node_count_each_element(j, i);
                    double devm = 0.0;
                    int tq = c->tri_or_quad(ie);
                    for (int l = 1; l <= 2; ++l) {
                        int nd = (l == 1) ? c->nodenum_at_cell(start_end_node(tq, id, 1), ie)
                                          : c->nodenum_at_cell(start_end_node(tq, id, tq - 1), ie);
                        double dx = c->x_node(i) - c->x_node(nd), dy = c->y_node(i) - c->y_node(nd);
                        double rl = std::sqrt(dx * dx + dy * dy);
                        double uvel1 = (u_node(k, i) + u_node(k - 1, i)) * 0.5;
                        double uvel2 = (u_node(k, nd) + u_node(k - 1, nd)) * 0.5;
                        double vvel1 = (v_node(k, i) + v_node(k - 1, i)) * 0.5;
                        double vvel2 = (v_node(k, nd) + v_node(k - 1, nd)) * 0.5;
                        double du = uvel1 - uvel2, dv = vvel1 - vvel2;
                        double dev = std::sqrt(du * du + dv * dv) / rl * dt;
                        if (dev > devm) devm = dev;
                    }
                    double velo_w = (w_node(k, i) + w_node(k - 1, i)) * 0.5;
                    int iw = (int)(2 * velo_w * dt / p.delta_z_min);
                    int idelta = std::max((int)(devm / F(1.e-1f)), iw);
                    summ = summ + (double)idelta / nadj;
                }
                nsub(k, i) = std::max(p.elm_min_iter, std::min(p.elm_max_iter, (int)summ));
            }
        }
    }
    // :94-201 face loop; after an error the remaining faces are skipped (the serial run stops)
    std::atomic<int> rc{GOM_OK};
    OMP_FOR
    for (int j = 1; j <= c->NF; ++j) {
        if (rc.load(std::memory_order_relaxed) != GOM_OK) continue;
        int n1 = c->nodenum_at_face(1, j), n2 = c->nodenum_at_face(2, j);
        double adv_turn_off_depth = std::max(c->h_node(n1), c->h_node(n2));
        int b = c->bottom_layer_at_face(j), t = top_f(j);
        if (std::fabs(adv_turn_off_depth) < p.adv_onoff_depth) {
            for (int k = b; k <= t; ++k) {
                un_ELM(k, j) = un_face(k, j);
                vn_ELM(k, j) = vn_face(k, j);
            }
            continue;
        }
        int a1 = c->adj_cellnum_at_face(1, j), a2 = c->adj_cellnum_at_face(2, j);
        int ie0;
        if (top_el(a1) != 0) ie0 = a1;
        else if (a2 != 0 && top_el(a2) != 0) ie0 = a2;
        else {
            for (int k = b; k <= t; ++k) {
                un_ELM(k, j) = un_face(k, j);
                vn_ELM(k, j) = vn_face(k, j);
            }
            continue;
        }
        for (int k = b; k <= t; ++k) {
            int nnel = ie0, jlev = k;
            double x0 = c->x_face(j), y0 = c->y_face(j), z0;
            if (k == top_el(nnel)) z0 = p.msl + eta_cell(nnel) - dz_cell(k, nnel) * 0.5;
            else z0 = c->zl(k) - dz_cell(k, nnel) * 0.5;
            double uuint = un_face(k, j) * c->cos_theta(j) - vn_face(k, j) * c->sin_theta(j);
            double vvint = un_face(k, j) * c->sin_theta(j) + vn_face(k, j) * c->cos_theta(j);
            double wdown = (w_node(k - 1, n1) + w_node(k - 1, n2)) * 0.5;
            double wup = (w_node(k, n1) + w_node(k, n2)) * 0.5;
            double wwint = (wdown + wup) * 0.5;
            double vmag = std::sqrt(uuint * uuint + vvint * vvint + wwint * wwint);
            if (vmag <= F(1.e-4f)) {
                un_ELM(k, j) = un_face(k, j);
                vn_ELM(k, j) = vn_face(k, j);
            } else {
                int bt_step = (int)((double)(nsub(k, n1) + nsub(k, n2)) * 0.5);
                double bt_dt = p.dt / bt_step;
                int ne = 0;
                int e = elm_backtrace(c, bt_step, bt_dt, uuint, vvint, wwint, x0, y0, z0, nnel, jlev, ne);
                if (e) {
                    set_err(c, GOM_E_ELM, e, j, k, 0.0, GOM_ENTITY_FACE);
                    rc = GOM_E_ELM;
                    break;
                }
                foot(k, j) = nnel;
                near(k, j) = ne;
                un_ELM(k, j) = uuint * c->cos_theta(j) + vvint * c->sin_theta(j);
                vn_ELM(k, j) = -uuint * c->sin_theta(j) + vvint * c->cos_theta(j);
            }
        }
    }
    return rc.load();
}

// solve_momentum_equation.f90:15-656
int gom_step_momentum(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    const gom_params &p = c->p;
    const int L = c->L;
    const double dt = p.dt, gravity = p.gravity, theta = p.theta;
    A2<double> AinvG1 = FD(c, GOM_F_AINVG1), AinvG2 = FD(c, GOM_F_AINVG2), AinvDZ1 = FD(c, GOM_F_AINVDZ1),
               AinvDZ2 = FD(c, GOM_F_AINVDZ2), Kh = FD(c, GOM_F_KH);
    A2<double> dz_face = FD(c, GOM_F_DZ_FACE), dzhalf_face = FD(c, GOM_F_DZHALF_FACE), Av = FD(c, GOM_F_AV);
    A2<double> un_face = FD(c, GOM_F_UN_FACE), vn_face = FD(c, GOM_F_VN_FACE), un_ELM = FD(c, GOM_F_UN_ELM),
               vn_ELM = FD(c, GOM_F_VN_ELM), u_node = FD(c, GOM_F_U_NODE), v_node = FD(c, GOM_F_V_NODE),
               rho_cell = FD(c, GOM_F_RHO_CELL), rho_node = FD(c, GOM_F_RHO_NODE);
    A1<double> eta_cell = FD1(c, GOM_F_ETA_CELL), eta_node = FD1(c, GOM_F_ETA_NODE), Gamma_B = FD1(c, GOM_F_GAMMA_B),
               Qu = FD1(c, GOM_F_QU_BOUNDARY);
    A1<int32_t> top_f = FI1(c, GOM_F_TOP_LAYER_FACE), top_el = FI1(c, GOM_F_TOP_LAYER_CELL),
                top_n = FI1(c, GOM_F_TOP_LAYER_NODE), wetdry = FI1(c, GOM_F_WETDRY_NODE);
    std::fill(c->fd[GOM_F_AINVG1].begin(), c->fd[GOM_F_AINVG1].end(), 0.0);
    std::fill(c->fd[GOM_F_AINVG2].begin(), c->fd[GOM_F_AINVG2].end(), 0.0);
    std::fill(c->fd[GOM_F_AINVDZ1].begin(), c->fd[GOM_F_AINVDZ1].end(), 0.0);
    std::fill(c->fd[GOM_F_AINVDZ2].begin(), c->fd[GOM_F_AINVDZ2].end(), 0.0);
    const int nmax = L + 1;
    // each packed run starts with rtemp0 = 0, as one call of the reference does
    std::vector<char> run_first_face(c->NF + 2, 0);
    for (size_t r = 0; r + 1 < c->run_face_start.size(); ++r) run_first_face[c->run_face_start[r] + 1] = 1;
    double rtemp0 = 0.0;
    const double c069 = F(0.69f);
    std::atomic<int> rc{GOM_OK};
    OMP_FOR_FIRSTPRIVATE(rtemp0)
    for (int j = 1; j <= c->NF; ++j) {
        if (run_first_face[j]) rtemp0 = 0.0;
        if (rc.load(std::memory_order_relaxed) != GOM_OK) continue;
        if (top_f(j) == 0) continue;
        double G1[GOM_ORACLE_MAXL + 1] = {0}, G2[GOM_ORACLE_MAXL + 1] = {0}, a[GOM_ORACLE_MAXL + 1] = {0},
               bd[GOM_ORACLE_MAXL + 1] = {0}, cu[GOM_ORACLE_MAXL + 1] = {0}, gam[GOM_ORACLE_MAXL + 1] = {0};
        double rhs[(GOM_ORACLE_MAXL + 1) * 3] = {0}, sol[(GOM_ORACLE_MAXL + 1) * 3] = {0};
        double temp[12] = {0};
        double rtemp1 = 0.0, rtemp2 = 0.0, rtemp3 = 0.0, rtemp4 = 0.0;
        int node1 = c->nodenum_at_face(1, j), node2 = c->nodenum_at_face(2, j);
        int tj = top_f(j), bj = c->bottom_layer_at_face(j);
        int nvl = tj - bj + 1;
        int a1 = c->adj_cellnum_at_face(1, j), a2 = c->adj_cellnum_at_face(2, j);
        int btype = c->boundary_type_of_face(j);
        // :120-169 matrix
        for (int k = bj + 1; k <= tj - 1; ++k) {
            int kk = tj - k + 1;
            a[kk - 1] = -dt * Av(k, j) / dzhalf_face(k, j);
            cu[kk - 1] = -dt * Av(k - 1, j) / dzhalf_face(k - 1, j);
            bd[kk - 1] = -a[kk - 1] + dz_face(k, j) - cu[kk - 1];
        }
        if (tj == bj) {
            bd[0] = dz_face(tj, j) + Gamma_B(j) * dt;
        } else {
            cu[0] = -dt * Av(tj - 1, j) / dzhalf_face(tj - 1, j);
            bd[0] = c->gamma_t[j - 1] * dt + dz_face(tj, j) - cu[0];
            a[nvl - 1] = -dt * Av(bj, j) / dzhalf_face(bj, j);
            bd[nvl - 1] = -a[nvl - 1] + dz_face(bj, j) + Gamma_B(j) * dt;
        }
        // :173-216 earth tide: not configured (no_Etide_species = 0)
        double detp_dx = 0.0, detp_dy = 0.0;
        for (int k = 1; k <= nvl; ++k) {
            int kk = tj - k + 1;
            G1[k - 1] = dz_face(kk, j) * (un_ELM(kk, j) + c->coriolis_factor(j) * dt * vn_face(kk, j));
            G2[k - 1] = dz_face(kk, j) * (vn_ELM(kk, j) - c->coriolis_factor(j) * dt * un_face(kk, j));
            if (a2 != 0) {
                // :269-301
                for (int l = 1; l <= 2; ++l) {
                    int nd = c->nodenum_at_face(l, j);
                    double utmp = (u_node(kk, nd) + u_node(kk - 1, nd)) * 0.5;
                    double vtmp = (v_node(kk, nd) + v_node(kk - 1, nd)) * 0.5;
                    temp[2 * l - 2] = utmp * c->cos_theta(j) + vtmp * c->sin_theta(j);
                    temp[2 * l - 1] = -utmp * c->sin_theta(j) + vtmp * c->cos_theta(j);
                }
                for (int l = 1; l <= 2; ++l) {
                    int ie = c->adj_cellnum_at_face(l, j);
                    double utmp = 0.0, vtmp = 0.0;
                    int tq = c->tri_or_quad(ie);
                    for (int ll = 1; ll <= tq; ++ll) {
                        int nd = c->nodenum_at_cell(ll, ie);
                        utmp = utmp + (u_node(kk, nd) + u_node(kk - 1, nd)) * 0.5 / tq;
                        vtmp = vtmp + (v_node(kk, nd) + v_node(kk - 1, nd)) * 0.5 / tq;
                    }
                    temp[2 * l + 2] = utmp * c->cos_theta(j) + vtmp * c->sin_theta(j);
                    temp[2 * l + 3] = -utmp * c->sin_theta(j) + vtmp * c->cos_theta(j);
                }
                double dudx = (temp[6] - temp[4]) / c->delta_j(j);
                double dvdx = (temp[7] - temp[5]) / c->delta_j(j);
                double dudy = (temp[2] - temp[0]) / c->face_length(j);
                double dvdy = (temp[3] - temp[1]) / c->face_length(j);
                double s = dvdx + dudy;
                double hdiff = p.smagorinsky * std::sqrt(dudx * dudx + dvdy * dvdy + 0.5 * (s * s));
                Kh(k, j) = hdiff * c->area(a1);
                hdiff = hdiff + p.ah_0;
                Kh(k, j) = Kh(k, j) + p.kh_0;
                double fl = c->face_length(j);
                double d2udy = 4.0 * (temp[2] + temp[0] - 2 * un_face(kk, j)) / (fl * fl);
                double d2vdy = 4.0 * (temp[3] + temp[1] - 2 * vn_face(kk, j)) / (fl * fl);
                for (int l = 1; l <= 2; ++l) {
                    int ie = c->adj_cellnum_at_face(l, j);
                    double ddx = c->x_cell(ie) - c->x_face(j), ddy = c->y_cell(ie) - c->y_face(j);
                    double rl = std::sqrt(ddx * ddx + ddy * ddy);
                    temp[2 * l + 6] = (temp[2 * l + 2] - un_face(kk, j)) / rl;
                    temp[2 * l + 7] = (temp[2 * l + 3] - vn_face(kk, j)) / rl;
                }
                double d2udx = 2.0 * (temp[8] + temp[10]) / c->delta_j(j);
                double d2vdx = 2.0 * (temp[9] + temp[11]) / c->delta_j(j);
                G1[k - 1] = G1[k - 1] + dz_face(kk, j) * dt * hdiff * (d2udx + d2udy);
                G2[k - 1] = G2[k - 1] + dz_face(kk, j) * dt * hdiff * (d2vdx + d2vdy);
            }
            // :350-376 barotropic gradient, (1-theta) part
            if (btype == 0) {
                rtemp0 = gravity * dt / c->delta_j(j) * (1.0 - theta) * (eta_cell(a2) - eta_cell(a1));
                rtemp1 = rtemp0 * c->cos_theta2(j);
                rtemp2 = rtemp0 * c->sin_theta2(j);
                G1[k - 1] = G1[k - 1] - dz_face(kk, j) * rtemp1;
            } else if (btype > 0) {
                int ie = c->ob_element_flag(a1);
                rtemp1 = gravity * dt / c->delta_j(j) * (1.0 - theta) * (c->eta_at_ob_old[ie - 1] - eta_cell(a1));
                G1[k - 1] = G1[k - 1] - dz_face(kk, j) * rtemp1;
            } else if (btype == -1) {
                G1[k - 1] = 0.0;
            }
            // :380-397
            if (wetdry(node1) == 0 && wetdry(node2) == 0) {
                rtemp0 = gravity * dt / c->face_length(j) * (1.0 - theta) * (eta_node(node2) - eta_node(node1));
                if (btype == 0) G2[k - 1] = G2[k - 1] - dz_face(kk, j) * (rtemp0 + rtemp2);
                else G2[k - 1] = G2[k - 1] - dz_face(kk, j) * rtemp0;
            }
            // :400-471 baroclinic
            if (p.baroclinic_flag == 1) {
                double sum1 = 0.0, sum2 = 0.0;
                for (int k2 = kk; k2 <= tj; ++k2) {
                    if (a2 != 0 && k2 >= c->bottom_layer_at_element(a1) && k2 <= top_el(a1) &&
                        k2 >= c->bottom_layer_at_element(a2) && k2 <= top_el(a2)) {
                        if (k2 == kk)
                            sum1 = sum1 + 0.5 * (rho_cell(k2, a2) - rho_cell(k2, a1)) * dz_face(k2, j);
                        else
                            sum1 = sum1 + 1.0 * (rho_cell(k2, a2) - rho_cell(k2, a1)) * dz_face(k2, j);
                    }
                    if (k2 >= c->bottom_layer_at_node(node1) && k2 <= top_n(node1) &&
                        k2 >= c->bottom_layer_at_node(node2) && k2 <= top_n(node2)) {
                        if (k2 == kk) sum2 = sum2 + 0.5 * (rho_node(k2, node2) - rho_node(k2, node1)) * dz_face(k2, j);
                        else sum2 = sum2 + 1.0 * (rho_node(k2, node2) - rho_node(k2, node1)) * dz_face(k2, j);
                    }
                }
                // the reference indexes dz_face with the top-down row k here (:455-456)
                rtemp1 = dz_face(k, j) * (-gravity * dt / (p.rho_o * c->delta_j(j))) * sum1;
                rtemp2 = dz_face(k, j) * (-gravity * dt / (p.rho_o * c->face_length(j))) * sum2;
                rtemp3 = rtemp1 * c->cos_theta2(j);
                rtemp4 = rtemp1 * c->sin_theta2(j);
                G1[k - 1] = G1[k - 1] + rtemp3 * c->spinup_baroclinic;
                G2[k - 1] = G2[k - 1] + (rtemp2 + rtemp4) * c->spinup_baroclinic;
            }
            // :474-477 wind at the top row
            if (k == 1) {
                G1[k - 1] = G1[k - 1] + dt * c->wind_stress_normal[j - 1];
                G2[k - 1] = G2[k - 1] + dt * c->wind_stress_tangnt[j - 1];
            }
            // :485-486 earth tide gradient (zero here)
            G1[k - 1] = G1[k - 1] + c069 * dz_face(kk, j) * gravity * dt * detp_dx;
            G2[k - 1] = G2[k - 1] + c069 * dz_face(kk, j) * gravity * dt * detp_dy;
            // :490-509 air pressure; on boundary faces rtemp0 is the value left from before
            if (a2 != 0) {
                for (int l = 1; l <= 2; ++l) {
                    temp[l - 1] = 0.0;
                    int ie = c->adj_cellnum_at_face(l, j);
                    int tq = c->tri_or_quad(ie);
                    for (int ll = 1; ll <= tq; ++ll)
                        temp[l - 1] = temp[l - 1] + c->air_p[c->nodenum_at_cell(ll, ie) - 1] / tq;
                }
                rtemp0 = -dt / p.rho_o * (temp[1] - temp[0]) / c->delta_j(j);
            }
            rtemp1 = rtemp0 * c->cos_theta2(j);
            rtemp2 = rtemp0 * c->sin_theta2(j);
            G1[k - 1] = G1[k - 1] + dz_face(kk, j) * rtemp1;
            rtemp3 = -dt / p.rho_o * ((c->air_p[node2 - 1] - c->air_p[node1 - 1]) / c->face_length(j));
            G2[k - 1] = G2[k - 1] + dz_face(kk, j) * (rtemp3 + rtemp2);
            // :519-535 (isflowside is never set; the land branch applies)
            if (btype == -1) G1[k - 1] = 0.0;
            // :544-551 river
            if (c->isflowside3(j) > 0) {
                int ibnd = c->isflowside3(j);
                G1[k - 1] = G1[k - 1] + dz_face(kk, j) * Qu(ibnd);
            }
            rhs[0 * nmax + k - 1] = G1[k - 1];
            rhs[1 * nmax + k - 1] = G2[k - 1];
            rhs[2 * nmax + k - 1] = dz_face(kk, j);
        }
        if (!tridiagonal_solver(nmax, nvl, 3, a, bd, cu, rhs, sol, gam)) {
            set_err(c, GOM_E_ZERO_PIVOT, 587, j, 0, 0.0, GOM_ENTITY_FACE);
            rc = GOM_E_ZERO_PIVOT;
            continue;
        }
        for (int k = 1; k <= nvl; ++k) {
            AinvG1(k, j) = sol[0 * nmax + k - 1];
            AinvG2(k, j) = sol[1 * nmax + k - 1];
        }
        if (btype == -1 && c->isflowside3(j) == 0)
            for (int k = 1; k <= nvl; ++k) AinvG1(k, j) = 0.0;
        for (int k = 1; k <= nvl; ++k) {
            AinvDZ1(k, j) = sol[2 * nmax + k - 1];
            AinvDZ2(k, j) = sol[2 * nmax + k - 1];
        }
        if (btype == -1)
            for (int k = 1; k <= nvl; ++k) AinvDZ1(k, j) = 0.0;
    }
    return rc.load();
}

// solve_free_surface_equation.f90:17-396 with pre_conj_grad.f90:9-230 (serial, CSR order)
int gom_step_free_surface(gom_ctx *c, int32_t *pcg_iters) {
    if (!c) return GOM_E_ARG;
    const gom_params &p = c->p;
    const double dt = p.dt, gravity = p.gravity, theta = p.theta;
    const int NC = c->NC;
    A2<double> dz_face = FD(c, GOM_F_DZ_FACE), AinvDZ1 = FD(c, GOM_F_AINVDZ1), AinvG1 = FD(c, GOM_F_AINVG1),
               un_face = FD(c, GOM_F_UN_FACE);
    A1<double> eta_cell = FD1(c, GOM_F_ETA_CELL), eta_new = FD1(c, GOM_F_ETA_CELL_NEW), eta_node = FD1(c, GOM_F_ETA_NODE);
    A1<int32_t> top_f = FI1(c, GOM_F_TOP_LAYER_FACE), top_el = FI1(c, GOM_F_TOP_LAYER_CELL),
                wetdry = FI1(c, GOM_F_WETDRY_NODE);
    std::vector<double> sparsem(5 * (size_t)NC, 0.0), rhs_1(NC, 0.0);
    auto SP = [&](int l, int i) -> double & { return sparsem[(size_t)(i - 1) * 5 + l]; };
    std::atomic<int> rc{GOM_OK};
    OMP_FOR
    for (int i = 1; i <= NC; ++i) {
        if (rc.load(std::memory_order_relaxed) != GOM_OK) continue;
        SP(0, i) = c->area(i);
        int tq = c->tri_or_quad(i);
        for (int l = 1; l <= tq; ++l) {
            int ii = c->adj_cellnum_at_cell(l, i);
            int j = c->facenum_at_cell(l, i);
            if (top_f(j) != 0) {
                double s = 0.0;
                int nvl = top_f(j) - c->bottom_layer_at_face(j) + 1;
                for (int k = 1; k <= nvl; ++k) s = s + dz_face(top_f(j) + 1 - k, j) * AinvDZ1(k, j);
                s = gravity * (dt * dt) * (theta * theta) * c->face_length(j) / c->delta_j(j) * s;
                s = s * c->cos_theta2(j);
                if (s < 0.0) {
                    set_err(c, GOM_E_NOT_SPD, 100, i, 0, s, GOM_ENTITY_CELL);
                    rc = GOM_E_NOT_SPD;
                    break;
                }
                SP(0, i) = SP(0, i) + s;
                if (ii != 0) SP(l, i) = -s;
            }
        }
        if (rc.load(std::memory_order_relaxed) != GOM_OK) continue;
        rhs_1[i - 1] = c->area(i) * eta_cell(i);
        for (int l = 1; l <= tq; ++l) {
            int j = c->facenum_at_cell(l, i);
            if (top_f(j) != 0) {
                double const1 = 0.0, const2 = 0.0;
                int nvl = top_f(j) - c->bottom_layer_at_face(j) + 1;
                for (int k = 1; k <= nvl; ++k) {
                    int kk = top_f(j) + 1 - k;
                    const1 = const1 + dz_face(kk, j) * un_face(kk, j);
                    const2 = const2 + dz_face(kk, j) * AinvG1(k, j);
                }
                double sgn = (double)c->sign_in_outflow(l, i);
                rhs_1[i - 1] = rhs_1[i - 1] - (1.0 - theta) * dt * sgn * c->face_length(j) * const1 -
                               theta * dt * sgn * c->face_length(j) * const2;
            }
        }
        if (c->ob_element_flag(i) > 0) {
            for (int l = 1; l <= tq; ++l) {
                int j = c->facenum_at_cell(l, i);
                if (c->boundary_type_of_face(j) > 0 && top_f(j) != 0) {
                    double s = 0.0;
                    int nvl = top_f(j) - c->bottom_layer_at_face(j) + 1;
                    for (int k = 1; k <= nvl; ++k) s = s + dz_face(top_f(j) + 1 - k, j) * AinvDZ1(k, j);
                    s = gravity * (dt * dt) * (theta * theta) * c->face_length(j) / c->delta_j(j) * s;
                    rhs_1[i - 1] = rhs_1[i - 1] + s * c->eta_at_ob_new[c->ob_element_flag(i) - 1];
                }
            }
        }
    }
    if (rc.load() != GOM_OK) return rc.load();
    // CSR (:233-258): diagonal first, then neighbours in local order (serial, as in the reference)
    std::vector<int> ia(NC + 1), ja;
    std::vector<double> a1;
    ja.reserve(5 * (size_t)NC);
    a1.reserve(5 * (size_t)NC);
    std::vector<double> x(NC);
    for (int i = 1; i <= NC; ++i) {
        ia[i - 1] = (int)ja.size();
        ja.push_back(i);
        a1.push_back(SP(0, i));
        x[i - 1] = eta_new(i);
        for (int l = 1; l <= c->tri_or_quad(i); ++l) {
            int ii = c->adj_cellnum_at_cell(l, i);
            if (ii != 0) {
                ja.push_back(ii);
                a1.push_back(SP(l, i));
            }
        }
    }
    ia[NC] = (int)ja.size();
    // pre_conj_grad.f90:46-221, once per packed run on that run's rows (the system is block
    // diagonal across runs); a context with one run is the reference's single solve
    std::vector<double> Minv(NC), r(NC), d(NC), q(NC), s(NC);
    int cgit2 = 0;
    const int nruns = (int)c->run_cell_start.size() - 1;
    for (int run = 0; run < nruns; ++run) {
        const int i0 = c->run_cell_start[run], i1 = c->run_cell_start[run + 1];
        OMP_FOR
        for (int i = i0; i < i1; ++i) {
            double sum1 = 0.0;
            for (int k = ia[i]; k < ia[i + 1]; ++k) {
                if (ja[k] == i + 1) Minv[i] = 1.0 / a1[k];
                sum1 = sum1 + a1[k] * x[ja[k] - 1];
            }
            r[i] = rhs_1[i] - sum1;
        }
        OMP_FOR
        for (int i = i0; i < i1; ++i) d[i] = Minv[i] * r[i];
        double delta_new = 0.0;
        OMP_FOR_SUM(delta_new)
        for (int i = i0; i < i1; ++i) delta_new = delta_new + r[i] * d[i];
        double delta_0 = delta_new;
        int run_it = 0;
        // A zero initial residual would make the reference divide 0 by 0 (alpha = delta/dq);
        // the restatement returns the initial guess instead.
        if (delta_0 != 0.0) {
            for (int cgit = 1; cgit <= p.max_iteration_pcg; ++cgit) {
                OMP_FOR
                for (int i = i0; i < i1; ++i) {
                    double sum1 = 0.0;
                    for (int k = ia[i]; k < ia[i + 1]; ++k) sum1 = sum1 + a1[k] * d[ja[k] - 1];
                    q[i] = sum1;
                }
                double dq = 0.0;
                OMP_FOR_SUM(dq)
                for (int i = i0; i < i1; ++i) dq = dq + d[i] * q[i];
                double alpha = delta_new / dq;
                OMP_FOR
                for (int i = i0; i < i1; ++i) {
                    x[i] = x[i] + alpha * d[i];
                    r[i] = r[i] - alpha * q[i];
                }
                OMP_FOR
                for (int i = i0; i < i1; ++i) s[i] = Minv[i] * r[i];
                double delta_old = delta_new;
                delta_new = 0.0;
                OMP_FOR_SUM(delta_new)
                for (int i = i0; i < i1; ++i) delta_new = delta_new + r[i] * s[i];
                double beta = delta_new / delta_old;
                OMP_FOR
                for (int i = i0; i < i1; ++i) d[i] = s[i] + beta * d[i];
                run_it = cgit;
                if (std::sqrt(delta_new * delta_new / (delta_0 * delta_0)) < p.error_tolerance) break;
            }
        }
        cgit2 = std::max(cgit2, run_it);
    }
    if (pcg_iters) *pcg_iters = cgit2;
    c->pcg_total += cgit2;
    for (int i = 1; i <= NC; ++i) eta_new(i) = x[i - 1];
    // :353-396 node elevation and wet/dry nodes
    OMP_FOR
    for (int i = 1; i <= c->NN; ++i) {
        wetdry(i) = 0;
        double sum1 = 0.0, sum0 = 0.0;
        for (int j = 1; j <= c->adj_cells_at_node(i); ++j) {
            int ie = c->adj_cellnum_at_node(j, i);
            if (top_el(ie) == 0) wetdry(i) = 1;
            else {
                sum1 = sum1 + c->area(ie) * eta_new(ie);
                sum0 = sum0 + c->area(ie);
            }
        }
        if (wetdry(i) == 0) eta_node(i) = sum1 / sum0;
    }
    OMP_FOR
    for (int i = 1; i <= c->NN; ++i) {
        if (wetdry(i) == 1) {
            double sum0 = 0.0;
            int icount = 0;
            for (int j = 1; j <= c->adj_nodes_at_node(i); ++j) {
                int nd = c->adj_nodenum_at_node(j, i);
                if (wetdry(nd) == 0) {
                    icount = icount + 1;
                    sum0 = sum0 + eta_node(nd);
                }
            }
            if (icount != 0) eta_node(i) = sum0 / icount;
        }
    }
    return GOM_OK;
}

// solve_velocities.f90:8-260
int gom_step_velocities(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    const gom_params &p = c->p;
    const int L = c->L;
    const double dt = p.dt, gravity = p.gravity, theta = p.theta;
    A2<double> un_new = FD(c, GOM_F_UN_FACE_NEW), vn_new = FD(c, GOM_F_VN_FACE_NEW), AinvG1 = FD(c, GOM_F_AINVG1),
               AinvG2 = FD(c, GOM_F_AINVG2), AinvDZ1 = FD(c, GOM_F_AINVDZ1), AinvDZ2 = FD(c, GOM_F_AINVDZ2),
               wn_new = FD(c, GOM_F_WN_CELL_NEW), dz_face = FD(c, GOM_F_DZ_FACE);
    A1<double> eta_new = FD1(c, GOM_F_ETA_CELL_NEW), eta_node = FD1(c, GOM_F_ETA_NODE), Qu = FD1(c, GOM_F_QU_BOUNDARY);
    A1<int32_t> top_f = FI1(c, GOM_F_TOP_LAYER_FACE), top_el = FI1(c, GOM_F_TOP_LAYER_CELL),
                wetdry = FI1(c, GOM_F_WETDRY_NODE);
    OMP_FOR
    for (int j = 1; j <= c->NF; ++j) {
        int n1 = c->nodenum_at_face(1, j), n2 = c->nodenum_at_face(2, j);
        int tj = top_f(j), bj = c->bottom_layer_at_face(j);
        int btype = c->boundary_type_of_face(j);
        if (tj == 0) {
            for (int k = 1; k <= L; ++k) {
                un_new(k, j) = 0.0;
                vn_new(k, j) = 0.0;
            }
            continue;
        }
        double rtemp2 = 0.0;
        for (int k = 1; k <= tj - bj + 1; ++k) {
            int kk = tj + 1 - k;
            if (btype == -1) {
                un_new(kk, j) = 0.0;
            } else if (btype == 0) {
                int a1 = c->adj_cellnum_at_face(1, j), a2 = c->adj_cellnum_at_face(2, j);
                double rtemp0 = theta * gravity * dt / c->delta_j(j) * (eta_new(a2) - eta_new(a1)) * AinvDZ1(k, j);
                double rtemp1 = rtemp0 * c->cos_theta2(j);
                rtemp2 = rtemp0 * c->sin_theta2(j);
                un_new(kk, j) = AinvG1(k, j) - rtemp1;
            } else {
                int a1 = c->adj_cellnum_at_face(1, j);
                double rtemp0 = theta * gravity * dt / c->delta_j(j) *
                                (c->eta_at_ob_new[c->ob_element_flag(a1) - 1] - eta_new(a1)) * AinvDZ1(k, j);
                un_new(kk, j) = AinvG1(k, j) - rtemp0;
            }
            if (wetdry(n1) == 0 && wetdry(n2) == 0) {
                double rtemp1 = theta * gravity * dt / c->face_length(j) * (eta_node(n2) - eta_node(n1)) * AinvDZ2(k, j);
                if (btype == 0) vn_new(kk, j) = AinvG2(k, j) - (rtemp1 + rtemp2);
                else vn_new(kk, j) = AinvG2(k, j) - rtemp1;
            }
            if (c->initial_wetdry_node(n1) == 1 || c->initial_wetdry_node(n2) == 1)
                vn_new(kk, j) = std::max(-5.0, std::min(vn_new(kk, j), 5.0));
        }
        if (c->isflowside3(j) > 0) {
            int ibnd = c->isflowside3(j);
            for (int k = bj; k <= tj; ++k) un_new(k, j) = Qu(ibnd);
        }
        for (int k = 1; k <= bj - 1; ++k) {
            un_new(k, j) = 0.0;
            vn_new(k, j) = 0.0;
        }
        for (int k = tj + 1; k <= L; ++k) {
            un_new(k, j) = un_new(tj, j);
            vn_new(k, j) = vn_new(tj, j);
        }
    }
    OMP_FOR
    for (int i = 1; i <= c->NC; ++i) {
        int t = top_el(i), b = c->bottom_layer_at_element(i);
        if (t == 0) {
            for (int k = 0; k <= L; ++k) wn_new(k, i) = 0.0;
            continue;
        }
        wn_new(b - 1, i) = 0.0;
        for (int k = b; k <= t; ++k) {
            double sum1 = 0.0;
            for (int l = 1; l <= c->tri_or_quad(i); ++l) {
                int jt = c->facenum_at_cell(l, i);
                if (k >= c->bottom_layer_at_face(jt) && k <= top_f(jt))
                    sum1 = sum1 + (double)c->sign_in_outflow(l, i) * c->face_length(jt) * dz_face(k, jt) * un_new(k, jt);
            }
            wn_new(k, i) = wn_new(k - 1, i) - sum1 / c->area(i);
        }
        for (int k = 0; k <= b - 2; ++k) wn_new(k, i) = 0.0;
        for (int k = t + 1; k <= L; ++k) wn_new(k, i) = wn_new(t, i);
    }
    return GOM_OK;
}

// update_vertical_layers_1.f90:18-333
int gom_step_layers(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    const gom_params &p = c->p;
    const int L = c->L;
    const double MSL = p.msl;
    A2<double> dz_cn = FD(c, GOM_F_DZ_CELL_NEW), dzh_cn = FD(c, GOM_F_DZHALF_CELL_NEW), wn_new = FD(c, GOM_F_WN_CELL_NEW),
               dz_fn = FD(c, GOM_F_DZ_FACE_NEW), dzh_fn = FD(c, GOM_F_DZHALF_FACE_NEW), dz_nn = FD(c, GOM_F_DZ_NODE_NEW),
               dzh_nn = FD(c, GOM_F_DZHALF_NODE_NEW);
    A1<double> eta_new = FD1(c, GOM_F_ETA_CELL_NEW), eta_node = FD1(c, GOM_F_ETA_NODE);
    A1<int32_t> top_el = FI1(c, GOM_F_TOP_LAYER_CELL), top_f = FI1(c, GOM_F_TOP_LAYER_FACE),
                top_n = FI1(c, GOM_F_TOP_LAYER_NODE);
    for (int i = 1; i <= c->NC; ++i) {
        int tnew = 0;
        double total = c->h_cell(i) + eta_new(i);
        int b = c->bottom_layer_at_element(i);
        if (total > p.dry_depth) {
            double tmp = MSL + eta_new(i);
            for (int k = L - 1; k >= 0; --k)
                if (tmp > c->zl(k) && tmp <= c->zl(k + 1)) {
                    tnew = k + 1;
                    dz_cn(tnew, i) = tmp - c->zl(k);
                    break;
                }
            if (tnew < b) {
                set_err(c, GOM_E_LAYER, 66, i, tnew, eta_new(i), GOM_ENTITY_CELL);
                return GOM_E_LAYER;
            }
            if (tnew == b) {
                dz_cn(tnew, i) = total;
                dzh_cn(tnew, i) = total;
            } else {
                dz_cn(b, i) = c->zl(b) - (MSL - c->h_cell(i));
                for (int k = b + 1; k <= tnew - 1; ++k) dz_cn(k, i) = c->delta_z(k);
                for (int k = b; k <= tnew - 1; ++k) dzh_cn(k, i) = (dz_cn(k + 1, i) + dz_cn(k, i)) * 0.5;
                dzh_cn(tnew, i) = dz_cn(tnew, i);
                dzh_cn(b - 1, i) = dz_cn(b, i);
            }
        }
        if (top_el(i) == 0 && tnew != 0)
            for (int k = 0; k <= L; ++k) wn_new(k, i) = 0.0;
        top_el(i) = tnew;
    }
    for (int j = 1; j <= c->NF; ++j) {
        int tnew = 0;
        int a1 = c->adj_cellnum_at_face(1, j), a2 = c->adj_cellnum_at_face(2, j);
        double eta_max = (a2 != 0) ? std::max(eta_new(a1), eta_new(a2)) : eta_new(a1);
        double total = c->h_face(j) + eta_max;
        int b = c->bottom_layer_at_face(j);
        if (total > p.dry_depth) {
            double tmp = MSL + eta_max;
            for (int k = L - 1; k >= 0; --k)
                if (tmp > c->zl(k) && tmp <= c->zl(k + 1)) {
                    tnew = k + 1;
                    dz_fn(tnew, j) = tmp - c->zl(k);
                    break;
                }
            if (tnew < b) {
                set_err(c, GOM_E_LAYER, 166, j, tnew, eta_max, GOM_ENTITY_FACE);
                return GOM_E_LAYER;
            }
            if (tnew == b) {
                dz_fn(tnew, j) = total;
                dzh_fn(tnew - 1, j) = total;
                dzh_fn(tnew, j) = total;
            } else {
                dz_fn(b, j) = c->zl(b) - (MSL - c->h_face(j));
                for (int k = b + 1; k <= tnew - 1; ++k) dz_fn(k, j) = c->delta_z(k);
                for (int k = b; k <= tnew - 1; ++k) dzh_fn(k, j) = (dz_fn(k + 1, j) + dz_fn(k, j)) * 0.5;
                dzh_fn(tnew, j) = dz_fn(tnew, j);
                dzh_fn(b - 1, j) = dz_fn(b, j);
            }
        }
        top_f(j) = tnew;
    }
    for (int i = 1; i <= c->NN; ++i) {
        int tnew = 0;
        double total = c->h_node(i) + eta_node(i);
        int b = c->bottom_layer_at_node(i);
        if (total > p.dry_depth) {
            double tmp = MSL + eta_node(i);
            for (int k = L - 1; k >= 0; --k)
                if (tmp > c->zl(k) && tmp <= c->zl(k + 1)) {
                    tnew = k + 1;
                    dz_nn(tnew, i) = tmp - c->zl(k);
                    break;
                }
            if (tnew < b) {
                set_err(c, GOM_E_LAYER, 224, i, tnew, eta_node(i), GOM_ENTITY_NODE);
                return GOM_E_LAYER;
            }
            if (tnew == b) {
                dz_nn(tnew, i) = total;
                dzh_nn(tnew, i) = total;
            } else {
                dz_nn(b, i) = c->zl(b) - (MSL - c->h_node(i));
                for (int k = b + 1; k <= tnew - 1; ++k) dz_nn(k, i) = c->delta_z(k);
                for (int k = b; k <= tnew - 1; ++k) dzh_nn(k, i) = (dz_nn(k + 1, i) + dz_nn(k, i)) * 0.5;
            }
        }
        top_n(i) = tnew;
    }
    for (int i = 1; i <= c->NC; ++i) {
        int nsum1 = 0, nsum2 = 0;
        for (int l = 1; l <= c->tri_or_quad(i); ++l) {
            nsum1 = nsum1 + top_n(c->nodenum_at_cell(l, i));
            nsum2 = nsum2 + top_f(c->facenum_at_cell(l, i));
        }
        if (nsum1 == 0) top_el(i) = 0;
        if (nsum2 == 0 && top_el(i) != 0) {
            set_err(c, GOM_E_DRY, 273, i, 0, 0.0, GOM_ENTITY_CELL);
            return GOM_E_DRY;
        }
    }
    for (int i = 1; i <= c->NC; ++i)
        for (int k = c->bottom_layer_at_element(i); k <= top_el(i) - 1; ++k)
            if (dzh_cn(k, i) < p.denominator_min_for_matrix) {
                set_err(c, GOM_E_LAYER, 284, i, k, dzh_cn(k, i), GOM_ENTITY_CELL);
                return GOM_E_LAYER;
            }
    for (int j = 1; j <= c->NF; ++j)
        for (int k = c->bottom_layer_at_face(j); k <= top_f(j) - 1; ++k)
            if (dzh_fn(k, j) < p.denominator_min_for_matrix) {
                set_err(c, GOM_E_LAYER, 301, j, k, dzh_fn(k, j), GOM_ENTITY_FACE);
                return GOM_E_LAYER;
            }
    for (int i = 1; i <= c->NN; ++i)
        for (int k = c->bottom_layer_at_node(i); k <= top_n(i) - 1; ++k)
            if (dzh_nn(k, i) < p.denominator_min_for_matrix) {
                set_err(c, GOM_E_LAYER, 318, i, k, dzh_nn(k, i), GOM_ENTITY_NODE);
                return GOM_E_LAYER;
            }
    return GOM_OK;
}

// calculate_velocity_at_node.f90:10-140
int gom_step_node_velocity(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    const int L = c->L;
    A2<double> un_new = FD(c, GOM_F_UN_FACE_NEW), vn_new = FD(c, GOM_F_VN_FACE_NEW), dz_face = FD(c, GOM_F_DZ_FACE),
               dzhalf_face = FD(c, GOM_F_DZHALF_FACE), ufl = FD(c, GOM_F_U_FACE_LEVEL), vfl = FD(c, GOM_F_V_FACE_LEVEL),
               u_node = FD(c, GOM_F_U_NODE), v_node = FD(c, GOM_F_V_NODE), w_node = FD(c, GOM_F_W_NODE),
               wn_cell = FD(c, GOM_F_WN_CELL);
    A1<int32_t> top_f = FI1(c, GOM_F_TOP_LAYER_FACE), top_el = FI1(c, GOM_F_TOP_LAYER_CELL);
    OMP_FOR
    for (int j = 1; j <= c->NF; ++j) {
        int t = top_f(j), b = c->bottom_layer_at_face(j);
        if (t == 0) continue;
        double uf[GOM_ORACLE_MAXL + 2] = {0}, vf[GOM_ORACLE_MAXL + 2] = {0};
        for (int k = b; k <= t; ++k) {
            uf[k] = un_new(k, j) * c->cos_theta(j) - vn_new(k, j) * c->sin_theta(j);
            vf[k] = un_new(k, j) * c->sin_theta(j) + vn_new(k, j) * c->cos_theta(j);
        }
        ufl(b - 1, j) = uf[b];
        vfl(b - 1, j) = vf[b];
        ufl(t, j) = uf[t];
        vfl(t, j) = vf[t];
        for (int k = b; k <= t - 1; ++k) {
            ufl(k, j) = uf[k] + dz_face(k, j) * 0.5 / dzhalf_face(k, j) * (uf[k + 1] - uf[k]);
            vfl(k, j) = vf[k] + dz_face(k, j) * 0.5 / dzhalf_face(k, j) * (vf[k + 1] - vf[k]);
        }
    }
    OMP_FOR
    for (int i = 1; i <= c->NN; ++i) {
        for (int k = 0; k <= L; ++k) {
            u_node(k, i) = 0.0;
            v_node(k, i) = 0.0;
            double weight = 0.0;
            int icount = 0;
            for (int j = 1; j <= c->adj_cells_at_node(i); ++j) {
                int isn = c->adj_cellnum_at_node(j, i);
                int nc = c->node_count_each_element(j, i);
                int tq = c->tri_or_quad(isn);
                for (int l = tq - 2; l <= tq - 1; ++l) {
                    int ifn = c->facenum_at_cell(start_end_node(tq, nc, l), isn);
                    double fw = (c->adj_cellnum_at_face(2, ifn) == 0) ? 2.0 : 1.0;
                    if (top_f(ifn) != 0 && k >= c->bottom_layer_at_face(ifn) - 1) {
                        int kvt = std::min(k, (int)top_f(ifn));
                        u_node(k, i) = u_node(k, i) + ufl(kvt, ifn) / c->face_length(ifn) * fw;
                        v_node(k, i) = v_node(k, i) + vfl(kvt, ifn) / c->face_length(ifn) * fw;
                        icount = icount + 1;
                    }
                    weight = weight + fw / c->face_length(ifn);
                }
            }
            if (icount != 0) {
                u_node(k, i) = u_node(k, i) / weight;
                v_node(k, i) = v_node(k, i) / weight;
            }
        }
    }
    OMP_FOR
    for (int i = 1; i <= c->NN; ++i) {
        for (int k = 0; k <= L; ++k) {
            w_node(k, i) = 0.0;
            double tw = 0.0;
            for (int j = 1; j <= c->adj_cells_at_node(i); ++j) {
                int ite = c->adj_cellnum_at_node(j, i);
                if (top_el(ite) != 0 && k >= c->bottom_layer_at_element(ite) - 1) {
                    int kvt = std::min(k, (int)top_el(ite));
                    tw = tw + c->area(ite);
                    w_node(k, i) = w_node(k, i) + wn_cell(kvt, ite) * c->area(ite);
                }
            }
            if (tw != 0.0) w_node(k, i) = w_node(k, i) / tw;
        }
    }
    return GOM_OK;
}

// solve_transport_equation_v19.f90:7-1482 (transport_solver = 1, tracers S and T)
// solve_transport_equation_ELM_v8.f90:7-346 (transport_solver = 2): temperature and salinity
// backtracked from every wet cell-layer centre (ELM_backtrace_v1 in transport mode), explicit
// horizontal diffusion, implicit vertical diffusion, node and face averages.  Reproduced as the
// reference has them: the horizontal sums use the face's second cell as the neighbour and the
// salinity sums go to temperature and the temperature sums to salinity (:137-151); the top row's
// upper coefficient is -dt + Kv/dzhalf (:188); no clamp; dry cells and dry nodes keep their
// previous values; face values are the mean of the two node values in every layer.  The heat
// source of :120 adds dt phi_sz / (rho_o cp dz) to every wet cell-layer (phi_sz from the host).
static int transport_elm(gom_ctx *c) {
    const gom_params &p = c->p;
    const int L = c->L, NC = c->NC, NF = c->NF, NN = c->NN;
    const double dt = p.dt;
    A2<double> salt_cell = FD(c, GOM_F_SALT_CELL), temp_cell = FD(c, GOM_F_TEMP_CELL), dz_cell = FD(c, GOM_F_DZ_CELL),
               dzh_c = FD(c, GOM_F_DZHALF_CELL), dz_face = FD(c, GOM_F_DZ_FACE), dz_cn = FD(c, GOM_F_DZ_CELL_NEW),
               wn_cell = FD(c, GOM_F_WN_CELL), u_node = FD(c, GOM_F_U_NODE), v_node = FD(c, GOM_F_V_NODE),
               Kh = FD(c, GOM_F_KH), Kv = FD(c, GOM_F_KV);
    A2<double> salt_new = FD(c, GOM_F_SALT_CELL_NEW), temp_new = FD(c, GOM_F_TEMP_CELL_NEW),
               salt_node = FD(c, GOM_F_SALT_NODE), temp_node = FD(c, GOM_F_TEMP_NODE),
               salt_face = FD(c, GOM_F_SALT_FACE), temp_face = FD(c, GOM_F_TEMP_FACE);
    A2<int32_t> nsub = FI(c, GOM_F_NUM_SUB_ELM);
    A1<double> eta_cell = FD1(c, GOM_F_ETA_CELL);
    A1<int32_t> top = FI1(c, GOM_F_TOP_LAYER_CELL), top_n = FI1(c, GOM_F_TOP_LAYER_NODE);
    std::vector<double> tc_bt((size_t)L * NC, 0.0), sc_bt((size_t)L * NC, 0.0), trhs((size_t)L * NC, 0.0),
        srhs((size_t)L * NC, 0.0);
    auto AT = [&](std::vector<double> &v, int k, int i) -> double & { return v[(size_t)(i - 1) * L + k - 1]; };
    // :59-125 backtracking
    std::atomic<int> rc{GOM_OK};
    OMP_FOR
    for (int i = 1; i <= NC; ++i) {
        if (rc.load(std::memory_order_relaxed) != GOM_OK) continue;
        if (top(i) == 0) continue;   // tc_bt = sc_bt = 0
        for (int k = c->bottom_layer_at_element(i); k <= top(i); ++k) {
            int nnel = i, jlev = k;
            double x0 = c->x_cell(i), y0 = c->y_cell(i), z0;
            if (k == top(nnel)) z0 = p.msl + eta_cell(nnel) - dz_cell(k, nnel) * 0.5;
            else z0 = c->zl(k) - dz_cell(k, nnel) * 0.5;
            double u_temp = 0.0, v_temp = 0.0;
            int bt_step = 0;
            const int tq = c->tri_or_quad(i);
            for (int l = 1; l <= tq; ++l) {
                int nd = c->nodenum_at_cell(l, i);
                u_temp = u_temp + (u_node(k, nd) + u_node(k - 1, nd)) * 0.5;
                v_temp = v_temp + (v_node(k, nd) + v_node(k - 1, nd)) * 0.5;
                bt_step = bt_step + nsub(k, nd);
            }
            u_temp = u_temp / tq;
            v_temp = v_temp / tq;
            bt_step = bt_step / tq;
            double uuint = u_temp, vvint = v_temp, wwint = (wn_cell(k, i) + wn_cell(k - 1, i)) * 0.5;
            double vmag = std::sqrt(uuint * uuint + vvint * vvint + wwint * wwint);
            if (vmag <= F(1.e-4f)) {
                AT(tc_bt, k, i) = temp_cell(k, i);
                AT(sc_bt, k, i) = salt_cell(k, i);
            } else {
                double bt_dt = dt / bt_step;
                int near = 0;
                ElmFinal fin;
                int e = elm_backtrace(c, bt_step, bt_dt, uuint, vvint, wwint, x0, y0, z0, nnel, jlev, near, &fin);
                double ttint = 0.0, ssint = 0.0;
                if (!e) e = elm_tracer_at_foot(c, fin, nnel, jlev, ttint, ssint);
                if (e) {
                    set_err(c, GOM_E_ELM, e, i, k, 0.0, GOM_ENTITY_CELL);
                    rc = GOM_E_ELM;
                    break;
                }
                AT(tc_bt, k, i) = ttint;
                AT(sc_bt, k, i) = ssint;
            }
            // :120 the per-layer heat source
            AT(tc_bt, k, i) = AT(tc_bt, k, i) + dt * c->phi_sz[(size_t)(i - 1) * L + k - 1] / (p.rho_o * 4186.0 * dz_cell(k, i));
        }
    }
    if (rc.load() != GOM_OK) return rc.load();
    // :133-154 explicit horizontal diffusion
    OMP_FOR
    for (int i = 1; i <= NC; ++i) {
        for (int k = c->bottom_layer_at_element(i); k <= top(i); ++k) {
            double sum1 = 0.0, sum2 = 0.0;
            for (int l = 1; l <= c->tri_or_quad(i); ++l) {
                int j = c->facenum_at_cell(l, i);
                int ie = c->adj_cellnum_at_face(2, j);
                if (ie != 0) {
                    double rtemp1 = c->face_length(j) * dz_face(k, j) * Kh(k, j) / c->delta_j(j);
                    sum1 = sum1 + rtemp1 * (salt_cell(k, ie) - salt_cell(k, i));
                    sum2 = sum2 + rtemp1 * (temp_cell(k, ie) - temp_cell(k, i));
                }
            }
            sum1 = sum1 * dt / (c->area(i) * dz_cell(k, i));
            sum2 = sum2 * dt / (c->area(i) * dz_cell(k, i));
            AT(trhs, k, i) = AT(tc_bt, k, i) + sum1;
            AT(srhs, k, i) = AT(sc_bt, k, i) + sum2;
        }
    }
    // :163-236 implicit vertical diffusion, extension below the bottom and above the top
    OMP_FOR
    for (int i = 1; i <= NC; ++i) {
        if (rc.load(std::memory_order_relaxed) != GOM_OK) continue;
        const int t = top(i), b = c->bottom_layer_at_element(i);
        if (t == 0) continue;
        const int nvl = t - b + 1;
        double am[GOM_ORACLE_MAXL + 1] = {0}, bm[GOM_ORACLE_MAXL + 1] = {0}, cm[GOM_ORACLE_MAXL + 1] = {0},
               gm[GOM_ORACLE_MAXL + 1] = {0}, rr[(GOM_ORACLE_MAXL + 1) * 2] = {0}, sol[(GOM_ORACLE_MAXL + 1) * 2] = {0};
        const int nmax = L + 1;
        for (int k = b + 1; k <= t - 1; ++k) {
            int kk = t - k + 1;
            am[kk - 1] = -dt * Kv(k, i) / dzh_c(k, i);
            cm[kk - 1] = -dt * Kv(k - 1, i) / dzh_c(k - 1, i);
            bm[kk - 1] = -am[kk - 1] + dz_cell(k, i) - cm[kk - 1];
        }
        if (t == b) {
            bm[0] = dz_cell(t, i);
        } else {
            cm[0] = -dt + Kv(t - 1, i) / dzh_c(t - 1, i);
            bm[0] = dz_cell(t, i) - cm[0];
            am[nvl - 1] = -dt * Kv(b, i) / dzh_c(b, i);
            bm[nvl - 1] = -am[nvl - 1] + dz_cell(b, i);
        }
        for (int k = 1; k <= nvl; ++k) {
            int kk = t - k + 1;
            rr[0 * nmax + k - 1] = dz_cell(kk, i) * AT(trhs, kk, i);
            rr[1 * nmax + k - 1] = dz_cell(kk, i) * AT(srhs, kk, i);
        }
        if (!tridiagonal_solver(nmax, nvl, 2, am, bm, cm, rr, sol, gm)) {
            set_err(c, GOM_E_ZERO_PIVOT, 210, i, 0, 0.0, GOM_ENTITY_CELL);
            rc = GOM_E_ZERO_PIVOT;
            continue;
        }
        for (int k = 1; k <= nvl; ++k) {
            int klev = t + 1 - k;
            temp_new(klev, i) = sol[0 * nmax + k - 1];
            salt_new(klev, i) = sol[1 * nmax + k - 1];
        }
        for (int k = 1; k <= b - 1; ++k) {
            temp_new(k, i) = temp_new(b, i);
            salt_new(k, i) = salt_new(b, i);
        }
        for (int k = t + 1; k <= L; ++k) {
            temp_new(k, i) = temp_new(t, i);
            salt_new(k, i) = salt_new(t, i);
        }
    }
    if (rc.load() != GOM_OK) return rc.load();
    // :262-330 node averages with the fill from above, then the extension of wet nodes
    OMP_FOR
    for (int i = 1; i <= NN; ++i) {
        for (int k = top_n(i); k >= c->bottom_layer_at_node(i); --k) {
            double sum0 = 0.0, sum1 = 0.0, sum2 = 0.0;
            int icount = 0;
            for (int l = 1; l <= c->adj_cells_at_node(i); ++l) {
                int ie = c->adj_cellnum_at_node(l, i);
                if (k >= c->bottom_layer_at_element(ie) && k <= top(ie)) {
                    sum0 = sum0 + c->area(ie) * dz_cn(k, ie);
                    sum1 = sum1 + c->area(ie) * dz_cn(k, ie) * temp_new(k, ie);
                    sum2 = sum2 + c->area(ie) * dz_cn(k, ie) * salt_new(k, ie);
                } else {
                    icount = icount + 1;
                }
            }
            if (sum0 == 0.0) {
                temp_node(k, i) = 0.0;
                salt_node(k, i) = 0.0;
            } else {
                temp_node(k, i) = sum1 / sum0;
                salt_node(k, i) = sum2 / sum0;
            }
            if (icount == c->adj_cells_at_node(i) && k != top_n(i)) {
                temp_node(k, i) = temp_node(k + 1, i);
                salt_node(k, i) = salt_node(k + 1, i);
            }
        }
        if (top_n(i) == 0) continue;
        const int kb = c->bottom_layer_at_node(i), kt = top_n(i);
        for (int k = 1; k <= kb - 1; ++k) {
            temp_node(k, i) = temp_node(kb, i);
            salt_node(k, i) = salt_node(kb, i);
        }
        for (int k = kt + 1; k <= L; ++k) {
            temp_node(k, i) = temp_node(kt, i);
            salt_node(k, i) = salt_node(kt, i);
        }
    }
    // :332-339 face values
    OMP_FOR
    for (int j = 1; j <= NF; ++j) {
        int n1 = c->nodenum_at_face(1, j), n2 = c->nodenum_at_face(2, j);
        for (int k = 1; k <= L; ++k) {
            salt_face(k, j) = (salt_node(k, n1) + salt_node(k, n2)) * F(0.5f);
            temp_face(k, j) = (temp_node(k, n1) + temp_node(k, n2)) * F(0.5f);
        }
    }
    return GOM_OK;
}

int gom_step_transport(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    const gom_params &p = c->p;
    if (!p.transport_flag) return GOM_OK;
    if (p.transport_solver == 2) return transport_elm(c);
    const int L = c->L, NC = c->NC, NF = c->NF, NN = c->NN;
    const double dt = p.dt, theta = p.theta, rho_o = p.rho_o;
    const int ntr = (p.is_salt ? 1 : 0) + (p.is_temp ? 1 : 0);
    if (ntr == 0) return GOM_OK;
    int tran_id[2];
    {
        int ii = 0;
        if (p.is_salt) tran_id[ii++] = 1;
        if (p.is_temp) tran_id[ii++] = 2;
    }
    A2<double> salt_cell = FD(c, GOM_F_SALT_CELL), temp_cell = FD(c, GOM_F_TEMP_CELL), dz_cell = FD(c, GOM_F_DZ_CELL),
               dz_cn = FD(c, GOM_F_DZ_CELL_NEW), dzh_c = FD(c, GOM_F_DZHALF_CELL), dzh_cn = FD(c, GOM_F_DZHALF_CELL_NEW),
               dz_face = FD(c, GOM_F_DZ_FACE), dz_fn = FD(c, GOM_F_DZ_FACE_NEW), un_face = FD(c, GOM_F_UN_FACE),
               un_new = FD(c, GOM_F_UN_FACE_NEW), wn_cell = FD(c, GOM_F_WN_CELL), wn_new = FD(c, GOM_F_WN_CELL_NEW),
               Kh = FD(c, GOM_F_KH), Kv = FD(c, GOM_F_KV);
    A1<int32_t> top_el = FI1(c, GOM_F_TOP_LAYER_CELL), top_f = FI1(c, GOM_F_TOP_LAYER_FACE),
                top_n = FI1(c, GOM_F_TOP_LAYER_NODE);
    const int LC = L + 2;  // con_cell (0:L+1)
    std::vector<double> con_cell((size_t)LC * NC * ntr, 0.0), con_cell_new((size_t)L * NC * ntr, 0.0),
        con_node_new((size_t)L * NN * ntr, 0.0), con_face_new((size_t)L * NF * ntr, 0.0);
    auto CC = [&](int k, int i, int t) -> double & { return con_cell[((size_t)(t - 1) * NC + (i - 1)) * LC + k]; };
    auto CN = [&](int k, int i, int t) -> double & { return con_cell_new[((size_t)(t - 1) * NC + (i - 1)) * L + k - 1]; };
    auto NDN = [&](int k, int i, int t) -> double & { return con_node_new[((size_t)(t - 1) * NN + (i - 1)) * L + k - 1]; };
    auto FCN = [&](int k, int j, int t) -> double & { return con_face_new[((size_t)(t - 1) * NF + (j - 1)) * L + k - 1]; };
    const double cp = 4186.0;
    // :88-173 load tracers
    for (int i3 = 1; i3 <= ntr; ++i3) {
        OMP_FOR
        for (int i = 1; i <= NC; ++i) {
            for (int k = 1; k <= L; ++k) CC(k, i, i3) = tran_id[i3 - 1] == 1 ? salt_cell(k, i) : temp_cell(k, i);
            CC(0, i, i3) = 0.0;
            CC(L + 1, i, i3) = 0.0;
            if (tran_id[i3 - 1] == 2 && p.heat_option == 2) {
                // :150-159 adds dt*phi_sw/(rho_o*cp*dz_top) to all layers; dry cells are skipped
                // (the reference would index dz_cell(0,i) there)
                int t = top_el(i);
                if (t > 0)
                    for (int k = 1; k <= L; ++k)
                        CC(k, i, i3) = CC(k, i, i3) + dt * c->phi_sw[i - 1] / (rho_o * cp * dz_cell(t, i));
            } else if (tran_id[i3 - 1] == 2 && p.heat_option == 1) {
                // :100-131 the per-layer source phi_sz over the wet layers
                for (int k = c->bottom_layer_at_element(i); k <= top_el(i); ++k)
                    CC(k, i, i3) = CC(k, i, i3) + dt * c->phi_sz[(size_t)(i - 1) * L + k - 1] / (rho_o * cp * dz_cell(k, i));
            }
        }
    }
    int Nt = p.trans_sub_iter;
    if (Nt == 0) Nt = 1;
    const double dt2 = dt / Nt;
    // work arrays: unassigned entries read as 0
    std::vector<double> Q_jk((size_t)L * NF), D_jk((size_t)L * NF), d_jk((size_t)L * NF), phi_jk((size_t)L * NF);
    std::vector<double> Q_ik((size_t)(L + 1) * NC), D_ik((size_t)(L + 1) * NC), d_ik((size_t)(L + 1) * NC),
        phi_ik((size_t)(L + 1) * NC);
    std::vector<double> r_jk((size_t)L * NF * ntr), r_ik((size_t)(L + 1) * NC * ntr), PSI_jk((size_t)L * NF * ntr),
        PSI_ik((size_t)(L + 1) * NC * ntr);
    auto QJ = [&](int k, int j) -> double & { return Q_jk[(size_t)(j - 1) * L + k - 1]; };
    auto DJ = [&](int k, int j) -> double & { return D_jk[(size_t)(j - 1) * L + k - 1]; };
    auto dJ = [&](int k, int j) -> double & { return d_jk[(size_t)(j - 1) * L + k - 1]; };
    auto pJ = [&](int k, int j) -> double & { return phi_jk[(size_t)(j - 1) * L + k - 1]; };
    auto QI = [&](int k, int i) -> double & { return Q_ik[(size_t)(i - 1) * (L + 1) + k]; };
    auto DI = [&](int k, int i) -> double & { return D_ik[(size_t)(i - 1) * (L + 1) + k]; };
    auto dI = [&](int k, int i) -> double & { return d_ik[(size_t)(i - 1) * (L + 1) + k]; };
    auto pI = [&](int k, int i) -> double & { return phi_ik[(size_t)(i - 1) * (L + 1) + k]; };
    auto RJ = [&](int k, int j, int t) -> double & { return r_jk[((size_t)(t - 1) * NF + j - 1) * L + k - 1]; };
    auto RI = [&](int k, int i, int t) -> double & { return r_ik[((size_t)(t - 1) * NC + i - 1) * (L + 1) + k]; };
    auto PJ = [&](int k, int j, int t) -> double & { return PSI_jk[((size_t)(t - 1) * NF + j - 1) * L + k - 1]; };
    auto PI_ = [&](int k, int i, int t) -> double & { return PSI_ik[((size_t)(t - 1) * NC + i - 1) * (L + 1) + k]; };
    std::vector<double> con_at_obk((size_t)L * c->NOB * ntr), con_at_qbk((size_t)L * c->NQB * ntr);
    auto OBK = [&](int k, int i, int t) -> double & { return con_at_obk[((size_t)(t - 1) * c->NOB + i - 1) * L + k - 1]; };
    auto QBK = [&](int k, int i, int t) -> double & { return con_at_qbk[((size_t)(t - 1) * c->NQB + i - 1) * L + k - 1]; };
    // con_at_ob(i, i3) for subcycle s: host array (n_ob, 2, Nt), slot 1 = salt, 2 = temperature
    auto con_ob = [&](int i, int i3, int s) {
        return c->con_at_ob[((size_t)s * 2 + (tran_id[i3 - 1] - 1)) * c->NOB + (i - 1)];
    };
    auto con_qb = [&](int i, int i3, int s) {
        return c->con_at_qb[((size_t)s * 2 + (tran_id[i3 - 1] - 1)) * c->NQB + (i - 1)];
    };
    for (int subcycle = 0; subcycle <= Nt - 1; ++subcycle) {
        std::fill(con_at_obk.begin(), con_at_obk.end(), 0.0);
        std::fill(con_at_qbk.begin(), con_at_qbk.end(), 0.0);
        std::fill(r_ik.begin(), r_ik.end(), 1.0);
        std::fill(r_jk.begin(), r_jk.end(), 1.0);
        // :232-321 open-boundary concentrations by upwind direction
        for (int i = 1; i <= c->NOB; ++i) {
            int i2 = c->ob_cell_id(i);
            int t = top_el(i2), b = c->bottom_layer_at_element(i2);
            for (int l = 1; l <= c->tri_or_quad(i2); ++l) {
                int j2 = c->facenum_at_cell(l, i2);
                if (c->boundary_type_of_face(j2) > 0) {
                    for (int k = b; k <= t; ++k) {
                        double dz_old = (dz_face(k, j2) + (dz_fn(k, j2) - dz_face(k, j2)) * subcycle / Nt);
                        double sg = (double)c->sign_in_outflow(l, i2);
                        double q2 = c->face_length(j2) * dz_old *
                                    ((1.0 - theta) * un_face(k, j2) * sg + theta * un_new(k, j2) * sg);
                        for (int i3 = 1; i3 <= ntr; ++i3)
                            OBK(k, i, i3) = (q2 <= 0.0) ? con_ob(i, i3, subcycle) : CC(k, i2, i3);
                    }
                }
            }
        }
        // :327-397 river concentrations
        for (int i = 1; i <= c->NQB; ++i) {
            int i2 = c->qb_cell(i);
            int t = top_el(i2), b = c->bottom_layer_at_element(i2);
            for (int k = b; k <= t; ++k)
                for (int i3 = 1; i3 <= ntr; ++i3) QBK(k, i, i3) = con_qb(i, i3, subcycle);
        }
        // :551-581 face coefficients
        OMP_FOR
        for (int j = 1; j <= NF; ++j) {
            int b = c->bottom_layer_at_face(j), t = top_f(j);
            for (int k = b; k <= t; ++k) {
                double dz_old = dz_face(k, j) + (dz_fn(k, j) - dz_face(k, j)) * subcycle / Nt;
                QJ(k, j) = c->face_length(j) * dz_old * ((1.0 - theta) * un_face(k, j) + theta * un_new(k, j));
                DJ(k, j) = c->face_length(j) * dz_old * Kh(k, j) / c->delta_j(j);
                dJ(k, j) = std::max(0.0, DJ(k, j) - 0.5 * std::fabs(QJ(k, j)));
                if (QJ(k, j) == 0.0) pJ(k, j) = 1.0;
                else pJ(k, j) = std::min(1.0, 2.0 * DJ(k, j) / std::fabs(QJ(k, j)));
            }
        }
        // :585-610 vertical coefficients
        OMP_FOR
        for (int i = 1; i <= NC; ++i) {
            int b = c->bottom_layer_at_element(i), t = top_el(i);
            for (int k = b; k <= t - 1; ++k) {
                QI(k, i) = c->area(i) * ((1.0 - theta) * wn_cell(k, i) + theta * wn_new(k, i));
                double dz_old = dzh_c(k, i) + (dzh_cn(k, i) - dzh_c(k, i)) * subcycle / Nt;
                DI(k, i) = c->area(i) * Kv(k, i) / dz_old;
                dI(k, i) = std::max(0.0, DI(k, i) - 0.5 * std::fabs(QI(k, i)));
                if (QI(k, i) == 0.0) pI(k, i) = 1.0;
                else pI(k, i) = std::min(1.0, 2.0 * DI(k, i) / std::fabs(QI(k, i)));
            }
        }
        // boundary concentrations of an open-boundary or river cell's layers, into a per-cell
        // buffer oqb (L, 2); only faces without a neighbour cell read it
        auto load_oqb = [&](double *oqb, int i, int b, int t) {
            int ith_ob = c->ob_element_flag(i), ith_Qb = c->Qb_element_flag(i);
            if (ith_ob > 0)
                for (int k = b; k <= t; ++k)
                    for (int i3 = 1; i3 <= ntr; ++i3) oqb[(size_t)(i3 - 1) * L + k - 1] = OBK(k, ith_ob, i3);
            if (ith_Qb > 0)
                for (int k = b; k <= t; ++k)
                    for (int i3 = 1; i3 <= ntr; ++i3) oqb[(size_t)(i3 - 1) * L + k - 1] = QBK(k, ith_Qb, i3);
        };
        auto face_open = [&](int j) {
            return c->boundary_type_of_face(j) != -1 || c->isflowside3(j) > 0;
        };
        // :615-904 limiter
        if (p.h_flux_limiter > 0 || p.v_flux_limiter > 0) {
            OMP_FOR
            for (int i = 1; i <= NC; ++i) {
                int t = top_el(i), b = c->bottom_layer_at_element(i);
                if (t == 0) continue;
                int nvl = t - b + 1;
                double sum1[2], sum2[2], s1a[2], s2a[2], cik[2], Q2[4];
                double oqb[2 * GOM_ORACLE_MAXL] = {0};
                auto OQB = [&](int k, int t3) { return oqb[(size_t)(t3 - 1) * L + k - 1]; };
                load_oqb(oqb, i, b, t);
                int tq = c->tri_or_quad(i);
                for (int k = b; k <= t; ++k) {
                    for (int i3 = 0; i3 < 2; ++i3) sum1[i3] = sum2[i3] = s1a[i3] = s2a[i3] = 0.0;
                    if (nvl != 1) {
                        if (k == b) {
                            for (int i3 = 1; i3 <= ntr; ++i3) {
                                double rt2 = std::fabs(0.5 * (QI(k, i) + std::fabs(QI(k, i))));
                                s1a[i3 - 1] = rt2 * (CC(k, i, i3) - CC(k + 1, i, i3));
                                s2a[i3 - 1] = rt2;
                            }
                        } else if (k == t) {
                            for (int i3 = 1; i3 <= ntr; ++i3) {
                                double rt1 = std::fabs(0.5 * (QI(k - 1, i) + std::fabs(QI(k - 1, i))));
                                s1a[i3 - 1] = rt1 * (CC(k, i, i3) - CC(k - 1, i, i3));
                                s2a[i3 - 1] = rt1;
                            }
                        } else {
                            for (int i3 = 1; i3 <= ntr; ++i3) {
                                double rt1 = std::fabs(0.5 * (QI(k - 1, i) + std::fabs(QI(k - 1, i))));
                                double rt2 = std::fabs(0.5 * (QI(k, i) + std::fabs(QI(k, i))));
                                s1a[i3 - 1] = rt1 * (CC(k, i, i3) - CC(k - 1, i, i3)) + rt2 * (CC(k, i, i3) - CC(k + 1, i, i3));
                                s2a[i3 - 1] = rt1 + rt2;
                            }
                        }
                    }
                    for (int l = 1; l <= tq; ++l) {
                        int j = c->facenum_at_cell(l, i);
                        int ii = c->adj_cellnum_at_cell(l, i);
                        if (face_open(j)) {
                            Q2[l - 1] = QJ(k, j) * (double)c->sign_in_outflow(l, i);
                            if (Q2[l - 1] < 0.0) {
                                for (int i3 = 1; i3 <= ntr; ++i3) cik[i3 - 1] = ii > 0 ? CC(k, ii, i3) : OQB(k, i3);
                                for (int i3 = 1; i3 <= ntr; ++i3) {
                                    sum1[i3 - 1] = sum1[i3 - 1] + std::fabs(Q2[l - 1]) * (CC(k, i, i3) - cik[i3 - 1]);
                                    sum2[i3 - 1] = sum2[i3 - 1] + std::fabs(Q2[l - 1]);
                                }
                            }
                        }
                    }
                    for (int i3 = 1; i3 <= ntr; ++i3) {
                        s1a[i3 - 1] = s1a[i3 - 1] + sum1[i3 - 1];
                        s2a[i3 - 1] = s2a[i3 - 1] + sum2[i3 - 1];
                    }
                    for (int l = 1; l <= tq; ++l) {
                        int j = c->facenum_at_cell(l, i);
                        int ii = c->adj_cellnum_at_cell(l, i);
                        if (face_open(j)) {
                            if (Q2[l - 1] >= 0.0) {
                                for (int i3 = 1; i3 <= ntr; ++i3) cik[i3 - 1] = ii > 0 ? CC(k, ii, i3) : OQB(k, i3);
                                for (int i3 = 1; i3 <= ntr; ++i3) {
                                    double rtemp = s2a[i3 - 1] * (cik[i3 - 1] - CC(k, i, i3));
                                    if (rtemp == 0.0) RJ(k, j, i3) = F(1.0f);
                                    else RJ(k, j, i3) = s1a[i3 - 1] / rtemp;
                                }
                            }
                        }
                    }
                }
                // :806-840 vertical ratios from the last layer's horizontal sums
                if (QI(t, i) >= 0.0) {
                    for (int k = b; k <= t - 1; ++k)
                        for (int i3 = 1; i3 <= ntr; ++i3) {
                            double rt1 = sum1[i3 - 1] + std::fabs(QI(k - 1, i)) * (CC(k, i, i3) - CC(k - 1, i, i3));
                            double rt2 = sum2[i3 - 1] + std::fabs(QI(k - 1, i));
                            double rtemp = (CC(k + 1, i, i3) - CC(k, i, i3)) * rt2;
                            if (rtemp == 0.0) RI(k, i, i3) = 1.0;
                            else RI(k, i, i3) = rt1 / rtemp;
                        }
                } else {
                    for (int k = b + 1; k <= t; ++k)
                        for (int i3 = 1; i3 <= ntr; ++i3) {
                            double rt1 = sum1[i3 - 1] + std::fabs(QI(k, i)) * (CC(k, i, i3) - CC(k + 1, i, i3));
                            double rt2 = sum2[i3 - 1] + std::fabs(QI(k, i));
                            double rtemp = (CC(k - 1, i, i3) - CC(k, i, i3)) * rt2;
                            if (rtemp == 0.0) RI(k - 1, i, i3) = 1.0;
                            else RI(k - 1, i, i3) = rt1 / rtemp;
                        }
                }
                for (int i3 = 1; i3 <= ntr; ++i3) {
                    RI(t, i, i3) = 1.0;
                    RI(b - 1, i, i3) = 1.0;
                }
            }
            auto limiter = [&](double small_phi, double r) {
                switch (p.h_flux_limiter) {
                case 1: return std::max(small_phi, std::min(F(1.0f), r)) - small_phi;
                case 2: return std::max(small_phi, (r + std::fabs(r)) / (F(1.0f) + std::fabs(r))) - small_phi;
                case 3: return std::max(std::max(small_phi, std::min(F(1.0f), 2.0 * r)), std::min(2.0, r)) - small_phi;
                default: return 0.0;
                }
            };
            OMP_FOR
            for (int i = 1; i <= NC; ++i) {
                int b = c->bottom_layer_at_element(i), t = top_el(i);
                for (int k = b; k <= t - 1; ++k)
                    for (int i3 = 1; i3 <= ntr; ++i3) PI_(k, i, i3) = limiter(pI(k, i), RI(k, i, i3));
            }
            OMP_FOR
            for (int j = 1; j <= NF; ++j) {
                int b = c->bottom_layer_at_face(j), t = top_f(j);
                for (int k = b; k <= t; ++k)
                    for (int i3 = 1; i3 <= ntr; ++i3) PJ(k, j, i3) = limiter(pJ(k, j), RJ(k, j, i3));
            }
        }
        // :921-1346 implicit vertical solve per cell
        std::atomic<int> rc{GOM_OK};
        OMP_FOR
        for (int i = 1; i <= NC; ++i) {
            if (rc.load(std::memory_order_relaxed) != GOM_OK) continue;
            int b = c->bottom_layer_at_element(i), t = top_el(i);
            if (t == 0) continue;
            int nvl = t - b + 1;
            double am[GOM_ORACLE_MAXL + 1] = {0}, bm[GOM_ORACLE_MAXL + 1] = {0}, cm[GOM_ORACLE_MAXL + 1] = {0},
                   gm[GOM_ORACLE_MAXL + 1] = {0}, rhs[2 * GOM_ORACLE_MAXL] = {0}, sol[2 * GOM_ORACLE_MAXL] = {0};
            double oqb[2 * GOM_ORACLE_MAXL] = {0};
            auto OQB = [&](int k, int t3) { return oqb[(size_t)(t3 - 1) * L + k - 1]; };
            double ar = c->area(i);
            for (int k = b + 1; k <= t - 1; ++k) {
                int kk = t + 1 - k;
                am[kk - 1] = -dt2 * dI(k, i);
                cm[kk - 1] = -dt2 * dI(k - 1, i);
                double dz_new = dz_cell(k, i) + (dz_cn(k, i) - dz_cell(k, i)) * (subcycle + 1) / Nt;
                bm[kk - 1] = -am[kk - 1] + ar * dz_new - cm[kk - 1];
            }
            if (t == b) {
                double dz_new = dz_cell(t, i) + (dz_cn(t, i) - dz_cell(t, i)) * (subcycle + 1) / Nt;
                bm[0] = ar * dz_new;
            } else {
                cm[0] = -dt2 * dI(t - 1, i);
                double dz_new = dz_cell(t, i) + (dz_cn(t, i) - dz_cell(t, i)) * (subcycle + 1) / Nt;
                bm[0] = ar * dz_new - cm[0];
                am[nvl - 1] = -dt2 * dI(b, i);
                dz_new = dz_cell(b, i) + (dz_cn(b, i) - dz_cell(b, i)) * (subcycle + 1) / Nt;
                bm[nvl - 1] = -am[nvl - 1] + ar * dz_new;
            }
            load_oqb(oqb, i, b, t);
            int tq = c->tri_or_quad(i);
            for (int k = b; k <= t; ++k) {
                int kk = t + 1 - k;
                double sQi[2] = {0, 0}, sQii[2] = {0, 0}, shd[2] = {0, 0}, shl[2] = {0, 0}, cik[2];
                for (int l = 1; l <= tq; ++l) {
                    int j = c->facenum_at_cell(l, i);
                    int ii = c->adj_cellnum_at_cell(l, i);
                    for (int i3 = 1; i3 <= ntr; ++i3) cik[i3 - 1] = ii > 0 ? CC(k, ii, i3) : OQB(k, i3);
                    if (face_open(j)) {
                        double q2 = QJ(k, j) * (double)c->sign_in_outflow(l, i);
                        if (q2 > 0.0) {
                            for (int i3 = 1; i3 <= ntr; ++i3) sQi[i3 - 1] = sQi[i3 - 1] + std::fabs(q2) * CC(k, i, i3);
                        } else if (q2 < 0.0) {
                            for (int i3 = 1; i3 <= ntr; ++i3) sQii[i3 - 1] = sQii[i3 - 1] + std::fabs(q2) * cik[i3 - 1];
                        }
                        for (int i3 = 1; i3 <= ntr; ++i3) shd[i3 - 1] = shd[i3 - 1] + dJ(k, j) * (cik[i3 - 1] - CC(k, i, i3));
                        for (int i3 = 1; i3 <= ntr; ++i3)
                            shl[i3 - 1] = shl[i3 - 1] + PJ(k, j, i3) * std::fabs(q2) * (CC(k, i, i3) - cik[i3 - 1]);
                    }
                }
                for (int i3 = 1; i3 <= ntr; ++i3) {
                    double h_adv = dt2 * (sQii[i3 - 1] - sQi[i3 - 1]);
                    double h_diff = dt2 * shd[i3 - 1];
                    double h_flux = 0.5 * dt2 * shl[i3 - 1];
                    double dz_old = dz_cell(k, i) + (dz_cn(k, i) - dz_cell(k, i)) * subcycle / Nt;
                    double v = ar * dz_old * CC(k, i, i3) + h_adv + h_diff;
                    if (p.h_flux_limiter > 0) v = v + h_flux;
                    rhs[(size_t)(i3 - 1) * L + kk - 1] = v;
                }
            }
            if (nvl != 1) {
                for (int k = b; k <= t; ++k) {
                    int kk = t + 1 - k;
                    for (int i3 = 1; i3 <= ntr; ++i3) {
                        double &R = rhs[(size_t)(i3 - 1) * L + kk - 1];
                        double v_adv, v_flux = 0.0;
                        if (k == b) {
                            double qp = std::fabs(0.5 * (QI(k, i) + std::fabs(QI(k, i))));
                            double qm = std::fabs(0.5 * (QI(k, i) - std::fabs(QI(k, i))));
                            v_adv = dt2 * (-qp * CC(k, i, i3) + qm * CC(k + 1, i, i3));
                            R = R + v_adv;
                            if (p.v_flux_limiter > 0) {
                                v_flux = 0.5 * dt2 * (-PI_(k, i, i3) * qp * (CC(k + 1, i, i3) - CC(k, i, i3)) +
                                                      PI_(k, i, i3) * qm * (CC(k, i, i3) - CC(k + 1, i, i3)));
                                R = R + v_flux;
                            }
                        } else if (k == t) {
                            double qp = std::fabs(0.5 * (QI(k - 1, i) + std::fabs(QI(k - 1, i))));
                            double qm = std::fabs(0.5 * (QI(k - 1, i) - std::fabs(QI(k - 1, i))));
                            v_adv = dt2 * (qp * CC(k - 1, i, i3) - qm * CC(k, i, i3));
                            R = R + v_adv;
                            if (p.v_flux_limiter > 0) {
                                v_flux = 0.5 * dt2 * (PI_(k - 1, i, i3) * qp * (CC(k, i, i3) - CC(k - 1, i, i3)) -
                                                      PI_(k - 1, i, i3) * qm * (CC(k - 1, i, i3) - CC(k, i, i3)));
                                R = R + v_flux;
                            }
                        } else {
                            double qp1 = std::fabs(0.5 * (QI(k - 1, i) + std::fabs(QI(k - 1, i))));
                            double qp = std::fabs(0.5 * (QI(k, i) + std::fabs(QI(k, i))));
                            double qm = std::fabs(0.5 * (QI(k, i) - std::fabs(QI(k, i))));
                            double qm1 = std::fabs(0.5 * (QI(k - 1, i) - std::fabs(QI(k - 1, i))));
                            v_adv = dt2 * (qp1 * CC(k - 1, i, i3) - qp * CC(k, i, i3) + qm * CC(k + 1, i, i3) -
                                           qm1 * CC(k, i, i3));
                            R = R + v_adv;
                            if (p.v_flux_limiter > 0) {
                                v_flux = 0.5 * dt2 *
                                         (PI_(k - 1, i, i3) * qp1 * (CC(k, i, i3) - CC(k - 1, i, i3)) -
                                          PI_(k, i, i3) * qp * (CC(k + 1, i, i3) - CC(k, i, i3)) +
                                          PI_(k, i, i3) * qm * (CC(k, i, i3) - CC(k + 1, i, i3)) -
                                          PI_(k - 1, i, i3) * qm1 * (CC(k - 1, i, i3) - CC(k, i, i3)));
                                R = R + v_flux;
                            }
                        }
                    }
                }
            }
            if (!tridiagonal_solver(L, nvl, ntr, am, bm, cm, rhs, sol, gm)) {
                set_err(c, GOM_E_ZERO_PIVOT, 1285, i, 0, 0.0, GOM_ENTITY_CELL);
                rc = GOM_E_ZERO_PIVOT;
                continue;
            }
            for (int k = b; k <= t; ++k) {
                int kk = t - k + 1;
                for (int i3 = 1; i3 <= ntr; ++i3) {
                    double s = sol[(size_t)(i3 - 1) * L + kk - 1];
                    if (s >= 0.0 && s <= 50.0) CN(k, i, i3) = s;
                    else if (s < 0.0) CN(k, i, i3) = 0.0;
                    else if (s > 50.0) CN(k, i, i3) = 50.0;
                }
            }
        }
        if (rc.load() != GOM_OK) return rc.load();
        // :1352-1372 copy back
        OMP_FOR
        for (int i = 1; i <= NC; ++i) {
            int b = c->bottom_layer_at_element(i), t = top_el(i);
            for (int k = b; k <= t; ++k)
                for (int i3 = 1; i3 <= ntr; ++i3) CC(k, i, i3) = CN(k, i, i3);
            for (int k = 0; k <= b - 1; ++k)
                for (int i3 = 1; i3 <= ntr; ++i3) CC(k, i, i3) = 0.0;
            for (int k = t + 1; k <= L + 1; ++k)
                for (int i3 = 1; i3 <= ntr; ++i3) CC(k, i, i3) = 0.0;
        }
    }
    // :1403-1467 node and face averages
    OMP_FOR
    for (int i = 1; i <= NN; ++i) {
        for (int k = top_n(i); k >= c->bottom_layer_at_node(i); --k) {
            if (top_n(i) == 0) break;
            for (int i3 = 1; i3 <= ntr; ++i3) {
                double s11 = 0.0, s22 = 0.0;
                int count1 = 0;
                for (int l = 1; l <= c->adj_cells_at_node(i); ++l) {
                    int ii = c->adj_cellnum_at_node(l, i);
                    if (k >= c->bottom_layer_at_element(ii) && k <= top_el(ii)) {
                        s11 = s11 + c->area(ii) * dz_cn(k, ii);
                        s22 = s22 + c->area(ii) * dz_cn(k, ii) * CN(k, ii, i3);
                    } else {
                        count1 = count1 + 1;
                    }
                }
                if (s11 == 0.0) NDN(k, i, i3) = 0.0;
                else NDN(k, i, i3) = s22 / s11;
                if (count1 == c->adj_cells_at_node(i) && k != top_n(i)) NDN(k, i, i3) = NDN(k + 1, i, i3);
            }
        }
    }
    OMP_FOR
    for (int j = 1; j <= NF; ++j) {
        int n1 = c->nodenum_at_face(1, j), n2 = c->nodenum_at_face(2, j);
        for (int k = c->bottom_layer_at_face(j); k <= top_f(j); ++k)
            for (int i3 = 1; i3 <= ntr; ++i3) FCN(k, j, i3) = (NDN(k, n1, i3) + NDN(k, n2, i3)) * 0.5;
    }
    // :1471-1482 write back (slot 1 = salinity, slot 2 = temperature)
    for (int i3 = 1; i3 <= ntr; ++i3) {
        int tid = tran_id[i3 - 1];
        int slot = tid;  // the reference copies con_*(:,:,1) to salt and (:,:,2) to temperature
        if (slot > ntr) continue;
        A2<double> dc = FD(c, tid == 1 ? GOM_F_SALT_CELL_NEW : GOM_F_TEMP_CELL_NEW);
        A2<double> dn = FD(c, tid == 1 ? GOM_F_SALT_NODE : GOM_F_TEMP_NODE);
        A2<double> df = FD(c, tid == 1 ? GOM_F_SALT_FACE : GOM_F_TEMP_FACE);
        OMP_FOR
        for (int i = 1; i <= NC; ++i)
            for (int k = 1; k <= L; ++k) dc(k, i) = CN(k, i, slot);
        OMP_FOR
        for (int i = 1; i <= NN; ++i)
            for (int k = 1; k <= L; ++k) dn(k, i) = NDN(k, i, slot);
        OMP_FOR
        for (int j = 1; j <= NF; ++j)
            for (int k = 1; k <= L; ++k) df(k, j) = FCN(k, j, slot);
    }
    return GOM_OK;
}

// calculate_density_full.f90:13-246 (ana_density 0) and calculate_density_linear.f90:10 (1)
namespace {
double eos_surface(double rtemp, double rsalt) {
    double t2 = rtemp * rtemp, t3 = t2 * rtemp, t4 = t2 * t2, t5 = t3 * t2;
    double sq = std::sqrt(rsalt);
    double sq3 = sq * sq * sq;
    double c0 = (double)(1000.0f - 0.157406f);
    return c0 + F(6.793952e-2f) * rtemp - F(9.095290e-3f) * t2 + F(1.001685e-4f) * t3 - F(1.120083e-6f) * t4 +
           F(6.536332e-9f) * t5 +
           rsalt * (F(0.824493f) - F(4.089900e-3f) * rtemp + F(7.643800e-5f) * t2 - F(8.246700e-7f) * t3 +
                    F(5.387500e-9f) * t4) +
           sq3 * (F(-5.72466e-3f) + F(1.022700e-4f) * rtemp - F(1.654600e-6f) * t2) + F(4.831400e-4f) * (rsalt * rsalt);
}
double eos_bulk(double rtemp, double rsalt, double pres) {
    double t2 = rtemp * rtemp, t3 = t2 * rtemp, t4 = t2 * t2;
    double sq = std::sqrt(rsalt);
    double sq3 = sq * sq * sq;
    double p2 = pres * pres;
    return F(19652.21f) + F(148.4206f) * rtemp - F(2.327105f) * t2 + F(1.360477e-2f) * t3 - F(5.155288e-5f) * t4 +
           pres * (F(3.239908f) + F(1.43713e-3f) * rtemp + F(1.16092e-4f) * t2 - F(5.77905e-7f) * t3) +
           p2 * (F(8.50935e-5f) - F(6.12293e-6f) * rtemp + F(5.2787e-8f) * t2) +
           rsalt * (F(54.6746f) - F(0.603459f) * rtemp + F(1.09987e-2f) * t2 - F(6.1670e-5f) * t3) +
           sq3 * (F(7.944e-2f) + F(1.6483e-2f) * rtemp - F(5.3009e-4f) * t2) +
           pres * rsalt * (F(2.2838e-3f) - F(1.0981e-5f) * rtemp - F(1.6078e-6f) * t2) +
           F(1.91075e-4f) * pres * sq3 - F(9.9348e-7f) * p2 * rsalt + F(2.08160e-8f) * rtemp * p2 * rsalt +
           F(9.1697e-10f) * t2 * p2 * rsalt;
}
}  // namespace

int gom_step_density(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    const gom_params &p = c->p;
    if (p.baroclinic_flag != 1) return GOM_OK;
    const int L = c->L;
    const double tmin = -5.0, tmax = 100.0, smin = -5.0, smax = 100.0;
    A2<double> rho_node = FD(c, GOM_F_RHO_NODE), rho_face = FD(c, GOM_F_RHO_FACE), rho_cell = FD(c, GOM_F_RHO_CELL),
               temp_node = FD(c, GOM_F_TEMP_NODE), salt_node = FD(c, GOM_F_SALT_NODE), temp_face = FD(c, GOM_F_TEMP_FACE),
               salt_face = FD(c, GOM_F_SALT_FACE), dz_node = FD(c, GOM_F_DZ_NODE), dz_face = FD(c, GOM_F_DZ_FACE);
    A1<int32_t> top_n = FI1(c, GOM_F_TOP_LAYER_NODE), top_f = FI1(c, GOM_F_TOP_LAYER_FACE),
                top_el = FI1(c, GOM_F_TOP_LAYER_CELL);
    const double c981 = F(9.81f), c1e5h = (double)(1.0e-5f * 0.5f), c1e5 = F(1.0e-5f);
    auto column = [&](A2<double> rho, A2<double> tt, A2<double> ss, A2<double> dz, int e, int b, int t, int site,
                      int kind) {
        for (int k = b; k <= t; ++k) {
            double rtemp = tt(k, e), rsalt = ss(k, e);
            if (rtemp < tmin || rtemp > tmax || rsalt < smin || rsalt > smax) {
                set_err(c, GOM_E_DENSITY, site, e, k, rtemp < tmin || rtemp > tmax ? rtemp : rsalt, kind);
                return false;
            }
            if (p.ana_density == 1) {
                rho(k, e) = F(1000.0f) + F(0.7f) * rsalt;
            } else {
                rho(k, e) = eos_surface(rtemp, rsalt);
                if (p.msl - c->zl(k) > F(100.0f)) {
                    double pres = F(0.0f);
                    for (int kk = k; kk <= t; ++kk) {
                        double ptmp = c981 * rho(kk, e) * dz(kk, e);
                        if (kk == k) pres = pres + c1e5h * ptmp;
                        else pres = pres + c1e5 * ptmp;
                    }
                    double sbm = eos_bulk(rtemp, rsalt, pres);
                    double ratio = 1.0 / (1.0 - pres / sbm);
                    rho(k, e) = rho(k, e) * ratio;
                }
            }
            if (rho(k, e) < F(980.0f)) {
                set_err(c, GOM_E_DENSITY, site, e, k, rho(k, e), kind);
                return false;
            }
        }
        for (int k = 1; k <= b - 1; ++k) rho(k, e) = rho(b, e);
        for (int k = t + 1; k <= L; ++k) rho(k, e) = rho(t, e);
        return true;
    };
    for (int i = 1; i <= c->NN; ++i)
        if (top_n(i) != 0)
            if (!column(rho_node, temp_node, salt_node, dz_node, i, c->bottom_layer_at_node(i), top_n(i), 43, GOM_ENTITY_NODE))
                return GOM_E_DENSITY;
    if (p.ana_density == 0)
        for (int j = 1; j <= c->NF; ++j)
            if (top_f(j) != 0)
                if (!column(rho_face, temp_face, salt_face, dz_face, j, c->bottom_layer_at_face(j), top_f(j), 130, GOM_ENTITY_FACE))
                    return GOM_E_DENSITY;
    for (int i = 1; i <= c->NC; ++i) {
        int t = top_el(i), b = c->bottom_layer_at_element(i);
        if (t == 0) continue;
        for (int k = b; k <= t; ++k) {
            rho_cell(k, i) = F(0.0f);
            int icount = 0;
            for (int l = 1; l <= c->tri_or_quad(i); ++l) {
                int nd = c->nodenum_at_cell(l, i);
                if (top_n(nd) != 0) {
                    icount = icount + 1;
                    rho_cell(k, i) = rho_cell(k, i) + rho_node(k, nd);
                }
            }
            if (icount == 0) {
                set_err(c, GOM_E_DRY, 224, i, k, 0.0, GOM_ENTITY_CELL);
                return GOM_E_DRY;
            }
            rho_cell(k, i) = rho_cell(k, i) / icount;
        }
        for (int k = 1; k <= b - 1; ++k) rho_cell(k, i) = rho_cell(b, i);
        for (int k = t + 1; k <= L; ++k) rho_cell(k, i) = rho_cell(t, i);
    }
    return GOM_OK;
}

// turbulence_closure_v1.f90:72-138 (i_turbulence_flag 1 and 2).  The reference routine is never
// called by its time loop and names arrays of another model; they map here to this model's:
// srho -> rho_face, velocity_normal/tangnt -> un/vn_face (the step's new velocities),
// dzhalf -> dzhalf_face (new), h_at_face_center -> h_face, ref_water_density -> rho_o.  The face
// viscosity of interface k (top of layer k) is Av(k, face); the transport diffusivity of a cell
// interface is the mean over the cell's wet faces of the face diffusivity at the level clamped to
// the face's wet range, as :446-470 forms it for nodes, with 1e-2 where no face is wet.
int gom_step_turbulence(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    const gom_params &p = c->p;
    if (p.turbulence_flag != 1 && p.turbulence_flag != 2) return GOM_OK;
    const int L = c->L;
    A2<double> rho_face = FD(c, GOM_F_RHO_FACE), un = FD(c, GOM_F_UN_FACE_NEW), vn = FD(c, GOM_F_VN_FACE_NEW),
               dzh = FD(c, GOM_F_DZHALF_FACE_NEW), av = FD(c, GOM_F_AV), kv = FD(c, GOM_F_KV);
    A1<int32_t> top_f = FI1(c, GOM_F_TOP_LAYER_FACE), top_el = FI1(c, GOM_F_TOP_LAYER_CELL);
    std::vector<double> kvf_store((size_t)(L + 1) * c->NF, 0.0);
    A2<double> kvf{kvf_store.data(), 0, L + 1};
    const double g = p.gravity;
    for (int i = 1; i <= c->NF; ++i) {
        int b = c->bottom_layer_at_face(i), t = top_f(i);
        double vmax = 0.0, vmin = 0.0;
        if (p.turbulence_flag == 2) {
            double h = c->h_face(i);
            if (h <= p.pp_h1) {
                vmax = p.pp_vdmax1;
                vmin = p.pp_vdmin1;
            } else if (h < p.pp_h2) {
                vmax = p.pp_vdmax1 + (p.pp_vdmax2 - p.pp_vdmax1) * (h - p.pp_h1) / (p.pp_h2 - p.pp_h1);
                vmin = p.pp_vdmin1 + (p.pp_vdmin2 - p.pp_vdmin1) * (h - p.pp_h1) / (p.pp_h2 - p.pp_h1);
            } else {
                vmax = p.pp_vdmax2;
                vmin = p.pp_vdmin2;
            }
        }
        for (int k = b; k <= t; ++k) {
            double ri;
            if (k == t) {
                ri = F(0.0f);
            } else {
                double drhodz = (rho_face(k + 1, i) - rho_face(k, i)) / dzh(k, i);
                double bvf = -g * (drhodz / p.rho_o + g / (double)(1.5e3f * 1.5e3f));
                double dundz = (un(k + 1, i) - un(k, i)) / dzh(k, i);
                double dutdz = (vn(k + 1, i) - vn(k, i)) / dzh(k, i);
                double shear2 = dundz * dundz + dutdz * dutdz;
                shear2 = std::max(shear2, 1.0e-10);
                ri = std::max(bvf / shear2, 0.0);
            }
            if (p.turbulence_flag == 1) {
                const double vdiffc = 1.0e-3, tdiffc = F(1.0f) * vdiffc;
                if (ri < F(0.25f)) {
                    av(k, i) = vdiffc;
                    kvf(k, i) = tdiffc;
                } else {
                    av(k, i) = 1.0e-5;
                    kvf(k, i) = 1.0e-5;
                }
            } else {
                double x = 1.0 + 5.0 * ri;
                av(k, i) = vmax / (x * x) + vmin;
                kvf(k, i) = av(k, i) / (F(1.0f) + F(5.0f) * ri) + p.pp_tdmin;
            }
        }
    }
    for (int i = 1; i <= c->NC; ++i) {
        int t = top_el(i);
        if (t == 0) continue;
        for (int k = c->bottom_layer_at_element(i); k <= t; ++k) {
            double sum = 0.0;
            int icount = 0;
            for (int l = 1; l <= c->tri_or_quad(i); ++l) {
                int isd = c->facenum_at_cell(l, i);
                if (top_f(isd) != 0) {
                    icount = icount + 1;
                    int klev = std::min(std::max(k, c->bottom_layer_at_face(isd)), top_f(isd));
                    sum = sum + kvf(klev, isd);
                }
            }
            kv(k, i) = icount == 0 ? F(1.0e-2f) : sum / icount;
        }
    }
    return GOM_OK;
}

// update_variables.f90:16-31 (state part; the vertical means feed output only)
int gom_step_swap(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    const int pairs[][2] = {{GOM_F_ETA_CELL, GOM_F_ETA_CELL_NEW},     {GOM_F_WN_CELL, GOM_F_WN_CELL_NEW},
                            {GOM_F_DZ_CELL, GOM_F_DZ_CELL_NEW},       {GOM_F_DZHALF_CELL, GOM_F_DZHALF_CELL_NEW},
                            {GOM_F_SALT_CELL, GOM_F_SALT_CELL_NEW},   {GOM_F_TEMP_CELL, GOM_F_TEMP_CELL_NEW},
                            {GOM_F_UN_FACE, GOM_F_UN_FACE_NEW},       {GOM_F_VN_FACE, GOM_F_VN_FACE_NEW},
                            {GOM_F_DZ_FACE, GOM_F_DZ_FACE_NEW},       {GOM_F_DZHALF_FACE, GOM_F_DZHALF_FACE_NEW},
                            {GOM_F_DZ_NODE, GOM_F_DZ_NODE_NEW},       {GOM_F_DZHALF_NODE, GOM_F_DZHALF_NODE_NEW}};
    for (auto &pr : pairs) c->fd[pr[0]] = c->fd[pr[1]];
    return GOM_OK;
}

// heat_term_by_term.f90:27-156 with sol_swr 2, before the transport: the air series at
// julian_day (no interval: zeros), the scalar terms, then per wet column phi_sw and phi_sz from its
// top and bottom temperatures (the top layer after the layer update, the old thicknesses).  Default-
// REAL constants widened from single precision; integer powers as products (x^4 = (x^2)^2,
// x^6 = (x^2 x)^2); exp, log and pow of the C library (the GPU's differ in the last bits)
// julian_to_localtime.f90:16-86 with its state: the hour of julian day jday.  The month table is
// saved between calls and set with the month; in a leap year (other than 1900) only while the
// month variable is 3 or more (so a run starting in January or February keeps a zero table)
static int local_hour(int year, int &month, int &table_set, double jday) {
    static const double leap[12] = {0, 32, 60, 91, 121, 152, 182, 213, 244, 274, 305, 335};
    static const double normal[12] = {0, 31, 59, 90, 120, 151, 181, 212, 243, 273, 304, 334};
    static const double leap_top[11] = {31, 60, 91, 121, 152, 182, 213, 244, 274, 305, 335};
    static const double normal_top[11] = {31, 59, 90, 120, 151, 181, 212, 243, 273, 304, 334};
    double m;
    if (year % 4 == 0) {
        if (year != 1900 && month >= 3) {
            int k = 0;
            while (k < 11 && jday > leap_top[k]) ++k;
            month = k + 1;
            table_set = 1;
        }
        m = table_set ? leap[month - 1] : 0.0;
    } else {
        int k = 0;
        while (k < 11 && jday > normal_top[k]) ++k;
        month = k + 1;
        table_set = 2;
        m = normal[month - 1];
    }
    const double day_temp = jday - m;
    const int day = (int)day_temp + 1;
    return (int)((day_temp + 1 - day) * 24.0);
}

static void heat_terms(gom_ctx *c) {
    const int L = c->L, NC = c->NC, n = (int)c->air_time.size();
    const double u2 = c->jday * 86400.0;
    double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int t = 1; t < n; ++t) {
        const double u1 = c->air_time[t - 1] - c->rdd_s, u3 = c->air_time[t] - c->rdd_s;
        if (u2 >= u1 && u2 <= u3) {
            for (int k = 0; k < 5; ++k) {
                const double v1 = c->air_values[(size_t)k * n + t - 1], v3 = c->air_values[(size_t)k * n + t];
                v[k] = (u2 - u1) * (v3 - v1) / (u3 - u1) + v1;
            }
            break;
        }
    }
    const double Ta = v[0], Tdew = v[1], w_speed = v[2], sol_rad = v[3], cloud = v[4];
    const double c2 = cloud * cloud;
    double phi_sn = 0.0;   // sol_swr 1 with the sun below the horizon: the reference leaves it unset
    if (c->sol_swr == 1) {
        // :64-83: the sun's elevation A0 at the local hour, and the clear-sky short-wave from it
        const int hr = local_hour(c->year, c->month, c->month_table_set, c->jday);
        const double pi = 3.141592653589793, deg2rad = pi / 180.0, rad2deg = 180.0 / pi;
        const double j_day = c->jday + 1;
        const double tau_d = 2.0 * pi * (double)((int)(j_day + 1) - 1) / 365.0;
        const double sdec = (double)0.006918f - (double)0.399912f * std::cos(tau_d) + (double)0.070257f * std::sin(tau_d) -
                            (double)0.006758f * std::cos(2.0 * tau_d) + (double)0.000907f * std::sin(2.0 * tau_d) -
                            (double)0.002697f * std::cos(3.0 * tau_d) + (double)0.001480f * std::sin(3.0 * tau_d);
        const double eqt = (double)0.170f * std::sin(4.0 * pi * (double)((int)j_day - 80) / 373.0) -
                           (double)0.129f * std::sin(2.0 * pi * (double)((int)j_day - 8) / 355.0);
        const double sm = 15.0 * (double)(int)(c->lon / 15.0);
        const double lha = (double)0.261799f * ((double)hr - (c->lon - sm) * (double)0.0666667f + eqt - 12.0);
        const double a0 = std::asin(std::sin(c->lat * deg2rad) * std::sin(sdec) +
                                    std::cos(c->lat * deg2rad) * std::cos(sdec) * std::cos(lha)) * rad2deg;
        if (a0 > 0.0) {
            const double a2 = a0 * a0, a3 = a2 * a0, a4 = a2 * a2;
            phi_sn = (1.0 - (double)0.65f * c2) * 24.0 *
                     ((double)2.0444f * a0 + (double)0.1296f * a2 - (double)1.941e-3f * a3 + (double)7.591e-6f * a4) *
                     (double)0.1314f;
        }
    } else {
        phi_sn = (1.0 - (double)0.65f * c2) * sol_rad;
    }
    const double xa = Ta + 273.15;
    double phi_ac;
    if (Ta >= 5.0) {
        const double x2 = xa * xa, x3 = x2 * xa;
        phi_ac = (double)5.31e-13f * (x3 * x3);
    } else {
        const double x2 = xa * xa;
        phi_ac = (double)5.67e-8f * (x2 * x2) * (1.0 - (double)0.261f * std::exp(-((double)7.77e-4f * (Ta * Ta))));
    }
    const double phi_an = phi_ac * (1.0 + (double)0.17f * c2) * 0.97;
    const double z0 = w_speed <= (double)2.3f ? (double)0.001f : (double)0.005f;
    const double alpha = std::log(c->wind_height / z0) / std::log(2.0 / z0);
    const double bz = c->fwz_b / std::pow(alpha, c->fwz_c);
    const double fwz = c->fwz_a + bz * std::pow(w_speed, c->fwz_c);
    const double ea = std::exp(2.3026 * (7.5 * Tdew / (Tdew + 237.3) + (double)0.6609f));
    A2<double> temp_cell = FD(c, GOM_F_TEMP_CELL), dz_cell = FD(c, GOM_F_DZ_CELL);
    A1<int32_t> top_el = FI1(c, GOM_F_TOP_LAYER_CELL);
    for (int i = 1; i <= NC; ++i) {
        double *phi_sz = c->phi_sz.data() + (size_t)(i - 1) * L;
        const int tl = top_el(i), b = c->bottom_layer_at_element(i);
        if (tl == 0) {
            for (int k = 1; k <= L; ++k) phi_sz[k - 1] = 0.0;
            continue;
        }
        const double Tw = temp_cell(tl, i);
        const double xw = Tw + (double)273.15f, x2 = xw * xw;
        const double phi_br = (double)(0.97f * 5.67e-8f) * (x2 * x2);
        const double es = Tw < 0.0 ? std::exp(2.3026 * (9.5 * Tw / (Tw + 265.5) + (double)0.6609f))
                                   : std::exp(2.3026 * (7.5 * Tw / (Tw + 237.3) + (double)0.6609f));
        const double phi_e = fwz * (es - ea);
        const double phi_c = 0.47 * fwz * (Tw - Ta);
        const double phi_n = phi_sn + phi_an - phi_br - phi_e - phi_c;
        const double phi_sw = c->sed_water_exchange * (c->t_sed - temp_cell(b, i));
        c->phi_sw[i - 1] = phi_sw;
        double sol_out = (1.0 - c->sol_absorb) * phi_sn * std::exp(-(c->light_extinction * dz_cell(tl, i)));
        phi_sz[tl - 1] = phi_n - sol_out;
        for (int k = tl - 1; k >= b; --k) {
            const double sol_in = sol_out;
            sol_out = sol_in * std::exp(-(c->light_extinction * dz_cell(k, i)));
            phi_sz[k - 1] = sol_in - sol_out;
        }
        for (int k = b; k <= tl; ++k) {
            phi_sz[k - 1] = phi_sz[k - 1] + sol_out * c->sed_temp_coeff;
            phi_sz[k - 1] = phi_sz[k - 1] + phi_sw;
        }
    }
}

int gom_step_all(gom_ctx *c, int32_t *pcg_iters) {
    if (!c) return GOM_E_ARG;
    int e;
    if (c->has_series) series_forcing(c);
    if ((e = gom_step_bottom_friction(c))) return e;
    if ((e = gom_step_boundary_velocity(c))) return e;
    if ((e = gom_step_advection(c))) return e;
    if ((e = gom_step_momentum(c))) return e;
    if ((e = gom_step_free_surface(c, pcg_iters))) return e;
    if ((e = gom_step_velocities(c))) return e;
    if ((e = gom_step_layers(c))) return e;
    if ((e = gom_step_node_velocity(c))) return e;
    if (c->has_series && c->heat_flag == 1) heat_terms(c);
    if ((e = gom_step_transport(c))) return e;
    if ((e = gom_step_density(c))) return e;
    if ((e = gom_step_turbulence(c))) return e;
    return gom_step_swap(c);
}

int gom_step_launch(gom_ctx *c) {
    if (!c) return GOM_E_ARG;
    c->pending_rc = gom_step_all(c, &c->pending_iters);
    return GOM_OK;
}

int gom_step_wait(gom_ctx *c, int32_t *pcg_iters) {
    if (!c) return GOM_E_ARG;
    if (pcg_iters) *pcg_iters = c->pending_iters;
    return c->pending_rc;
}

// spec: check_conservation.f90:28-57
// read_main_inp.f90:1143-1154 (station ids), kept for write_tser_out_files
int gom_push_hurricane_frame(gom_ctx *c, const double *frame) {
    if (!c || !frame || !c->has_series || c->hur_flag != 1) return GOM_E_ARG;
    c->hur_next.assign(frame, frame + 3 * (size_t)c->NN);
    c->hur_ready = true;
    return GOM_OK;
}

int gom_push_hurricane_center(gom_ctx *c, double x, double y, double julian_day) {
    if (!c || !c->has_series || c->hur_flag != 1 || c->hur_method != 2) return GOM_E_ARG;
    c->track_next[0] = x;
    c->track_next[1] = y;
    c->track_next[2] = julian_day;
    c->track_ready = true;
    return GOM_OK;
}

int gom_set_stations(gom_ctx *c, int32_t hloc, int32_t n_stations, const int32_t *station_cell,
                     const int32_t *station_node) {
    if (!c || (hloc != 1 && hloc != 2) || n_stations < 0) return GOM_E_ARG;
    const int32_t *ids = hloc == 1 ? station_cell : station_node;
    if (n_stations > 0 && !ids) return GOM_E_ARG;
    for (int q = 0; q < n_stations; ++q)
        if (ids[q] < 1 || ids[q] > (hloc == 1 ? c->NC : c->NN)) return GOM_E_ARG;
    c->tser_hloc = hloc;
    c->tser_station.assign(ids, ids + n_stations);
    return GOM_OK;
}

// write_tser_out_files.f90:9-330 with the node means of update_variables.f90:36-72; one record of
// 7 + 4 L values per station: eta, H, ubar, u(1:L), vbar, v(1:L), sbar, salt(1:L), tbar,
// temp(1:L), air pressure
int gom_station_series(gom_ctx *c, double *out) {
    const int n = c ? (int)c->tser_station.size() : 0;
    if (!c || (n > 0 && !out)) return GOM_E_ARG;
    const int L = c->L, rec = 7 + 4 * L;
    A1<double> eta_cell = FD1(c, GOM_F_ETA_CELL), eta_node = FD1(c, GOM_F_ETA_NODE);
    A2<double> u_node = FD(c, GOM_F_U_NODE), v_node = FD(c, GOM_F_V_NODE);
    A2<double> salt_cell = FD(c, GOM_F_SALT_CELL), temp_cell = FD(c, GOM_F_TEMP_CELL);
    A2<double> salt_node = FD(c, GOM_F_SALT_NODE), temp_node = FD(c, GOM_F_TEMP_NODE);
    A1<int32_t> top_el = FI1(c, GOM_F_TOP_LAYER_CELL), top_nd = FI1(c, GOM_F_TOP_LAYER_NODE);
    for (int is = 1; is <= n; ++is) {
        double *o = out + (long)(is - 1) * rec;
        // record slots: eta, H, then for X in u, v, salt, temp the mean at X(0) and X(1:L)
        auto U = [&](int k) -> double & { return o[2 + k]; };
        auto V = [&](int k) -> double & { return o[3 + L + k]; };
        auto S = [&](int k) -> double & { return o[4 + 2 * L + k]; };
        auto T = [&](int k) -> double & { return o[5 + 3 * L + k]; };
        if (c->tser_hloc == 1) {
            const int ie = c->tser_station[is - 1];
            o[0] = eta_cell(ie);
            o[1] = c->h_cell(ie) + eta_cell(ie);
            double u_cell[GOM_ORACLE_MAXL + 1] = {0.0}, v_cell[GOM_ORACLE_MAXL + 1] = {0.0};
            double ubar = 0.0, vbar = 0.0, sbar = 0.0, tbar = 0.0;
            if (top_el(ie) != 0) {
                const int nvl = top_el(ie) - c->bottom_layer_at_element(ie) + 1;
                for (int k = c->bottom_layer_at_element(ie); k <= top_el(ie); ++k) {
                    for (int l = 1; l <= c->tri_or_quad(ie); ++l) {
                        const int nd = c->nodenum_at_cell(l, ie);
                        u_cell[k] = u_cell[k] + u_node(k - 1, nd) + u_node(k, nd);
                    }
                    u_cell[k] = u_cell[k] / (c->tri_or_quad(ie) * 2);
                }
                for (int k = c->bottom_layer_at_element(ie); k <= top_el(ie); ++k) ubar = ubar + u_cell[k];
                ubar = ubar / nvl;
                for (int k = c->bottom_layer_at_element(ie); k <= top_el(ie); ++k) {
                    for (int l = 1; l <= c->tri_or_quad(ie); ++l) {
                        const int nd = c->nodenum_at_cell(l, ie);
                        v_cell[k] = v_cell[k] + v_node(k - 1, nd) + v_node(k, nd);
                    }
                    v_cell[k] = v_cell[k] / (c->tri_or_quad(ie) * 2);
                }
                for (int k = c->bottom_layer_at_element(ie); k <= top_el(ie); ++k) vbar = vbar + v_cell[k];
                vbar = vbar / nvl;
                for (int k = c->bottom_layer_at_element(ie); k <= top_el(ie); ++k) sbar = sbar + salt_cell(k, ie);
                sbar = sbar / nvl;
                for (int k = c->bottom_layer_at_element(ie); k <= top_el(ie); ++k) tbar = tbar + temp_cell(k, ie);
                tbar = tbar / nvl;
            }
            U(0) = ubar;
            V(0) = vbar;
            S(0) = sbar;
            T(0) = tbar;
            for (int k = 1; k <= L; ++k) {
                U(k) = u_cell[k];
                V(k) = v_cell[k];
                S(k) = salt_cell(k, ie);
                T(k) = temp_cell(k, ie);
            }
            // :312: air_p1 has n_nodes entries and is read at the cell id
            o[6 + 4 * L] = ie <= c->NN ? c->air_p[ie - 1] : 0.0;
        } else {
            const int i = c->tser_station[is - 1];
            o[0] = eta_node(i);
            o[1] = c->h_node(i) + eta_node(i);
            const int nvl = top_nd(i) - c->bottom_layer_at_node(i) + 1;
            double ubar = 0.0, vbar = 0.0, sbar = 0.0, tbar = 0.0;
            if (nvl != 0) {
                double su = 0.0, sv = 0.0, ss = 0.0, st = 0.0;
                for (int k = c->bottom_layer_at_node(i) - 1; k <= top_nd(i); ++k) {
                    su = su + u_node(k, i);
                    sv = sv + v_node(k, i);
                }
                ubar = su / (nvl + 1);
                vbar = sv / (nvl + 1);
                for (int k = c->bottom_layer_at_node(i); k <= top_nd(i); ++k) {
                    ss = ss + salt_node(k, i);
                    st = st + temp_node(k, i);
                }
                sbar = ss / nvl;
                tbar = st / nvl;
            }
            U(0) = ubar;
            V(0) = vbar;
            S(0) = sbar;
            T(0) = tbar;
            for (int k = 1; k <= L; ++k) {
                U(k) = u_node(k, i);
                V(k) = v_node(k, i);
                S(k) = salt_node(k, i);
                T(k) = temp_node(k, i);
            }
            o[6 + 4 * L] = c->air_p[i - 1];
        }
    }
    return GOM_OK;
}

int gom_conservation(gom_ctx *c, double *volume, double *salt_mass) {
    if (!c) return GOM_E_ARG;
    A2<double> dz_cell = FD(c, GOM_F_DZ_CELL), salt = FD(c, GOM_F_SALT_CELL);
    A1<int32_t> top_el = FI1(c, GOM_F_TOP_LAYER_CELL);
    double v = 0.0, s = 0.0;
    for (int i = 1; i <= c->NC; ++i) {
        for (int k = c->bottom_layer_at_element(i); k <= top_el(i); ++k) {
            double vv = c->area(i) * dz_cell(k, i);
            v = v + vv;
            s = s + vv * salt(k, i);
        }
    }
    if (volume) *volume = v;
    if (salt_mass) *salt_mass = s;
    return GOM_OK;
}

// ---------------------------------------------------------------- test hooks (KATs only)
// The restated building blocks, callable one at a time by the known-answer tests.
// threads of the OpenMP timing build (n > 0 sets them); returns the count a parallel loop uses
// (always 1 in the serial build)
int gom_oracle_threads(int32_t n) {
#ifdef GOM_ORACLE_OMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

int gom_oracle_tridiagonal(int32_t n, int32_t nc, const double *a, const double *b, const double *c,
                           const double *rhs, double *sol) {
    if (n <= 0 || nc <= 0) return GOM_E_ARG;
    std::vector<double> gam(n + 1, 0.0);
    return tridiagonal_solver(n, n, nc, a, b, c, rhs, sol, gam.data()) ? GOM_OK : GOM_E_ZERO_PIVOT;
}

int gom_oracle_bilinear(const double *xq, const double *yq, double x, double y, double *shapef) {
    double xi = 0.0, eta = 0.0;
    return bilinear_interpolation(xq[0], xq[1], xq[2], xq[3], yq[0], yq[1], yq[2], yq[3], x, y, xi, eta, shapef);
}

int gom_oracle_check_intersection(const double *seg, double *xy) {
    int iflag = 0;
    check_intersection(seg[0], seg[1], seg[2], seg[3], seg[4], seg[5], seg[6], seg[7], iflag, xy[0], xy[1]);
    return iflag;
}

}  // extern "C"
