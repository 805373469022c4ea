// k_hydro.cu -- bottom friction, river boundary velocity, ELM advection and the per-face momentum
// tridiagonal solves of GOM's per-timestep core, for sm_103a.
//
// References (GOM_Rv1.1.0/source):
//   calculate_bottom_friction.f90:9-73, compute_boundary_velocity.f90:60-94,
//   solve_nonlinear_advection.f90:14-204, ELM_backtrace_v1.f90:15-200,
//   search_straight_line.f90:15-399, check_intersection.f90:14-50,
//   bilinear_interpolation.f90:8-121, solve_momentum_equation.f90:15-656,
//   tridiagonal_solver.f90:15-90.
#include <type_traits>

#include "gom_launch.h"
#include "gom_scan.cuh"

namespace gom {

// ============================================================================================
// calculate_bottom_friction.f90:21-63; bf_flag 3 is the constant-Cd extension. One thread per face.
template <typename R> __global__ void k_bottom_friction(Geom g, StateT<R> s, Params p) {
    int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (j > g.NF) return;
    const int L = g.L;
    double cdb = 0.0, gb = 0.0;
    double hf = g.h_face[j - 1];
    if (p.bf_flag >= 1 && p.bf_flag <= 3 && hf > p.dry_depth) {
        int k = g.bottom_face[j - 1];
        if (p.bf_flag == 1) {
            double hr = fmax(1.0, hf);
            double chezy = pow(hr, 1.0 / 6.0) / g.manning[j - 1];
            cdb = p.gravity / (chezy * chezy);
        } else if (p.bf_flag == 2) {
            double lg = log(fmax(0.5, s.dzhalf_face[ix0(k - 1, j, L)]) / g.bf_height[j - 1]);
            cdb = p.von_karman * p.von_karman / (lg * lg);
        } else {
            cdb = p.cd_const;
        }
        double u = s.un_face[ix(k, j, L)], v = s.vn_face[ix(k, j, L)];
        gb = cdb * sqrt(u * u + v * v);
    }
    s.cdb[j - 1] = (R)cdb;
    s.gamma_b[j - 1] = (R)gb;
}

template <typename R> cudaError_t launch_bottom_friction(const LaunchT<R> &x) {
    k_bottom_friction<<<blocks_for(x.g.NF, 256), 256, 0, x.stream>>>(x.g, x.s, x.p);
    return cudaGetLastError();
}

// compute_boundary_velocity.f90:71-92. One thread per river cell.
template <typename R> __global__ void k_boundary_velocity(Geom g, StateT<R> s, Forcing f, Params p, gom_status *st) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i > g.NQB) return;
    int j = g.qb_face[i - 1];
    int n1 = g.face_node(1, j), n2 = g.face_node(2, j);
    double depth = g.h_face[j - 1] + (s.eta_node[n1 - 1] + s.eta_node[n2 - 1]) * 0.5;
    if (depth < p.dry_depth) {
        record_error(st, GOM_E_DRY, 80, i, 0, depth);
        return;
    }
    s.qu_boundary[i - 1] = -f.q_add[i - 1] / (g.face_length[j - 1] * depth);
}

template <typename R> cudaError_t launch_boundary_velocity(const LaunchT<R> &x) {
    if (x.g.NQB == 0) return cudaSuccess;
    k_boundary_velocity<<<blocks_for(x.g.NQB, 128), 128, 0, x.stream>>>(x.g, x.s, x.f, x.p, x.status);
    return cudaGetLastError();
}

// ============================================================================================
// ELM
// check_intersection.f90:14-50.  tt1 = delta1/delta and tt2 = delta2/delta must both lie in
// [0, 1]; the sign test is exact, the upper bound is decided from |delta_i| against |delta|
// unless the two are within 1e-9 of each other, and tt1 is divided out only for a hit.
__device__ __forceinline__ int unit_range(double num, double den) {
    // 1 if fl(num/den) in [0,1], 0 if not (den != 0)
    if (num == 0.0) return 1;
    if ((num < 0.0) != (den < 0.0)) return 0;
    double an = fabs(num), ad = fabs(den);
    if (an < ad * (1.0 - 1e-9)) return 1;
    if (an > ad * (1.0 + 1e-9)) return 0;
    return num / den <= 1.0;
}

__device__ __forceinline__ int check_intersection(double x1, double x2, double x3, double x4, double y1, double y2,
                                                  double y3, double y4, double &xin, double &yin) {
    double delta = (x2 - x1) * (y3 - y4) - (y2 - y1) * (x3 - x4);
    if (delta == 0.0) return 0;
    double delta1 = (x3 - x1) * (y3 - y4) - (y3 - y1) * (x3 - x4);
    if (!unit_range(delta1, delta)) return 0;
    double delta2 = (x2 - x1) * (y3 - y1) - (y2 - y1) * (x3 - x1);
    if (!unit_range(delta2, delta)) return 0;
    double tt1 = delta1 / delta;
    xin = x1 + (x2 - x1) * tt1;
    yin = y1 + (y2 - y1) * tt1;
    return 1;
}

// bilinear_interpolation.f90:8-121: returns 0 or GOM_ELM_BILINEAR
// (T = T: the reference arithmetic; T = float: the mixed path, on element-local coordinates)
template <typename T>
__device__ int bilinear_interpolation(T x1, T x2, T x3, T x4, T y1, T y2, T y3, T y4, T x, T y, T shapef[4]) {
    const T small3 = (T)F(1.e-5f), small_06 = (T)F(1.e-6f), b11 = (T)F(1.1f);
    T xi = T(0.0), eta = T(0.0);
    T x0 = (x1 + x2 + x3 + x4) / T(4.0);
    T y0 = (y1 + y2 + y3 + y4) / T(4.0);
    T axi0 = x2 - x1 + x3 - x4, axi1 = y2 - y1 + y3 - y4;
    T aet0 = x3 + x4 - x1 - x2, aet1 = y3 + y4 - y1 - y2;
    T bxy0 = x1 - x2 + x3 - x4, bxy1 = y1 - y2 + y3 - y4;
    T dxi = T(2.0) * ((x3 - x4) * (y1 - y2) - (y3 - y4) * (x1 - x2));
    T deta = T(2.0) * ((x4 - x1) * (y3 - y2) - (y4 - y1) * (x3 - x2));
    if ((fabs(bxy0) < small3 && fabs(bxy1) < small3) || (fabs(dxi) < small3 && fabs(deta) < small3)) {
        T dd = axi0 * aet1 - axi1 * aet0;
        if (dd == T(0.0)) return GOM_ELM_BILINEAR;
        xi = T(4.0) * (aet1 * (x - x0) - aet0 * (y - y0)) / dd;
        eta = T(4.0) * (axi0 * (y - y0) - axi1 * (x - x0)) / dd;
    } else if (fabs(dxi) < small3 && fabs(deta) >= small3) {
        eta = T(4.0) * (bxy1 * (x - x0) - bxy0 * (y - y0)) / deta;
        T t1 = axi0 + eta * bxy0, t2 = axi1 + eta * bxy1;
        T dd = t1 * t1 + t2 * t2;
        if (dd == T(0.0)) return GOM_ELM_BILINEAR;
        xi = ((T(4.0) * (x - x0) - eta * aet0) * (axi0 + eta * bxy0) + (T(4.0) * (y - y0) - eta * aet1) * (axi1 + eta * bxy1)) / dd;
    } else if (fabs(dxi) >= small3 && fabs(deta) < small3) {
        xi = T(4.0) * (bxy1 * (x - x0) - bxy0 * (y - y0)) / dxi;
        T t1 = aet0 + xi * bxy0, t2 = aet1 + xi * bxy1;
        T dd = t1 * t1 + t2 * t2;
        if (dd == T(0.0)) return GOM_ELM_BILINEAR;
        eta = ((T(4.0) * (x - x0) - xi * axi0) * (aet0 + xi * bxy0) + (T(4.0) * (y - y0) - xi * axi1) * (aet1 + xi * bxy1)) / dd;
    } else {
        T beta = aet1 * axi0 - aet0 * axi1 - 4 * (bxy1 * (x - x0) - bxy0 * (y - y0));
        T gamma = T(4.0) * (aet0 * (y - y0) - aet1 * (x - x0));
        T delta = beta * beta - 4 * gamma * dxi;
        if (delta == T(0.0)) {
            xi = -beta / 2 / dxi;
            eta = (T(4.0) * (bxy1 * (x - x0) - bxy0 * (y - y0)) - xi * dxi) / deta;
        } else if (delta > 0) {
            T sq = sqrt(delta);
            T rx[2] = {(-beta + sq) / 2 / dxi, (-beta - sq) / 2 / dxi};
            int icount = 0;
            for (int i = 0; i < 2; ++i) {
                T re = (4 * (bxy1 * (x - x0) - bxy0 * (y - y0)) - rx[i] * dxi) / deta;
                if (fabs(rx[i]) <= b11 && fabs(re) <= b11) {
                    xi = rx[i];
                    eta = re;
                    icount = icount + 1;
                }
            }
            if (!(icount == 2 && fabs(rx[0] - rx[1]) < small_06) && icount != 1) return GOM_ELM_BILINEAR;
        } else {
            return GOM_ELM_BILINEAR;
        }
    }
    if (fabs(xi) > b11 || fabs(eta) > b11) return GOM_ELM_BILINEAR;
    xi = fmin(T(1.0), fmax(xi, -T(1.0)));
    eta = fmin(T(1.0), fmax(eta, -T(1.0)));
    shapef[0] = (1 - xi) * (1 - eta) / 4;
    shapef[1] = (1 + xi) * (1 - eta) / 4;
    shapef[2] = (1 + xi) * (1 + eta) / 4;
    shapef[3] = (1 - xi) * (1 + eta) / 4;
    return 0;
}

template <typename R> __device__ __forceinline__ int top_el(const StateT<R> &s, int e) { return e == 0 ? 0 : s.top_cell[e - 1]; }

__device__ __forceinline__ double area_sum(const Geom &g, int nel, double x, double y) {
    int tq = g.tri_or_quad[nel - 1];
    double a = 0.0;
    for (int l = 1; l <= tq; ++l) {
        int n1 = g.cell_node(l, nel), n2 = g.cell_node(start_end_node(tq, l, 1), nel);
        a = a + fabs(calculate_area(g.x_node[n1 - 1], g.x_node[n2 - 1], x, g.y_node[n1 - 1], g.y_node[n2 - 1], y));
    }
    return a;
}

// ---------------------------------------------------------------- point-in-element tests
// The reference's test (search_straight_line.f90, ELM_backtrace_v1.f90:151-164): the sum of the
// areas of the triangles (point, edge) against the element area, relative tolerance small_06.
// For a convex counter-clockwise element with edge cross products c_l = e_l x (p - a_l) the
// excess sum - area equals the sum of |c_l| over the negative c_l (exactly, in exact arithmetic).
// The mixed path evaluates the c_l in FP32 on element-local coordinates with a bound on their
// error and decides from the bound when the margin allows; otherwise it evaluates the reference's
// FP64 expression.  Either way the decision is the FP64 reference's.
__device__ __forceinline__ bool in_elem64(const Geom &g, int nel, double x, double y) {
    double ar = g.area[nel - 1];
    return quotient_lt(fabs(area_sum(g, nel, x, y) - ar), ar, F(1.e-6f));
}
__device__ __forceinline__ bool out_elem64(const Geom &g, int nel, double x, double y) {
    double ar = g.area[nel - 1];
    return quotient_gt(fabs(area_sum(g, nel, x, y) - ar), ar, F(1.e-6f));
}

// element nodes as FP32 offsets from the element centre
struct LocalElem {
    int tq;
    double xc, yc;
    float x[4], y[4];
    float ar;
};

// FP32 node offsets of every element, formed once per context
__global__ void k_elem_local(Geom g, float *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i > g.NC) return;
    int tq = g.tri_or_quad[i - 1];
    double xc = g.x_cell[i - 1], yc = g.y_cell[i - 1];
    float *o = out + (long)(i - 1) * 8;
    for (int l = 0; l < 4; ++l) {
        o[l] = 0.0f;
        o[4 + l] = 0.0f;
        if (l < tq) {
            int n = g.cell_node(l + 1, i);
            o[l] = (float)(g.x_node[n - 1] - xc);
            o[4 + l] = (float)(g.y_node[n - 1] - yc);
        }
    }
}

cudaError_t launch_elem_local(const Geom &g, float *out, cudaStream_t stream) {
    k_elem_local<<<blocks_for(g.NC, 256), 256, 0, stream>>>(g, out);
    return cudaGetLastError();
}

__device__ __forceinline__ void load_local(const Geom &g, int nel, LocalElem &e) {
    e.tq = g.tri_or_quad[nel - 1];
    e.xc = g.x_cell[nel - 1];
    e.yc = g.y_cell[nel - 1];
    e.ar = (float)g.area[nel - 1];
    const float4 *v = reinterpret_cast<const float4 *>(g.elem_local + (long)(nel - 1) * 8);
    const float4 xs = v[0], ys = v[1];
    e.x[0] = xs.x;
    e.x[1] = xs.y;
    e.x[2] = xs.z;
    e.x[3] = xs.w;
    e.y[0] = ys.x;
    e.y[1] = ys.y;
    e.y[2] = ys.z;
    e.y[3] = ys.w;
}

// 1: inside by the reference's test, 0: outside, -1: not decidable in FP32.  near: an edge line
// passes within the FP32 error bound of the point.
__device__ __forceinline__ int classify_f32(const LocalElem &e, float px, float py, bool &near) {
    const float u = 5.97e-8f;   // 2^-24
    float lo = 0.0f, hi = 0.0f;
    near = false;
    float twice_area = 0.0f;   // counter-clockwise elements only (as cell.inp requires)
    for (int l = 0; l < e.tq; ++l) {
        int m = l + 1 == e.tq ? 0 : l + 1;
        twice_area += e.x[l] * e.y[m] - e.x[m] * e.y[l];
    }
    if (!(twice_area > 0.0f)) {
        near = true;
        return -1;
    }
    for (int l = 0; l < e.tq; ++l) {
        int m = l + 1 == e.tq ? 0 : l + 1;
        float ex = e.x[m] - e.x[l], ey = e.y[m] - e.y[l];
        float dx = px - e.x[l], dy = py - e.y[l];
        float c = ex * dy - ey * dx;
        // inputs rounded from FP64 differences, two subtractions, two products, one subtraction
        float mag = (fabsf(e.x[m]) + fabsf(e.x[l]) + fabsf(e.y[m]) + fabsf(e.y[l])) *
                    (fabsf(px) + fabsf(py) + fabsf(e.x[l]) + fabsf(e.y[l]));
        float bnd = 16.0f * u * mag + 1e-30f;
        if (c <= -bnd) {
            lo += -c - bnd;
            hi += -c + bnd;
        } else if (c < bnd) {
            hi += fmaxf(-c, 0.0f) + bnd;
        }
        if (fabsf(c) < 2.0f * bnd) near = true;
    }
    const float thr = (float)F(1.e-6f) * e.ar;
    if (hi < thr * (1.0f - 1e-4f)) return 1;
    if (lo > thr * (1.0f + 1e-4f)) return 0;
    return -1;
}

__device__ __forceinline__ bool in_elem_mixed(const Geom &g, int nel, double x, double y) {
    LocalElem e;
    load_local(g, nel, e);
    bool near;
    int r = classify_f32(e, (float)(x - e.xc), (float)(y - e.yc), near);
    return r >= 0 ? r == 1 : in_elem64(g, nel, x, y);
}
__device__ __forceinline__ bool out_elem_mixed(const Geom &g, int nel, double x, double y) {
    LocalElem e;
    load_local(g, nel, e);
    bool near;
    int r = classify_f32(e, (float)(x - e.xc), (float)(y - e.yc), near);
    return r >= 0 ? r == 0 : out_elem64(g, nel, x, y);
}

// search_straight_line.f90:15-399 (mode 1). Returns 0 or a GOM_ELM_* site.  start_on_edge: the
// start point is the midpoint of an edge of the start element (the first substep of a face), for
// which the reference's start test (:37-46) always passes -- its area excess is zero up to FP64
// rounding, far below the tolerance -- so it is not evaluated.  MIXED selects the FP32-filtered
// point-in-element tests (same decisions).
template <typename R, bool MIXED>
__device__ int search_straight_line(const Geom &g, const StateT<R> &s, const Params &p, int &nnel, int &jlev, double time,
                                    double x0, double y0, double z0, double &xt, double &yt, double &zt, int &nfl,
                                    bool start_on_edge) {
    const double small_06 = F(1.e-6f);
    const double MSL = p.msl;
    const int L = g.L;
    if (top_el(s, nnel) == 0 || MSL - g.h_cell[nnel - 1] > MSL + s.eta_cell[nnel - 1]) return GOM_ELM_START_DRY;
    nfl = 0;
    double trm = time;
    int nel = nnel;
    if (!start_on_edge && (MIXED ? out_elem_mixed(g, nel, x0, y0) : out_elem64(g, nel, x0, y0)))
        return GOM_ELM_START_OUTSIDE;
    if (!(MIXED ? in_elem_mixed(g, nel, xt, yt) : in_elem64(g, nel, xt, yt))) {
        const double c1 = 1.0 - 1.0e-4;
        double xcg = c1 * x0 + 1.0e-4 * g.x_cell[nel - 1];
        double ycg = c1 * y0 + 1.0e-4 * g.y_cell[nel - 1];
        double pathl = sqrt((xt - xcg) * (xt - xcg) + (yt - ycg) * (yt - ycg));
        if ((xcg == xt && ycg == yt) || pathl == 0.0) return GOM_ELM_ZERO_PATH;
        int iflag = 0, nel_j = 0;
        double xin = 0.0, yin = 0.0;
        int tq = g.tri_or_quad[nel - 1];
        for (int l = 1; l <= tq; ++l) {
            int jd1 = g.cell_node(start_end_node(tq, l, 1), nel);
            int jd2 = g.cell_node(start_end_node(tq, l, 2), nel);
            iflag = check_intersection(xcg, xt, g.x_node[jd1 - 1], g.x_node[jd2 - 1], ycg, yt, g.y_node[jd1 - 1],
                                       g.y_node[jd2 - 1], xin, yin);
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
            int tqn = g.tri_or_quad[nel - 1];
            int md1 = g.cell_node(start_end_node(tqn, nel_j, 1), nel);
            int md2 = g.cell_node(start_end_node(tqn, nel_j, 2), nel);
            double dist = sqrt((xin - xt) * (xin - xt) + (yin - yt) * (yin - yt));
            if (dist / pathl > 1.0 + 1.0e-4) return GOM_ELM_OVERSHOOT;
            zin = zt - dist / pathl * (zt - zin);
            trm = trm * dist / pathl;
            pathl = sqrt((xin - xt) * (xin - xt) + (yin - yt) * (yin - yt));
            if (pathl == 0.0 || trm == 0.0) return GOM_ELM_ZERO_REMAIN;
            int adjc = g.cell_adj(nel_j, nel);
            if (adjc == 0 || top_el(s, adjc) == 0) {
                int isd = g.cell_face(nel_j, nel);
                if (g.face_node(1, isd) + g.face_node(2, isd) != md1 + md2) return GOM_ELM_FACE_MISMATCH;
                xin = c1 * xin + 1.0e-4 * g.x_cell[nel - 1];
                yin = c1 * yin + 1.0e-4 * g.y_cell[nel - 1];
                nfl = 1;
                xt = xin;
                yt = yin;
                zt = zin;
                nnel = nel;
                break;
            }
            nel = adjc;
            if (MIXED ? in_elem_mixed(g, nel, xt, yt) : in_elem64(g, nel, xt, yt)) {
                nnel = nel;
                break;
            }
            tqn = g.tri_or_quad[nel - 1];
            bool found = false;
            for (int l = 1; l <= tqn; ++l) {
                int jd1 = g.cell_node(start_end_node(tqn, l, 1), nel);
                int jd2 = g.cell_node(start_end_node(tqn, l, 2), nel);
                if ((jd1 == md1 && jd2 == md2) || (jd2 == md1 && jd1 == md2)) continue;
                iflag = check_intersection(xcg, xt, g.x_node[jd1 - 1], g.x_node[jd2 - 1], ycg, yt, g.y_node[jd1 - 1],
                                           g.y_node[jd2 - 1], xin, yin);
                if (iflag == 1) {
                    nel_j = l;
                    found = true;
                    break;
                }
            }
            if (found) continue;
            if (iflag == 0) return GOM_ELM_NO_NEXT_EDGE;
        }
    } else {
        nnel = nel;
    }
    if (top_el(s, nnel) == 0 || MSL - g.h_cell[nnel - 1] > MSL + s.eta_cell[nnel - 1]) return GOM_ELM_END_DRY;
    zt = fmin(fmax(zt, MSL - g.h_cell[nnel - 1]), MSL + s.eta_cell[nnel - 1]);
    if (zt <= g.z_level[0] || zt > g.z_level[L]) return GOM_ELM_Z_RANGE;
    // :376-396 the level k with z_level(k) < zt <= z_level(k+1), unique for increasing levels:
    // searched from the start layer outwards instead of from the bottom (same k)
    {
        int k = min(max(jlev - 1, 0), L - 1);
        while (k < L - 1 && zt > g.z_level[k + 1]) ++k;
        while (k > 0 && zt <= g.z_level[k]) --k;
        jlev = k + 1;
    }
    jlev = min(max(jlev, g.bottom_cell[nnel - 1]), top_el(s, nnel));
    return 0;
}

// diagnostic for foot parity: (x, y) lies within 1e-12 m of an edge line of element nel, tested
// as cross^2 < (1e-12)^2 * |edge|^2 (cross = edge x (point - edge start)): no root, no division
__device__ bool near_edge_line(const Geom &g, int nel, double x, double y) {
    int tq = g.tri_or_quad[nel - 1];
    for (int l = 1; l <= tq; ++l) {
        int a = g.cell_node(l, nel), b = g.cell_node(start_end_node(tq, l, 1), nel);
        double ex = g.x_node[b - 1] - g.x_node[a - 1], ey = g.y_node[b - 1] - g.y_node[a - 1];
        double cr = ex * (y - g.y_node[a - 1]) - ey * (x - g.x_node[a - 1]);
        if (cr * cr < 1e-24 * (ex * ex + ey * ey)) return true;
    }
    return false;
}

// ELM_backtrace_v1.f90:40-200 (mode 1).  The first substep starts at the face midpoint, on an
// edge of the start element.  MIXED: the same walk (FP64 foot coordinates, the reference's
// point-in-element decisions), interpolation weights and velocities in FP32 on element-local
// coordinates.
template <typename R, bool MIXED>
__device__ int elm_backtrace(const Geom &g, const StateT<R> &s, const Params &p, int bt_step, double bt_dt, double &uu,
                             double &vv, double &ww, double x0, double y0, double z0, int &nnel, int &jlev,
                             int &near_edge) {
    const double small_06 = F(1.e-6f);
    const int L = g.L;
    for (int idt = 1; idt <= bt_step; ++idt) {
        double xt = x0 - bt_dt * uu;
        double yt = y0 - bt_dt * vv;
        double zt = z0 - bt_dt * ww;
        int nfl = 0;
        int e = search_straight_line<R, MIXED>(g, s, p, nnel, jlev, bt_dt, x0, y0, z0, xt, yt, zt, nfl, idt == 1);
        if (e) return e;
        int tq = g.tri_or_quad[nnel - 1];
        double zup = (jlev == s.top_cell[nnel - 1]) ? p.msl + s.eta_cell[nnel - 1] : g.z_level[jlev];
        if (zt > zup) return GOM_ELM_Z_ABOVE;
        if constexpr (MIXED) {
            const float zrat = (float)(zup - zt) / (float)s.dz_cell[ix(jlev, nnel, L)];
            LocalElem el;
            load_local(g, nnel, el);
            const float px = (float)(xt - el.xc), py = (float)(yt - el.yc);
            bool near;
            const int cls = classify_f32(el, px, py, near);
            float sta[4];
            if (tq == 3) {
                const float ar = el.ar;
                sta[0] = calculate_area_t(px, el.x[1], el.x[2], py, el.y[1], el.y[2]) / ar;
                sta[1] = calculate_area_t(el.x[0], px, el.x[2], el.y[0], py, el.y[2]) / ar;
                sta[2] = calculate_area_t(el.x[0], el.x[1], px, el.y[0], el.y[1], py) / ar;
                sta[0] = fmaxf(0.0f, fminf(1.0f, sta[0]));
                sta[1] = fmaxf(0.0f, fminf(1.0f, sta[1]));
                if (sta[0] + sta[1] > 1.0f) {
                    sta[2] = 0.0f;
                    sta[1] = 1.0f - sta[0];
                } else {
                    sta[2] = 1.0f - sta[0] - sta[1];
                }
            } else {
                if (cls >= 0 ? cls == 0 : out_elem64(g, nnel, xt, yt)) return GOM_ELM_QUAD_OUTSIDE;
                int b = bilinear_interpolation<float>(el.x[0], el.x[1], el.x[2], el.x[3], el.y[0], el.y[1], el.y[2],
                                                      el.y[3], px, py, sta);
                if (b) return b;
            }
            float fu = 0.0f, fv = 0.0f, fw = 0.0f;
            for (int l = 1; l <= tq; ++l) {
                int nd = g.cell_node(l, nnel);
                long i1 = ix0(jlev - 1, nd, L), i2 = ix0(jlev, nd, L);
                float w = sta[l - 1];
                fu = fu + ((float)s.u_node[i2] * (1.0f - zrat) + (float)s.u_node[i1] * zrat) * w;
                fv = fv + ((float)s.v_node[i2] * (1.0f - zrat) + (float)s.v_node[i1] * zrat) * w;
                fw = fw + ((float)s.w_node[i2] * (1.0f - zrat) + (float)s.w_node[i1] * zrat) * w;
            }
            uu = fu;
            vv = fv;
            ww = fw;
            if (near && near_edge_line(g, nnel, xt, yt)) near_edge = 1;
        } else {
            double zrat = (zup - zt) / s.dz_cell[ix(jlev, nnel, L)];
            double vxn[4], vyn[4], vzn[4], sta[4];
            for (int l = 1; l <= tq; ++l) {
                int nd = g.cell_node(l, nnel);
                long i1 = ix0(jlev - 1, nd, L), i2 = ix0(jlev, nd, L);
                vxn[l - 1] = s.u_node[i2] * (1 - zrat) + s.u_node[i1] * zrat;
                vyn[l - 1] = s.v_node[i2] * (1 - zrat) + s.v_node[i1] * zrat;
                vzn[l - 1] = s.w_node[i2] * (1 - zrat) + s.w_node[i1] * zrat;
            }
            int n1 = g.cell_node(1, nnel), n2 = g.cell_node(2, nnel), n3 = g.cell_node(3, nnel);
            double X1 = g.x_node[n1 - 1], X2 = g.x_node[n2 - 1], X3 = g.x_node[n3 - 1];
            double Y1 = g.y_node[n1 - 1], Y2 = g.y_node[n2 - 1], Y3 = g.y_node[n3 - 1];
            double ar = g.area[nnel - 1];
            if (tq == 3) {
                sta[0] = calculate_area(xt, X2, X3, yt, Y2, Y3) / ar;
                sta[1] = calculate_area(X1, xt, X3, Y1, yt, Y3) / ar;
                sta[2] = calculate_area(X1, X2, xt, Y1, Y2, yt) / ar;
                sta[0] = fmax(0.0, fmin(1.0, sta[0]));
                sta[1] = fmax(0.0, fmin(1.0, sta[1]));
                if (sta[0] + sta[1] > 1) {
                    sta[2] = 0;
                    sta[1] = 1.0 - sta[0];
                } else {
                    sta[2] = 1.0 - sta[0] - sta[1];
                }
            } else {
                int n4 = g.cell_node(4, nnel);
                double X4 = g.x_node[n4 - 1], Y4 = g.y_node[n4 - 1];
                double aa1 = calculate_area(X1, X2, xt, Y1, Y2, yt);
                double aa2 = calculate_area(X2, X3, xt, Y2, Y3, yt);
                double aa3 = calculate_area(X3, X4, xt, Y3, Y4, yt);
                double aa4 = calculate_area(X4, X1, xt, Y4, Y1, yt);
                double aa = fabs(aa1) + fabs(aa2) + fabs(aa3) + fabs(aa4);
                if (quotient_gt(fabs(aa - ar), ar, small_06)) return GOM_ELM_QUAD_OUTSIDE;
                int b = bilinear_interpolation<double>(X1, X2, X3, X4, Y1, Y2, Y3, Y4, xt, yt, sta);
                if (b) return b;
            }
            uu = 0.0;
            vv = 0.0;
            ww = 0.0;
            for (int j = 0; j < tq; ++j) {
                uu = uu + vxn[j] * sta[j];
                vv = vv + vyn[j] * sta[j];
                ww = ww + vzn[j] * sta[j];
            }
            if (near_edge_line(g, nnel, xt, yt)) near_edge = 1;
        }
        if (nfl == 1) break;
        x0 = xt;
        y0 = yt;
        z0 = zt;
    }
    return 0;
}

// solve_nonlinear_advection.f90:52-87.  The reference evaluates, for every node, layer and
// adjacent cell, INT(dev/0.1) of the two cell edges meeting at the node; dev depends only on the
// edge (it is symmetric in its two nodes), so k_elm_edge_dev evaluates it once per edge (= face)
// and layer, and k_elm_substeps combines the edges of each node.  INT(dev/0.1) and
// INT(2*w*dt/delta_z_min) are 0 whenever the operands lie more than 1e-9 below the thresholds;
// that usual case is decided from squared quantities without square roots or divisions, every
// other case is computed exactly as the reference does.
template <typename R> __global__ void k_elm_edge_dev(Geom g, StateT<R> s, Params p, int *idev) {
    unsigned t = flat_tid();
    const int L = g.L;
    if (t >= (unsigned)g.NF * L) return;
    int j, k;
    split_index(t, L, j, k);
    j += 1;
    k += 1;
    int n1 = g.face_node(1, j), n2 = g.face_node(2, j);
    if constexpr (sizeof(R) == sizeof(float)) {
        // mixed path: the same count in FP32 (the node velocities are FP32 already)
        const float dt = (float)p.dt, c01 = 0.1f;
        const float dx = (float)(g.x_node[n1 - 1] - g.x_node[n2 - 1]), dy = (float)(g.y_node[n1 - 1] - g.y_node[n2 - 1]);
        const float rl2 = dx * dx + dy * dy;
        float du = (s.u_node[ix0(k, n1, L)] + s.u_node[ix0(k - 1, n1, L)]) * 0.5f -
                   (s.u_node[ix0(k, n2, L)] + s.u_node[ix0(k - 1, n2, L)]) * 0.5f;
        float dv = (s.v_node[ix0(k, n1, L)] + s.v_node[ix0(k - 1, n1, L)]) * 0.5f -
                   (s.v_node[ix0(k, n2, L)] + s.v_node[ix0(k - 1, n2, L)]) * 0.5f;
        float sq = du * du + dv * dv;
        int id = 0;
        if (!(sq < rl2 * (c01 * c01 / (dt * dt)) * (1.0f - 1e-5f))) id = (int)(sqrtf(sq) / sqrtf(rl2) * dt / c01);
        idev[t] = id;
        return;
    }
    const double dt = p.dt;
    const double c01 = F(1.e-1f);
    const double kthr = c01 * c01 / (dt * dt) * (1.0 - 1e-9);
    double dx = g.x_node[n1 - 1] - g.x_node[n2 - 1], dy = g.y_node[n1 - 1] - g.y_node[n2 - 1];
    double rl2 = dx * dx + dy * dy;
    double u1 = (s.u_node[ix0(k, n1, L)] + s.u_node[ix0(k - 1, n1, L)]) * 0.5;
    double v1 = (s.v_node[ix0(k, n1, L)] + s.v_node[ix0(k - 1, n1, L)]) * 0.5;
    double u2 = (s.u_node[ix0(k, n2, L)] + s.u_node[ix0(k - 1, n2, L)]) * 0.5;
    double v2 = (s.v_node[ix0(k, n2, L)] + s.v_node[ix0(k - 1, n2, L)]) * 0.5;
    double du = u1 - u2, dv = v1 - v2;
    double sq = du * du + dv * dv;
    int id = 0;
    if (!(sq < rl2 * kthr)) {
        double dev = sqrt(sq) / sqrt(rl2) * dt;
        id = (int)(dev / c01);
    }
    idev[t] = id;
}

__device__ __forceinline__ int wrap_edge(int l, int tq) { return l <= 0 ? l + tq : l; }

template <typename R> __global__ void k_elm_substeps(Geom g, StateT<R> s, Params p, const int *idev) {
    unsigned t = flat_tid();
    const int L = g.L;
    if (t >= (unsigned)g.NN * L) return;
    int i, k;
    split_index(t, L, i, k);
    i += 1;
    k += 1;
    int nadj = g.adj_cells_at_node[i - 1];
    int iw;
    if constexpr (sizeof(R) == sizeof(float)) {
        // mixed path: the same count in FP32
        float aw = 2.0f * ((s.w_node[ix0(k, i, L)] + s.w_node[ix0(k - 1, i, L)]) * 0.5f) * (float)p.dt;
        float dzm = (float)p.delta_z_min;
        iw = fabsf(aw) < dzm * (1.0f - 1e-5f) ? 0 : (int)(aw / dzm);
    } else {
        const double dt = p.dt;
        double wi = (s.w_node[ix0(k, i, L)] + s.w_node[ix0(k - 1, i, L)]) * 0.5;
        double aw = 2 * wi * dt;
        iw = fabs(aw) < p.delta_z_min * (1.0 - 1e-9) ? 0 : (int)(aw / p.delta_z_min);
    }
    using Sum = typename std::conditional<sizeof(R) == sizeof(float), float, double>::type;
    Sum summ = Sum(0);
    for (int j = 1; j <= nadj; ++j) {
        int ie = g.node_cell(j, i), id = g.node_count(j, i);
        int tq = g.tri_or_quad[ie - 1];
        // edges (id, id+1) and (id-1, id) of cell ie: local faces id-1 and id-2
        int fa = g.cell_face(wrap_edge(id - 1, tq), ie);
        int fb = g.cell_face(wrap_edge(id - 2, tq), ie);
        int imax = max(idev[ix(k, fa, L)], idev[ix(k, fb, L)]);
        int idelta = max(imax, iw);
        if (idelta != 0) summ = summ + (Sum)idelta / (Sum)nadj;   // 0/nadj adds exactly 0
    }
    s.num_sub_elm[ix(k, i, L)] = max(p.elm_min_iter, min(p.elm_max_iter, (int)summ));
}

// solve_nonlinear_advection.f90:94-201: one thread per face walks the face's wet layers (a warp's
// FP64 work is spread over 32 faces instead of idling on dry layers)
template <typename R>
__device__ void elm_face_layer(const Geom &g, const StateT<R> &s, const Params &p, gom_status *st, int j, int k, int ie0,
                               int n1, int n2, double ct, double sn) {
    const int L = g.L;
    long o = ix(k, j, L);
    double unf = s.un_face[o], vnf = s.vn_face[o];
    int nnel = ie0, jlev = k;
    double x0 = g.x_face[j - 1], y0 = g.y_face[j - 1], z0;
    if (k == s.top_cell[nnel - 1]) z0 = p.msl + s.eta_cell[nnel - 1] - s.dz_cell[ix(k, nnel, L)] * 0.5;
    else z0 = g.z_level[k] - s.dz_cell[ix(k, nnel, L)] * 0.5;
    double uu = unf * ct - vnf * sn;
    double vv = unf * sn + vnf * ct;
    double wdown = (s.w_node[ix0(k - 1, n1, L)] + s.w_node[ix0(k - 1, n2, L)]) * 0.5;
    double wup = (s.w_node[ix0(k, n1, L)] + s.w_node[ix0(k, n2, L)]) * 0.5;
    double ww = (wdown + wup) * 0.5;
    double vmag = sqrt(uu * uu + vv * vv + ww * ww);
    if (vmag <= F(1.e-4f)) {
        s.un_elm[o] = s.un_face[o];
        s.vn_elm[o] = s.vn_face[o];
        return;
    }
    int bt_step = (int)((double)(s.num_sub_elm[ix(k, n1, L)] + s.num_sub_elm[ix(k, n2, L)]) * 0.5);
    double bt_dt = p.dt / bt_step;
    int near = 0;
    int e = elm_backtrace<R, sizeof(R) == sizeof(float)>(g, s, p, bt_step, bt_dt, uu, vv, ww, x0, y0, z0, nnel, jlev,
                                                          near);
    if (e) {
        record_error(st, GOM_E_ELM, e, j, k, 0.0);
        return;
    }
    s.elm_foot[o] = nnel;
    s.elm_near_edge[o] = near;
    s.un_elm[o] = (R)(uu * ct + vv * sn);
    s.vn_elm[o] = (R)(-uu * sn + vv * ct);
}

template <typename R, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_elm_faces(Geom g, StateT<R> s, Params p, gom_status *st) {
    unsigned tid = flat_tid();
    if (tid >= (unsigned)g.NF) return;
    int j = g.face_order[tid];
    const int L = g.L;
    int b = g.bottom_face[j - 1], tf = s.top_face[j - 1];
    for (int k = 1; k <= L; ++k) {
        long o = ix(k, j, L);
        s.elm_foot[o] = 0;
        s.elm_near_edge[o] = 0;
        if (k < b || k > tf) {
            s.un_elm[o] = R(0);
            s.vn_elm[o] = R(0);
        }
    }
    if (tf < b) return;
    int n1 = g.face_node(1, j), n2 = g.face_node(2, j);
    bool shallow = fabs(fmax(g.h_node[n1 - 1], g.h_node[n2 - 1])) < p.adv_onoff_depth;
    int a1 = g.face_cell(1, j), a2 = g.face_cell(2, j);
    int ie0 = 0;
    if (s.top_cell[a1 - 1] != 0) ie0 = a1;
    else if (a2 != 0 && s.top_cell[a2 - 1] != 0) ie0 = a2;
    if (shallow || ie0 == 0) {
        for (int k = b; k <= tf; ++k) {
            long o = ix(k, j, L);
            s.un_elm[o] = s.un_face[o];
            s.vn_elm[o] = s.vn_face[o];
        }
        return;
    }
    double ct = g.cos_theta[j - 1], sn = g.sin_theta[j - 1];
    for (int k = b; k <= tf; ++k) elm_face_layer(g, s, p, st, j, k, ie0, n1, n2, ct, sn);
}

// The same walk with one thread per wet face-layer of a walked face, taken from a compact list
// (gom_scan.cuh): the layers of one face sit on neighbouring lanes, walk nearly the same path and
// read the same element and node data, and no lane idles on a dry layer.  Warps take 4x32 entries
// at a time from a work queue, so a warp that drew long walks does not hold up the others.
struct FaceWalkRange {
    const int *bottom_face, *top_face, *top_cell, *face_cell, *face_node;
    const double *h_node;
    double adv_onoff_depth;
    __device__ int2 operator()(int i) const {
        const int b = bottom_face[i], tf = top_face[i];
        const int n1 = face_node[2 * i], n2 = face_node[2 * i + 1];
        const bool shallow = fabs(fmax(h_node[n1 - 1], h_node[n2 - 1])) < adv_onoff_depth;
        const int a1 = face_cell[2 * i], a2 = face_cell[2 * i + 1];
        const bool start = top_cell[a1 - 1] != 0 || (a2 != 0 && top_cell[a2 - 1] != 0);
        return (tf >= b && !shallow && start) ? make_int2(b, tf) : make_int2(1, 0);
    }
};

// every face-layer's result before the walk: no foot, the face's own velocity inside the wet
// range (what a walk that is skipped leaves), 0 outside it
template <typename R> __global__ void k_elm_init(Geom g, StateT<R> s) {
    unsigned t = flat_tid();
    if (t >= (unsigned)g.NF * g.L) return;
    int j, k;
    split_index(t, g.L, j, k);
    s.elm_foot[t] = 0;
    s.elm_near_edge[t] = 0;
    const bool wet = k + 1 >= g.bottom_face[j] && k + 1 <= s.top_face[j];
    s.un_elm[t] = wet ? s.un_face[t] : R(0);
    s.vn_elm[t] = wet ? s.vn_face[t] : R(0);
}

template <typename R, int BS>
__global__ void __launch_bounds__(BS) k_elm_list(Geom g, StateT<R> s, Params p, const int *list, int *count,
                                                 gom_status *st) {
    const int n = count[0];
    const int lane = threadIdx.x & 31;
    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&count[1], 128);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        for (int r = 0; r < 4; ++r) {
            const int e = base + 32 * r + lane;
            if (e >= n) break;
            const int code = list[e];
            const int j = list_entity(code), k = list_layer(code);
            const int n1 = g.face_node(1, j), n2 = g.face_node(2, j);
            const int a1 = g.face_cell(1, j);
            const int ie0 = s.top_cell[a1 - 1] != 0 ? a1 : g.face_cell(2, j);
            elm_face_layer(g, s, p, st, j, k, ie0, n1, n2, g.cos_theta[j - 1], g.sin_theta[j - 1]);
        }
    }
}

template <typename R, int BS> cudaError_t launch_elm_list(const LaunchT<R> &x) {
    const Geom &g = x.g;
    k_elm_init<<<blocks_for((long)g.NF * g.L, 256), 256, 0, x.stream>>>(g, x.s);
    FaceWalkRange r{g.bottom_face, x.s.top_face, x.s.top_cell, g.adj_cellnum_at_face, g.nodenum_at_face, g.h_node,
                    x.p.adv_onoff_depth};
    cudaError_t e = build_layer_list(g.NF, r, x.w.fl_off, x.w.fl_bsum, x.w.fl_list, x.w.fl_count, x.stream);
    if (e != cudaSuccess) return e;
    k_elm_list<R, BS><<<x.num_sms * (2048 / BS), BS, 0, x.stream>>>(g, x.s, x.p, x.w.fl_list, x.w.fl_count,
                                                                      x.status);
    return cudaGetLastError();
}

template <typename R> __global__ void k_copy_elm(Geom g, StateT<R> s) {
    unsigned t = flat_tid();
    if (t >= (unsigned)g.NF * g.L) return;
    s.un_elm[t] = s.un_face[t];
    s.vn_elm[t] = s.vn_face[t];
    s.elm_foot[t] = 0;
    s.elm_near_edge[t] = 0;
}

template <typename R> cudaError_t launch_elm_walk(const LaunchT<R> &x) {
    // variants: threads per block and minimum resident blocks per SM (register budget)
    const int v = x.w.fl_list ? x.tune[TUNE_ELM] : 0;
    switch (v) {
    case 5: return launch_elm_list<R, 64>(x);
    case 6: return launch_elm_list<R, 128>(x);
    case 1: k_elm_faces<R, 32, 1><<<blocks_for(x.g.NF, 32), 32, 0, x.stream>>>(x.g, x.s, x.p, x.status); break;
    case 2: k_elm_faces<R, 128, 1><<<blocks_for(x.g.NF, 128), 128, 0, x.stream>>>(x.g, x.s, x.p, x.status); break;
    case 3: k_elm_faces<R, 64, 12><<<blocks_for(x.g.NF, 64), 64, 0, x.stream>>>(x.g, x.s, x.p, x.status); break;
    case 4: k_elm_faces<R, 64, 16><<<blocks_for(x.g.NF, 64), 64, 0, x.stream>>>(x.g, x.s, x.p, x.status); break;
    default: k_elm_faces<R, 64, 1><<<blocks_for(x.g.NF, 64), 64, 0, x.stream>>>(x.g, x.s, x.p, x.status); break;
    }
    return cudaGetLastError();
}

template <typename R> cudaError_t launch_elm_walk_only(const LaunchT<R> &x) { return launch_elm_walk(x); }

template <typename R> cudaError_t launch_advection(const LaunchT<R> &x) {
    long nfl = (long)x.g.NF * x.g.L;
    if (x.p.advection_flag == 0) {
        k_copy_elm<<<blocks_for(nfl, 256), 256, 0, x.stream>>>(x.g, x.s);
        return cudaGetLastError();
    }
    if (x.p.elm_backtrace_flag == 1) {
        k_elm_edge_dev<<<blocks_for(nfl, 256), 256, 0, x.stream>>>(x.g, x.s, x.p, x.w.idev);
        long nnl = (long)x.g.NN * x.g.L;
        k_elm_substeps<<<blocks_for(nnl, 256), 256, 0, x.stream>>>(x.g, x.s, x.p, x.w.idev);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_elm_walk(x);
}

// ============================================================================================
// solve_momentum_equation.f90:15-656, one thread per face column.
//
// rtemp0 of the reference carries over between faces: on a boundary face whose nodes are not both
// wet, the air-pressure term at :503-505 reuses the last rtemp0 assigned for an earlier wet face
// (serial order).  prev_rtemp0() restates that by walking back to the nearest such face.
template <typename R>
__device__ double face_final_rtemp0(const Geom &g, const StateT<R> &s, const Forcing &f, const Params &p, int j,
                                    bool &known) {
    known = true;
    int a2 = g.face_cell(2, j);
    if (a2 != 0) {
        double t1 = 0.0, t2 = 0.0;
        int ie = g.face_cell(1, j);
        int tq = g.tri_or_quad[ie - 1];
        for (int ll = 1; ll <= tq; ++ll) t1 = t1 + f.air_p[g.cell_node(ll, ie) - 1] / tq;
        tq = g.tri_or_quad[a2 - 1];
        for (int ll = 1; ll <= tq; ++ll) t2 = t2 + f.air_p[g.cell_node(ll, a2) - 1] / tq;
        return -p.dt / p.rho_o * (t2 - t1) / g.delta_j[j - 1];
    }
    int n1 = g.face_node(1, j), n2 = g.face_node(2, j);
    if (s.wetdry_node[n1 - 1] == 0 && s.wetdry_node[n2 - 1] == 0)
        return p.gravity * p.dt / g.face_length[j - 1] * (1.0 - p.theta) * (s.eta_node[n2 - 1] - s.eta_node[n1 - 1]);
    known = false;
    return 0.0;
}

template <typename R>
__device__ double prev_rtemp0(const Geom &g, const StateT<R> &s, const Forcing &f, const Params &p, int j) {
    int first = 1;   // first face of j's run: the walk never leaves the run (each starts at 0)
    if (g.NR > 1) {
        int lo = 0, hi = g.NR;
        while (hi - lo > 1) {
            int mid = (lo + hi) >> 1;
            if (g.run_face_start[mid] <= j - 1) lo = mid;
            else hi = mid;
        }
        first = g.run_face_start[lo] + 1;
    }
    for (int jj = j - 1; jj >= first; --jj) {
        if (s.top_face[jj - 1] == 0) continue;
        bool known;
        double v = face_final_rtemp0(g, s, f, p, jj, known);
        if (known) return v;
    }
    return 0.0;
}

// Per-face terms (elevation gradients, air pressure, geometry) are formed in FP64 once per face
// and rounded to R; the layer loop, the Smagorinsky diffusion, the baroclinic integral and the
// tridiagonal solve run in R.  With R = double every expression is the reference's.
template <typename R>
__global__ void __launch_bounds__(256) k_momentum(Geom g, StateT<R> s, Forcing f, Params p, gom_status *st) {
    unsigned tid = flat_tid();
    if (tid >= (unsigned)g.NF) return;
    int j = g.face_order[tid];
    const int L = g.L;
    int tj = s.top_face[j - 1];
    if (tj == 0) return;
    const double dt = p.dt, gravity = p.gravity, theta = p.theta;
    const R dtR = (R)dt;
    int bj = g.bottom_face[j - 1];
    int nvl = tj - bj + 1;
    int node1 = g.face_node(1, j), node2 = g.face_node(2, j);
    int a1 = g.face_cell(1, j), a2 = g.face_cell(2, j);
    int btype = g.boundary_type_of_face[j - 1];
    const double dj = g.delta_j[j - 1], fl = g.face_length[j - 1];
    const double ct = g.cos_theta[j - 1], sn = g.sin_theta[j - 1], ct2 = g.cos_theta2[j - 1], sn2 = g.sin_theta2[j - 1];
    const R ctR = (R)ct, snR = (R)sn, ct2R = (R)ct2, sn2R = (R)sn2;
    const R cordt = (R)(g.coriolis_factor[j - 1] * dt);
    R a[GOM_MAXL], bd[GOM_MAXL], cu[GOM_MAXL], gam[GOM_MAXL];
    R rhs[GOM_MAXL][3];
    // :120-169
    for (int k = bj + 1; k <= tj - 1; ++k) {
        int kk = tj - k + 1;
        a[kk - 1] = -dtR * s.av[ix0(k, j, L)] / s.dzhalf_face[ix0(k, j, L)];
        cu[kk - 1] = -dtR * s.av[ix0(k - 1, j, L)] / s.dzhalf_face[ix0(k - 1, j, L)];
        bd[kk - 1] = -a[kk - 1] + s.dz_face[ix(k, j, L)] - cu[kk - 1];
    }
    if (tj == bj) {
        bd[0] = s.dz_face[ix(tj, j, L)] + s.gamma_b[j - 1] * dtR;
    } else {
        cu[0] = -dtR * s.av[ix0(tj - 1, j, L)] / s.dzhalf_face[ix0(tj - 1, j, L)];
        bd[0] = (R)f.gamma_t[j - 1] * dtR + s.dz_face[ix(tj, j, L)] - cu[0];
        a[nvl - 1] = -dtR * s.av[ix0(bj, j, L)] / s.dzhalf_face[ix0(bj, j, L)];
        bd[nvl - 1] = -a[nvl - 1] + s.dz_face[ix(bj, j, L)] + s.gamma_b[j - 1] * dtR;
    }
    bool wet_nodes = s.wetdry_node[node1 - 1] == 0 && s.wetdry_node[node2 - 1] == 0;
    double eta_n1 = s.eta_node[node1 - 1], eta_n2 = s.eta_node[node2 - 1];
    const R c069 = (R)F(0.69f);
    int ibnd = g.isflowside3[j - 1];
    double eta1 = s.eta_cell[a1 - 1];
    double eta2 = a2 != 0 ? s.eta_cell[a2 - 1] : 0.0;
    int ba1 = g.bottom_cell[a1 - 1], ta1 = s.top_cell[a1 - 1];
    int ba2 = a2 != 0 ? g.bottom_cell[a2 - 1] : 0, ta2 = a2 != 0 ? s.top_cell[a2 - 1] : 0;
    int bn1 = g.bottom_node[node1 - 1], tn1 = s.top_node[node1 - 1];
    int bn2 = g.bottom_node[node2 - 1], tn2 = s.top_node[node2 - 1];
    R bt1, along, air1, air2, bc_dj, bc_fl;
    if constexpr (sizeof(R) == sizeof(float)) {
        // Mixed path: the same terms from FP64 differences of elevations and pressures, the
        // divisions and products in FP32 (no FP64 division per face)
        const float gdt = (float)(gravity * dt), om = (float)(1.0 - theta), dtr = (float)(dt / p.rho_o);
        const float inv_dj = 1.0f / (float)dj, inv_fl = 1.0f / (float)fl;
        float bt_rtemp1 = 0.0f, bt_rtemp2 = 0.0f;
        if (btype == 0) {
            float rtemp0 = gdt * inv_dj * om * (float)(eta2 - eta1);
            bt_rtemp1 = rtemp0 * ct2R;
            bt_rtemp2 = rtemp0 * sn2R;
        } else if (btype > 0) {
            int ie = g.ob_element_flag[a1 - 1];
            bt_rtemp1 = gdt * inv_dj * om * (float)(f.eta_at_ob_old[ie - 1] - eta1);
        }
        const float along0 = wet_nodes ? gdt * inv_fl * om * (float)(eta_n2 - eta_n1) : 0.0f;
        const double pref = f.air_p[node1 - 1];
        float rt0_air;
        if (a2 != 0) {
            // mean air pressure of each adjacent cell, relative to a node value
            float m1 = 0.0f, m2 = 0.0f;
            int tqa = g.tri_or_quad[a1 - 1], tqb = g.tri_or_quad[a2 - 1];
            for (int ll = 1; ll <= tqa; ++ll) m1 += (float)(f.air_p[g.cell_node(ll, a1) - 1] - pref);
            for (int ll = 1; ll <= tqb; ++ll) m2 += (float)(f.air_p[g.cell_node(ll, a2) - 1] - pref);
            rt0_air = -dtr * (m2 / (float)tqb - m1 / (float)tqa) * inv_dj;
        } else if (wet_nodes) {
            rt0_air = along0;
        } else {
            rt0_air = (float)prev_rtemp0(g, s, f, p, j);
        }
        const float rtemp3_air = -dtr * (float)(f.air_p[node2 - 1] - pref) * inv_fl;
        bt1 = bt_rtemp1;
        along = (btype == 0) ? (along0 + bt_rtemp2) : along0;
        air1 = rt0_air * ct2R;
        air2 = rtemp3_air + rt0_air * sn2R;
        bc_dj = -(gdt / (float)p.rho_o) * inv_dj;
        bc_fl = -(gdt / (float)p.rho_o) * inv_fl;
    } else {
        // rtemp0 reaching the air-pressure term of a boundary face
        double rt0_air;
        if (a2 != 0) {
            bool known;
            rt0_air = face_final_rtemp0(g, s, f, p, j, known);
        } else if (wet_nodes) {
            rt0_air = gravity * dt / fl * (1.0 - theta) * (eta_n2 - eta_n1);
        } else {
            rt0_air = prev_rtemp0(g, s, f, p, j);
        }
        double rtemp3_air = -dt / p.rho_o * ((f.air_p[node2 - 1] - f.air_p[node1 - 1]) / fl);
        // Terms the reference re-evaluates in every layer although their operands do not depend
        // on the layer; evaluated once per face with the same expression, hence the same value.
        double bt_rtemp1 = 0.0, bt_rtemp2 = 0.0;    // (1-theta) barotropic gradient across the face
        if (btype == 0) {
            double rtemp0 = gravity * dt / dj * (1.0 - theta) * (eta2 - eta1);
            bt_rtemp1 = rtemp0 * ct2;
            bt_rtemp2 = rtemp0 * sn2;
        } else if (btype > 0) {
            int ie = g.ob_element_flag[a1 - 1];
            bt_rtemp1 = gravity * dt / dj * (1.0 - theta) * (f.eta_at_ob_old[ie - 1] - eta1);
        }
        double along_rtemp0 = wet_nodes ? gravity * dt / fl * (1.0 - theta) * (eta_n2 - eta_n1) : 0.0;
        bt1 = (R)bt_rtemp1;
        along = (R)((btype == 0) ? (along_rtemp0 + bt_rtemp2) : along_rtemp0);
        air1 = (R)(rt0_air * ct2);
        air2 = (R)(rtemp3_air + rt0_air * sn2);
        bc_dj = (R)(-gravity * dt / (p.rho_o * dj));
        bc_fl = (R)(-gravity * dt / (p.rho_o * fl));
    }
    const R djR = (R)dj, flR = (R)fl, fl2 = (R)(fl * fl);
    const R gdt0 = (R)(gravity * dt);
    const R wsn = (R)(dt * f.wind_stress_normal[j - 1]), wst = (R)(dt * f.wind_stress_tangnt[j - 1]);
    const R qub = ibnd > 0 ? (R)s.qu_boundary[ibnd - 1] : R(0);
    const R smag = (R)p.smagorinsky, ah0 = (R)p.ah_0, kh0 = (R)p.kh_0, area1 = (R)g.area[a1 - 1];
    R rl1 = R(0), rl2 = R(0), inv_tq1 = R(0), inv_tq2 = R(0);
    int tq1 = 0, tq2 = 0;
    if (a2 != 0) {
        double ddx = g.x_cell[a1 - 1] - g.x_face[j - 1], ddy = g.y_cell[a1 - 1] - g.y_face[j - 1];
        double ddx2 = g.x_cell[a2 - 1] - g.x_face[j - 1], ddy2 = g.y_cell[a2 - 1] - g.y_face[j - 1];
        if constexpr (sizeof(R) == sizeof(float)) {
            rl1 = sqrtf((float)ddx * (float)ddx + (float)ddy * (float)ddy);
            rl2 = sqrtf((float)ddx2 * (float)ddx2 + (float)ddy2 * (float)ddy2);
        } else {
            rl1 = (R)sqrt(ddx * ddx + ddy * ddy);
            rl2 = (R)sqrt(ddx2 * ddx2 + ddy2 * ddy2);
        }
        tq1 = g.tri_or_quad[a1 - 1];
        tq2 = g.tri_or_quad[a2 - 1];
        inv_tq1 = tq1 == 4 ? R(0.25) : R(0);   // x/4 == x*0.25 exactly; triangles divide
        inv_tq2 = tq2 == 4 ? R(0.25) : R(0);
    }
    const R spin = (R)f.scal[2];
    const R half = R(0.5);
    for (int k = 1; k <= nvl; ++k) {
        int kk = tj - k + 1;
        R dzk = s.dz_face[ix(kk, j, L)];
        R unk = s.un_face[ix(kk, j, L)], vnk = s.vn_face[ix(kk, j, L)];
        R G1 = dzk * (s.un_elm[ix(kk, j, L)] + cordt * vnk);
        R G2 = dzk * (s.vn_elm[ix(kk, j, L)] - cordt * unk);
        if (a2 != 0) {
            // :269-344 Smagorinsky horizontal diffusion
            R tmp[12];
            for (int l = 1; l <= 2; ++l) {
                int nd = g.face_node(l, j);
                R ut = (s.u_node[ix0(kk, nd, L)] + s.u_node[ix0(kk - 1, nd, L)]) * half;
                R vt = (s.v_node[ix0(kk, nd, L)] + s.v_node[ix0(kk - 1, nd, L)]) * half;
                tmp[2 * l - 2] = ut * ctR + vt * snR;
                tmp[2 * l - 1] = -ut * snR + vt * ctR;
            }
            for (int l = 1; l <= 2; ++l) {
                int ie = l == 1 ? a1 : a2;
                int tq = l == 1 ? tq1 : tq2;
                R itq = l == 1 ? inv_tq1 : inv_tq2;
                R ut = R(0), vt = R(0);
                for (int ll = 1; ll <= tq; ++ll) {
                    int nd = g.cell_node(ll, ie);
                    R uu = (s.u_node[ix0(kk, nd, L)] + s.u_node[ix0(kk - 1, nd, L)]) * half;
                    R vv = (s.v_node[ix0(kk, nd, L)] + s.v_node[ix0(kk - 1, nd, L)]) * half;
                    ut = ut + (itq != R(0) ? uu * itq : uu / (R)tq);
                    vt = vt + (itq != R(0) ? vv * itq : vv / (R)tq);
                }
                tmp[2 * l + 2] = ut * ctR + vt * snR;
                tmp[2 * l + 3] = -ut * snR + vt * ctR;
            }
            R dudx = (tmp[6] - tmp[4]) / djR;
            R dvdx = (tmp[7] - tmp[5]) / djR;
            R dudy = (tmp[2] - tmp[0]) / flR;
            R dvdy = (tmp[3] - tmp[1]) / flR;
            R sdd = dvdx + dudy;
            R hdiff = smag * sqrt(dudx * dudx + dvdy * dvdy + half * (sdd * sdd));
            R khv = hdiff * area1;
            hdiff = hdiff + ah0;
            s.kh[ix(k, j, L)] = khv + kh0;
            R d2udy = R(4) * (tmp[2] + tmp[0] - R(2) * unk) / fl2;
            R d2vdy = R(4) * (tmp[3] + tmp[1] - R(2) * vnk) / fl2;
            tmp[8] = (tmp[4] - unk) / rl1;
            tmp[9] = (tmp[5] - vnk) / rl1;
            tmp[10] = (tmp[6] - unk) / rl2;
            tmp[11] = (tmp[7] - vnk) / rl2;
            R d2udx = R(2) * (tmp[8] + tmp[10]) / djR;
            R d2vdx = R(2) * (tmp[9] + tmp[11]) / djR;
            G1 = G1 + dzk * dtR * hdiff * (d2udx + d2udy);
            G2 = G2 + dzk * dtR * hdiff * (d2vdx + d2vdy);
        }
        // :350-397 barotropic gradients at (1-theta)
        if (btype >= 0) G1 = G1 - dzk * bt1;
        else G1 = R(0);
        if (wet_nodes) G2 = G2 - dzk * along;
        // :400-471 baroclinic pressure gradient (density differences formed in FP64)
        if (p.baroclinic_flag == 1) {
            R sum1 = R(0), sum2 = R(0);
            for (int k2 = kk; k2 <= tj; ++k2) {
                R dz2 = s.dz_face[ix(k2, j, L)];
                if (a2 != 0 && k2 >= ba1 && k2 <= ta1 && k2 >= ba2 && k2 <= ta2) {
                    R dr = (R)(s.rho_cell[ix(k2, a2, L)] - s.rho_cell[ix(k2, a1, L)]);
                    sum1 = sum1 + (k2 == kk ? half * dr : dr) * dz2;
                }
                if (k2 >= bn1 && k2 <= tn1 && k2 >= bn2 && k2 <= tn2) {
                    R dr = (R)(s.rho_node[ix(k2, node2, L)] - s.rho_node[ix(k2, node1, L)]);
                    sum2 = sum2 + (k2 == kk ? half * dr : dr) * dz2;
                }
            }
            R dzrow = s.dz_face[ix(k, j, L)];   // the reference uses the top-down row here
            R rtemp1 = dzrow * bc_dj * sum1;
            R rtemp2 = dzrow * bc_fl * sum2;
            R rtemp3 = rtemp1 * ct2R;
            R rtemp4 = rtemp1 * sn2R;
            G1 = G1 + rtemp3 * spin;
            G2 = G2 + (rtemp2 + rtemp4) * spin;
        }
        if (k == 1) {
            G1 = G1 + wsn;
            G2 = G2 + wst;
        }
        // :485-486 tide-generating potential, zero in this build (kept for the signed-zero result)
        G1 = G1 + c069 * dzk * gdt0 * R(0);
        G2 = G2 + c069 * dzk * gdt0 * R(0);
        // :490-509 air pressure
        G1 = G1 + dzk * air1;
        G2 = G2 + dzk * air2;
        if (btype == -1) G1 = R(0);
        if (ibnd > 0) G1 = G1 + dzk * qub;
        rhs[k - 1][0] = G1;
        rhs[k - 1][1] = G2;
        rhs[k - 1][2] = dzk;
    }
    if (!thomas<3>(nvl, a, bd, cu, rhs, gam)) {
        record_error(st, GOM_E_ZERO_PIVOT, 587, j, 0, 0.0);
        return;
    }
    bool zero_g1 = (btype == -1 && ibnd == 0);
    bool zero_dz1 = (btype == -1);
    for (int k = 1; k <= L; ++k) {
        long o = ix(k, j, L);
        if (k <= nvl) {
            s.ainvg1[o] = zero_g1 ? R(0) : rhs[k - 1][0];
            s.ainvg2[o] = rhs[k - 1][1];
            s.ainvdz1[o] = zero_dz1 ? R(0) : rhs[k - 1][2];
            s.ainvdz2[o] = rhs[k - 1][2];
        } else {
            s.ainvg1[o] = R(0);
            s.ainvg2[o] = R(0);
            s.ainvdz1[o] = R(0);
            s.ainvdz2[o] = R(0);
        }
    }
}

template <typename R> __global__ void k_zero_face_columns(Geom g, StateT<R> s) {
    // faces that are dry keep zero results (the reference zeroes all four arrays first)
    unsigned t = flat_tid();
    const int L = g.L;
    if (t >= (unsigned)g.NF * L) return;
    int j = (int)(t / (unsigned)L) + 1;
    if (s.top_face[j - 1] != 0) return;
    s.ainvg1[t] = R(0);
    s.ainvg2[t] = R(0);
    s.ainvdz1[t] = R(0);
    s.ainvdz2[t] = R(0);
}

template <typename R> cudaError_t launch_momentum_columns_only(const LaunchT<R> &x) {
    const int bs = x.tune[TUNE_MOMENTUM] == 1 ? 64 : x.tune[TUNE_MOMENTUM] == 2 ? 256 : 128;
    k_momentum<<<blocks_for(x.g.NF, bs), bs, 0, x.stream>>>(x.g, x.s, x.f, x.p, x.status);
    return cudaGetLastError();
}

template <typename R> cudaError_t launch_momentum(const LaunchT<R> &x) {
    long nfl = (long)x.g.NF * x.g.L;
    k_zero_face_columns<<<blocks_for(nfl, 256), 256, 0, x.stream>>>(x.g, x.s);
    const int bs = x.tune[TUNE_MOMENTUM] == 1 ? 64 : x.tune[TUNE_MOMENTUM] == 2 ? 256 : 128;
    k_momentum<<<blocks_for(x.g.NF, bs), bs, 0, x.stream>>>(x.g, x.s, x.f, x.p, x.status);
    return cudaGetLastError();
}

GOM_INSTANTIATE_LAUNCH(launch_bottom_friction)
GOM_INSTANTIATE_LAUNCH(launch_boundary_velocity)
GOM_INSTANTIATE_LAUNCH(launch_advection)
GOM_INSTANTIATE_LAUNCH(launch_momentum)
GOM_INSTANTIATE_LAUNCH(launch_elm_walk_only)
GOM_INSTANTIATE_LAUNCH(launch_momentum_columns_only)

}  // namespace gom
