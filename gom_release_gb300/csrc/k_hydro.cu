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
// Manning's Cdb depends on the static depth alone and comes formed on the host (the C library's
// pow, as the reference calls it); the log law's comes formed on the host for the static bottom
// half-thickness of a column with more than one layer, and is formed here only for a column of
// one layer, whose half-thickness is its depth (CUDA's log, within 1 ulp of the C library's).
template <typename R> __global__ void k_bottom_friction(Geom g, StateT<R> s, Params p) {
    int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (j > g.NF) return;
    const int L = g.L;
    double cdb = 0.0, gb = 0.0;
    double hf = g.h_face[j - 1];
    if (p.bf_flag >= 1 && p.bf_flag <= 3 && hf > p.dry_depth) {
        int k = g.bottom_face[j - 1];
        if (p.bf_flag == 1) {
            cdb = g.cdb_static[j - 1];
        } else if (p.bf_flag == 2) {
            const double dzh = s.dzhalf_face[ix0(k - 1, j, L)];
            if (dzh == g.cdb_arg[j - 1]) {
                cdb = g.cdb_static[j - 1];
            } else {
                double lg = log(fmax(0.5, dzh) / g.bf_height[j - 1]);
                cdb = p.von_karman * p.von_karman / (lg * lg);
            }
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
        record_error(st, GOM_E_DRY, 80, i, 0, depth, GOM_ENTITY_OTHER);
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
    // 1 if fl(num/den) in [0,1], 0 if not (den != 0); the tests on the bit patterns, with NaN
    // operands on the FP64 comparisons
    if (is_zero(num)) return 1;
    if (nan_bits(num) || nan_bits(den)) {
        if ((num < 0.0) != (den < 0.0)) return 0;
        return num / den <= 1.0;
    }
    if ((fbits(num) ^ fbits(den)) < 0) return 0;   // numbers, neither zero: the sign bits differ
    double an = fabs(num), ad = fabs(den);
    if (lt_of_nonneg(an, ad * (1.0 - 1e-9))) return 1;
    if (gt_nonneg(an, ad * (1.0 + 1e-9))) return 0;
    const double q = num / den;   // two numbers of one sign: +0 or more, or NaN (inf / inf)
    return !nan_bits(q) && fbits(q) <= fbits(1.0);
}

__device__ __forceinline__ int check_intersection(double x1, double x2, double x3, double x4, double y1, double y2,
                                                  double y3, double y4, double &xin, double &yin) {
    double delta = (x2 - x1) * (y3 - y4) - (y2 - y1) * (x3 - x4);
    if (is_zero(delta)) return 0;
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

// squared node-to-node length of each face in FP32, from the FP64 coordinate differences
__global__ void k_edge_len2(Geom g, float *out) {
    int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (j > g.NF) return;
    const int n1 = g.face_node(1, j), n2 = g.face_node(2, j);
    const float dx = (float)(g.x_node[n1 - 1] - g.x_node[n2 - 1]), dy = (float)(g.y_node[n1 - 1] - g.y_node[n2 - 1]);
    out[j - 1] = dx * dx + dy * dy;
}

cudaError_t launch_edge_len2(const Geom &g, float *out, cudaStream_t stream) {
    k_edge_len2<<<blocks_for(g.NF, 256), 256, 0, stream>>>(g, out);
    return cudaGetLastError();
}

__global__ void k_to_float(const double *in, float *out, long n) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)in[i];
}

__global__ void k_to_double(const float *in, double *out, long n) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (double)in[i];
}

cudaError_t launch_to_double(const float *in, double *out, long n, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    k_to_double<<<blocks_for(n, 256), 256, 0, stream>>>(in, out, n);
    return cudaGetLastError();
}

// MSL - h of every cell (the bottom of its water column), static
__global__ void k_cell_zbot(Geom g, double msl, double *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < g.NC) out[i] = msl - g.h_cell[i];
}

cudaError_t launch_cell_zbot(const Geom &g, double msl, double *out, cudaStream_t stream) {
    k_cell_zbot<<<blocks_for(g.NC, 256), 256, 0, stream>>>(g, msl, out);
    return cudaGetLastError();
}

// FP32 copy of the cell bottom heights for the mixed walk: a bottom above the lowest level stays
// above its FP32 copy (the walk's range test then fails only where the FP64 one does)
__global__ void k_cell_zbot_f(Geom g, const double *zbot, float *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.NC) return;
    const float z0f = (float)g.z_level[0];
    float zf = (float)zbot[i];
    if (zbot[i] > g.z_level[0] && !(zf > z0f)) zf = nextafterf(z0f, INFINITY);
    out[i] = zf;
}

cudaError_t launch_cell_zbot_f(const Geom &g, const double *zbot, float *out, cudaStream_t stream) {
    k_cell_zbot_f<<<blocks_for(g.NC, 256), 256, 0, stream>>>(g, zbot, out);
    return cudaGetLastError();
}

cudaError_t launch_to_float(const double *in, float *out, long n, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    k_to_float<<<blocks_for(n, 256), 256, 0, stream>>>(in, out, n);
    return cudaGetLastError();
}

cudaError_t launch_elem_local(const Geom &g, float *out, cudaStream_t stream) {
    k_elem_local<<<blocks_for(g.NC, 256), 256, 0, stream>>>(g, out);
    return cudaGetLastError();
}

__device__ __forceinline__ void load_local(const Geom &g, int nel, LocalElem &e) {
    e.tq = g.tri_or_quad[nel - 1];
    e.xc = g.x_cell[nel - 1];
    e.yc = g.y_cell[nel - 1];
    e.ar = g.area_f[nel - 1];
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

// v[i] of a 4-entry register array for a run-time i in 0..3 (selects: a dynamic index would put
// the array in local memory)
__device__ __forceinline__ float sel4(const float (&v)[4], int i) {
    return i == 0 ? v[0] : i == 1 ? v[1] : i == 2 ? v[2] : v[3];
}

// 1: inside by the reference's test, 0: outside, -1: not decidable in FP32.  near: an edge line
// passes within the FP32 error bound of the point.  (px, py) is within u (|px| + |py| + pext) of
// the point's exact offset from the element centre (pext = 0: rounded from the FP64 offset).
__device__ __forceinline__ int classify_f32(const LocalElem &e, float px, float py, bool &near, float pext = 0.0f) {
    const float u = 5.97e-8f;   // 2^-24
    float lo = 0.0f, hi = 0.0f;
    near = false;
    float twice_area = 0.0f;   // counter-clockwise elements only (as cell.inp requires)
    // (loops unrolled over the 4 slots so that every index is a constant)
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        if (l >= e.tq) break;
        const bool wrap = l + 1 == e.tq;
        const float xm = wrap ? e.x[0] : e.x[(l + 1) & 3], ym = wrap ? e.y[0] : e.y[(l + 1) & 3];
        twice_area += e.x[l] * ym - xm * e.y[l];
    }
    if (!(twice_area > 0.0f)) {
        near = true;
        return -1;
    }
    if (e.tq == 4) {
        // the excess identity needs a convex quad (then its two-triangle area is the polygon's)
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            const int m = (l + 1) & 3, n = (l + 2) & 3;
            const float turn = (e.x[m] - e.x[l]) * (e.y[n] - e.y[m]) - (e.y[m] - e.y[l]) * (e.x[n] - e.x[m]);
            const float mag = (fabsf(e.x[l]) + fabsf(e.x[m]) + fabsf(e.x[n])) * (fabsf(e.y[l]) + fabsf(e.y[m]) + fabsf(e.y[n]));
            if (!(turn > 16.0f * u * mag)) {
                near = true;
                return -1;
            }
        }
    }
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        if (l >= e.tq) break;
        const bool wrap = l + 1 == e.tq;
        const float xm = wrap ? e.x[0] : e.x[(l + 1) & 3], ym = wrap ? e.y[0] : e.y[(l + 1) & 3];
        float ex = xm - e.x[l], ey = ym - e.y[l];
        float dx = px - e.x[l], dy = py - e.y[l];
        float c = ex * dy - ey * dx;
        // inputs rounded from FP64 differences, two subtractions, two products, one subtraction
        float mag = (fabsf(xm) + fabsf(e.x[l]) + fabsf(ym) + fabsf(e.y[l])) *
                    (fabsf(px) + fabsf(py) + pext + fabsf(e.x[l]) + fabsf(e.y[l]));
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

// The last FP32 classification of the search (mixed path): when the search ends because the foot
// tested inside element nnel, the caller reuses that element's local data and test instead of
// repeating them.
struct LastTest {
    bool valid = false;
    LocalElem el;
    float px, py;
    int cls;
    bool near;
};

// Mixed path: check_intersection.f90 on element-local FP32 coordinates, deciding only where an
// error bound on the FP32 determinants settles the reference's FP64 outcome (tt1 and tt2 in [0, 1],
// the sign and magnitude tests of unit_range): 1 crossed (crossing point set), 0 not crossed,
// -1 not decidable in FP32.  Bound: with Mx, My the sums of the |coordinates|, every coordinate
// difference is within 2u Mx (2u My) of its exact value (rounding of the FP64 offsets to FP32 and
// of the difference), so each determinant of two products is within about 12.3 u Mx My; 16 u Mx
// My is used.
__device__ __forceinline__ int cross_f32(float x1, float x2, float x3, float x4, float y1, float y2, float y3,
                                         float y4, float &xin, float &yin) {
    const float u = 5.97e-8f;   // 2^-24
    const float ax = x2 - x1, ay = y2 - y1, bx = x3 - x4, by = y3 - y4, cx = x3 - x1, cy = y3 - y1;
    const float mx = fabsf(x1) + fabsf(x2) + fabsf(x3) + fabsf(x4), my = fabsf(y1) + fabsf(y2) + fabsf(y3) + fabsf(y4);
    const float ed = 16.0f * u * mx * my + 1e-30f, e1 = ed, e2 = ed;
    const float delta = ax * by - ay * bx;
    if (fabsf(delta) <= ed) return -1;
    const float d1 = cx * by - cy * bx;
    const float d2 = ax * cy - ay * cx;
    // tt = d / delta in [0, 1]: d on delta's side of 0 and |d| <= |delta|; a parameter settled
    // outside decides "not crossed" whatever the other one is
    int r = 1;
    const float dd[2] = {d1, d2}, ee[2] = {e1, e2};
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const float d = dd[q], e = ee[q];
        const float m = fabsf(d) - fabsf(delta);
        if (fabsf(d) > e && (d < 0.0f) != (delta < 0.0f)) return 0;   // tt < 0
        if (m > e + ed) return 0;                                      // tt > 1
        if (fabsf(d) <= e || fabsf(m) <= e + ed) r = -1;               // tt near 0 or 1
    }
    if (r < 0) return -1;
    const float t1 = d1 / delta;
    xin = x1 + ax * t1;
    yin = y1 + ay * t1;
    return 1;
}

// Mixed path: the element-to-element walk of search_straight_line.f90:47-283 with the segment,
// the crossing points and the remaining-path bookkeeping in FP32 on coordinates relative to the
// centre of the element being crossed (re-based in FP64 at every element); every edge and
// in-element decision is the reference's (FP32 under an error bound, FP64 where that does not
// settle it), the foot itself stays FP64.  Entered when the foot is not in the start
// element; on return the foot is in nnel (last holds that test) or nfl = 1 (stopped at a dry or
// land edge, foot moved to the crossing point).
// edge l of element nel crossed by the segment (xcg, ycg) -> (xt, yt): the FP32 decision, or the
// reference's FP64 check_intersection where that is not settled; crossing point in nel's frame
__device__ __forceinline__ bool crosses(const Geom &g, int nel, const LocalElem &e, int l, float sx, float sy, float tx,
                                        float ty, double xcg, double ycg, double xt, double yt, float &xin,
                                        float &yin) {
    const int a = l % e.tq, b = (l + 1) % e.tq;   // local nodes start_end_node(tq, l, 1..2) - 1
    const int r = cross_f32(sx, tx, sel4(e.x, a), sel4(e.x, b), sy, ty, sel4(e.y, a), sel4(e.y, b), xin, yin);
    if (r >= 0) return r == 1;
    const int jd1 = g.cell_node(start_end_node(e.tq, l, 1), nel), jd2 = g.cell_node(start_end_node(e.tq, l, 2), nel);
    double xi = 0.0, yi = 0.0;
    if (!check_intersection(xcg, xt, g.x_node[jd1 - 1], g.x_node[jd2 - 1], ycg, yt, g.y_node[jd1 - 1],
                            g.y_node[jd2 - 1], xi, yi))
        return false;
    xin = (float)(xi - e.xc);
    yin = (float)(yi - e.yc);
    return true;
}

template <typename R>
__device__ int walk_f32(const Geom &g, const StateT<R> &s, int &nnel, double time, double x0, double y0, double z0,
                        double &xt, double &yt, double &zt, int &nfl, LastTest &last) {
    const double c1d = 1.0 - 1.0e-4;
    const float c1 = (float)c1d;
    int nel = nnel;
    LocalElem e;
    load_local(g, nel, e);
    // the reference's nudged start xcg = c1 x0 + 1e-4 x_cell is c1 (x0 - x_cell) from the centre
    float sx = c1 * (float)(x0 - e.xc), sy = c1 * (float)(y0 - e.yc);
    float tx = (float)(xt - e.xc), ty = (float)(yt - e.yc);
    float pathl = sqrtf((tx - sx) * (tx - sx) + (ty - sy) * (ty - sy));
    if (pathl == 0.0f) return GOM_ELM_ZERO_PATH;
    // the reference's FP64 segment start, for the edges FP32 cannot decide
    const double xcg = c1d * x0 + 1.0e-4 * g.x_cell[nel - 1], ycg = c1d * y0 + 1.0e-4 * g.y_cell[nel - 1];
    int nel_j = 0;
    float xin = 0.0f, yin = 0.0f;
    for (int l = 1; l <= e.tq; ++l) {
        if (crosses(g, nel, e, l, sx, sy, tx, ty, xcg, ycg, xt, yt, xin, yin)) {
            nel_j = l;
            break;
        }
    }
    if (nel_j == 0) return GOM_ELM_NO_FIRST_EDGE;
    // A walk that stops on an edge takes its foot from that crossing point, formed in FP64: FP32
    // offsets lose the small components of a path running nearly along the edge.  The height
    // there is the reference's zin, the product of the remaining-path ratios of all crossings,
    // which telescopes to |T - crossing| / |T - start|.
    const double pathl0 = sqrt((xt - xcg) * (xt - xcg) + (yt - ycg) * (yt - ycg));
    auto stop_at_edge = [&](int el, int l, const LocalElem &le, float fxin, float fyin, double &xi, double &yi) {
        const int q = le.tq;
        const int jd1 = g.cell_node(start_end_node(q, l, 1), el), jd2 = g.cell_node(start_end_node(q, l, 2), el);
        if (!check_intersection(xcg, xt, g.x_node[jd1 - 1], g.x_node[jd2 - 1], ycg, yt, g.y_node[jd1 - 1],
                                g.y_node[jd2 - 1], xi, yi)) {
            xi = le.xc + (double)fxin;   // not reached: the FP32 crossing decision is the FP64 one
            yi = le.yc + (double)fyin;
        }
        const double dist = sqrt((xi - xt) * (xi - xt) + (yi - yt) * (yi - yt));
        zt = zt - dist / pathl0 * (zt - z0);
    };
    // FP64 distance from the crossing on edge l of element el to the foot (the reference's dist)
    auto dist64 = [&](int el, int l) {
        const int q = g.tri_or_quad[el - 1];
        const int jd1 = g.cell_node(start_end_node(q, l, 1), el), jd2 = g.cell_node(start_end_node(q, l, 2), el);
        double xi = 0.0, yi = 0.0;
        check_intersection(xcg, xt, g.x_node[jd1 - 1], g.x_node[jd2 - 1], ycg, yt, g.y_node[jd1 - 1],
                           g.y_node[jd2 - 1], xi, yi);
        return sqrt((xi - xt) * (xi - xt) + (yi - yt) * (yi - yt));
    };
    int prev_el = 0, prev_l = 0;   // the previous crossing (none: the remaining path is pathl0)
    int iteration = 0;
    for (;;) {
        iteration = iteration + 1;
        if (iteration > 1000) {
            double xi, yi;
            stop_at_edge(nel, nel_j, e, xin, yin, xi, yi);
            nfl = 1;
            xt = xi;
            yt = yi;
            nnel = nel;
            last.valid = false;
            return 0;
        }
        const int tqn = e.tq;
        const int md1 = g.cell_node(start_end_node(tqn, nel_j, 1), nel);
        const int md2 = g.cell_node(start_end_node(tqn, nel_j, 2), nel);
        // the reference's checks of the remaining path (:199-222): the FP32 lengths lose accuracy
        // on paths nearly along an edge, so a check they fail is repeated with FP64 crossings
        const float dist = sqrtf((xin - tx) * (xin - tx) + (yin - ty) * (yin - ty));
        if (dist > pathl * (1.0f + 0.5e-4f) || dist == 0.0f) {
            const double d = dist64(nel, nel_j);
            const double dprev = prev_el ? dist64(prev_el, prev_l) : pathl0;
            if (gt_nonneg(d / dprev, 1.0 + 1.0e-4)) return GOM_ELM_OVERSHOOT;   // d / dprev: +0 or more
            if (is_zero(d) || is_zero(time * d / pathl0)) return GOM_ELM_ZERO_REMAIN;
        }
        pathl = dist;
        prev_el = nel;
        prev_l = nel_j;
        const int adjc = g.cell_adj(nel_j, nel);
        if (adjc == 0 || top_el(s, adjc) == 0) {
            const int isd = g.cell_face(nel_j, nel);
            if (g.face_node(1, isd) + g.face_node(2, isd) != md1 + md2) return GOM_ELM_FACE_MISMATCH;
            double xi, yi;
            stop_at_edge(nel, nel_j, e, xin, yin, xi, yi);
            nfl = 1;
            xt = c1d * xi + 1.0e-4 * g.x_cell[nel - 1];
            yt = c1d * yi + 1.0e-4 * g.y_cell[nel - 1];
            nnel = nel;
            last.valid = false;
            return 0;
        }
        nel = adjc;
        LocalElem e2;
        load_local(g, nel, e2);
        const float dx = (float)(e.xc - e2.xc), dy = (float)(e.yc - e2.yc);
        sx += dx;
        sy += dy;
        xin += dx;
        yin += dy;
        e = e2;
        tx = (float)(xt - e.xc);
        ty = (float)(yt - e.yc);
        last.el = e;
        last.px = tx;
        last.py = ty;
        last.cls = classify_f32(e, tx, ty, last.near);
        if (last.cls >= 0 ? last.cls == 1 : in_elem64(g, nel, xt, yt)) {
            nnel = nel;
            last.valid = true;
            return 0;
        }
        bool found = false;
        for (int l = 1; l <= e.tq; ++l) {
            const int jd1 = g.cell_node(start_end_node(e.tq, l, 1), nel);
            const int jd2 = g.cell_node(start_end_node(e.tq, l, 2), nel);
            if ((jd1 == md1 && jd2 == md2) || (jd2 == md1 && jd1 == md2)) continue;
            if (crosses(g, nel, e, l, sx, sy, tx, ty, xcg, ycg, xt, yt, xin, yin)) {
                nel_j = l;
                found = true;
                break;
            }
        }
        if (!found) return GOM_ELM_NO_NEXT_EDGE;
    }
}

template <typename R>
__device__ int search_straight_line(const Geom &g, const StateT<R> &s, const Params &p, int &nnel, int &jlev, double time,
                                    double x0, double y0, double z0, double &xt, double &yt, double &zt, int &nfl,
                                    bool first_substep) {
    const double small_06 = F(1.e-6f);
    const int L = g.L;
    // The reference's start tests (:26-46) are known to pass and not evaluated, except the dry
    // test of the first substep.  The start-in-element test of the first substep: the start is the
    // midpoint of an edge of the start element, area excess zero up to FP64 rounding, far below
    // the tolerance.  Both tests of a later substep: it starts at the previous foot, and the
    // previous search ended only after that foot tested inside nnel (the complementary test on the
    // same operands) and nnel passed the same dry test (:370).
    if (first_substep && s.dry_cell[nnel - 1])
        return GOM_ELM_START_DRY;
    nfl = 0;
    double trm = time;
    int nel = nnel;
    if (!in_elem64(g, nel, xt, yt)) {
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
            if (gt_nonneg(dist / pathl, 1.0 + 1.0e-4)) return GOM_ELM_OVERSHOOT;   // dist / pathl: +0 or more
            zin = zt - dist / pathl * (zt - zin);
            trm = trm * dist / pathl;
            pathl = sqrt((xin - xt) * (xin - xt) + (yin - yt) * (yin - yt));
            if (is_zero(pathl) || is_zero(trm)) return GOM_ELM_ZERO_REMAIN;
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
            if (in_elem64(g, nel, xt, yt)) {
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
    if (s.dry_cell[nnel - 1]) return GOM_ELM_END_DRY;
    zt = fmin(fmax(zt, g.zbot_cell[nnel - 1]), s.ztop_cell[nnel - 1]);
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

// the last substep's foot, the surface or level height above it and the interpolation weights
// (the ELM transport interpolates the tracers with them, ELM_backtrace_v1.f90:216-473)
struct ElmFinal {
    double xt, yt, zt, zup;
    double staint[4];
};

// Mixed path of ELM_backtrace_v1.f90:40-200.  The foot is an FP32 offset (dx, dy) from an FP64
// origin (ox, oy), the start point: the foot's FP64 position is ox + dx, formed only where an FP64
// decision or the final position needs it, so a substep whose foot stays in its element runs on
// the FP32 pipe alone.  The element-local offset px = bx + dx with bx = ox - x_centre rounded to
// FP32 once per element is within u (|px| + |bx|) + 2^-53 |ox + dx| of the exact offset of that
// FP64 position; classify_f32 decides the reference's point-in-element test under that bound
// (pext = |bx| + |by| + 2^-28 (|ox| + |oy|)) and in_elem64 at the FP64 position decides the rest,
// so every decision is the FP64 test of one well-defined point.  A foot that leaves its element
// is walked by walk_f32 from the FP64 positions.  The height and the layer search are FP32 (the
// level heights and the column's bottom and surface heights rounded to FP32; near a level the
// neighbouring layers give the same interpolated velocity), velocities and weights FP32.
template <typename R>
__device__ int elm_backtrace_mixed(const Geom &g, const StateT<R> &s, int bt_step, double bt_dt, double &uu,
                                   double &vv, double &ww, double x0, double y0, double z0, int &nnel, int &jlev,
                                   int &near_edge, ElmFinal *fin) {
    const int L = g.L;
    const float btf = (float)bt_dt;
    const double ox = x0, oy = y0;
    const float omag = ldexpf(fabsf((float)ox) + fabsf((float)oy), -28);
    float uf = (float)uu, vf = (float)vv, wf = (float)ww;
    float dx0 = 0.0f, dy0 = 0.0f, zs = (float)z0;   // start of the substep
    int bel = 0;                                    // element of (bx, by)
    float bx = 0.0f, by = 0.0f;
    LastTest last;
    for (int idt = 1; idt <= bt_step; ++idt) {
        const float dxt = dx0 - btf * uf, dyt = dy0 - btf * vf;
        float zt = zs - btf * wf;
        // start tests of search_straight_line.f90:26-46: only the dry test of the first substep
        // is evaluated (the others are known to pass, as in the FP64 path)
        if (idt == 1 && s.dry_cell[nnel - 1]) return GOM_ELM_START_DRY;
        int nfl = 0;
        double xt64 = 0.0, yt64 = 0.0;   // the foot moved onto an edge crossing (nfl = 1)
        {
            LocalElem &el = last.el;
            load_local(g, nnel, el);
            if (bel != nnel) {
                bx = (float)(ox - el.xc);
                by = (float)(oy - el.yc);
                bel = nnel;
            }
            last.px = bx + dxt;
            last.py = by + dyt;
            last.cls = classify_f32(el, last.px, last.py, last.near, fabsf(bx) + fabsf(by) + omag);
            last.valid = true;
            if (!(last.cls >= 0 ? last.cls == 1 : in_elem64(g, nnel, ox + (double)dxt, oy + (double)dyt))) {
                double xt = ox + (double)dxt, yt = oy + (double)dyt, ztd = zt;
                last.valid = false;
                int e = walk_f32(g, s, nnel, bt_dt, ox + (double)dx0, oy + (double)dy0, (double)zs, xt, yt, ztd, nfl,
                                 last);
                if (e) return e;
                zt = (float)ztd;
                xt64 = xt;
                yt64 = yt;
            }
        }
        if (s.dry_cell[nnel - 1]) return GOM_ELM_END_DRY;
        zt = fminf(fmaxf(zt, g.zbot_cell_f[nnel - 1]), s.ztop_cell_f[nnel - 1]);
        if (zt <= g.z_level_f[0] || zt > g.z_level_f[L]) return GOM_ELM_Z_RANGE;
        {
            int k = min(max(jlev - 1, 0), L - 1);
            while (k < L - 1 && zt > g.z_level_f[k + 1]) ++k;
            while (k > 0 && zt <= g.z_level_f[k]) --k;
            jlev = k + 1;
        }
        jlev = min(max(jlev, g.bottom_cell[nnel - 1]), top_el(s, nnel));
        const bool top_layer = jlev == s.top_cell[nnel - 1];
        const float zup = top_layer ? s.ztop_cell_f[nnel - 1] : g.z_level_f[jlev];
        if (zt > zup) return GOM_ELM_Z_ABOVE;
        const float zrat = (zup - zt) / (float)s.dz_cell[ix(jlev, nnel, L)];
        if (!last.valid) {   // the walk stopped on an edge: the foot is the FP64 crossing point
            load_local(g, nnel, last.el);
            last.px = (float)(xt64 - last.el.xc);
            last.py = (float)(yt64 - last.el.yc);
            last.cls = classify_f32(last.el, last.px, last.py, last.near);
        }
        // the foot's FP64 position, formed where needed
        auto foot_x = [&]() { return nfl ? xt64 : ox + (double)dxt; };
        auto foot_y = [&]() { return nfl ? yt64 : oy + (double)dyt; };
        const LocalElem &el = last.el;
        const float px = last.px, py = last.py;
        const int tq = el.tq;
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
            if (last.cls >= 0 ? last.cls == 0 : out_elem64(g, nnel, foot_x(), foot_y())) return GOM_ELM_QUAD_OUTSIDE;
            int b = bilinear_interpolation<float>(el.x[0], el.x[1], el.x[2], el.x[3], el.y[0], el.y[1], el.y[2],
                                                  el.y[3], px, py, sta);
            if (b) return b;
        }
        float fu = 0.0f, fv = 0.0f, fw = 0.0f;
#pragma unroll
        for (int l = 1; l <= 4; ++l) {
            if (l > tq) break;
            int nd = g.cell_node(l, nnel);
            long i1 = ix0(jlev - 1, nd, L), i2 = ix0(jlev, nd, L);
            float w = sta[l - 1];
            fu = fu + ((float)s.u_node[i2] * (1.0f - zrat) + (float)s.u_node[i1] * zrat) * w;
            fv = fv + ((float)s.v_node[i2] * (1.0f - zrat) + (float)s.v_node[i1] * zrat) * w;
            fw = fw + ((float)s.w_node[i2] * (1.0f - zrat) + (float)s.w_node[i1] * zrat) * w;
        }
        uf = fu;
        vf = fv;
        wf = fw;
        if (last.near && near_edge_line(g, nnel, foot_x(), foot_y())) near_edge = 1;
        if (fin) {
            const double zup64 = top_layer ? s.ztop_cell[nnel - 1] : g.z_level[jlev];
            *fin = ElmFinal{foot_x(), foot_y(), (double)zt, zup64, {0.0, 0.0, 0.0, 0.0}};
#pragma unroll
            for (int l = 0; l < 4; ++l)
                if (l < tq) fin->staint[l] = sta[l];
        }
        if (nfl == 1) break;
        dx0 = dxt;
        dy0 = dyt;
        zs = zt;
    }
    uu = uf;
    vv = vf;
    ww = wf;
    return 0;
}

// ELM_backtrace_v1.f90:40-200 (mode 1).  The first substep starts at the face midpoint, on an
// edge of the start element (the ELM transport starts at the cell centre).  MIXED: see
// elm_backtrace_mixed.
template <typename R, bool MIXED>
__device__ int elm_backtrace(const Geom &g, const StateT<R> &s, const Params &p, int bt_step, double bt_dt, double &uu,
                             double &vv, double &ww, double x0, double y0, double z0, int &nnel, int &jlev,
                             int &near_edge, ElmFinal *fin = nullptr) {
    if constexpr (MIXED) {
        return elm_backtrace_mixed(g, s, bt_step, bt_dt, uu, vv, ww, x0, y0, z0, nnel, jlev, near_edge, fin);
    } else {
        const double small_06 = F(1.e-6f);
        const int L = g.L;
        for (int idt = 1; idt <= bt_step; ++idt) {
            double xt = x0 - bt_dt * uu;
            double yt = y0 - bt_dt * vv;
            double zt = z0 - bt_dt * ww;
            int nfl = 0;
            int e = search_straight_line<R>(g, s, p, nnel, jlev, bt_dt, x0, y0, z0, xt, yt, zt, nfl, idt == 1);
            if (e) return e;
            int tq = g.tri_or_quad[nnel - 1];
            const bool top_layer = jlev == s.top_cell[nnel - 1];
            const double zup = top_layer ? s.ztop_cell[nnel - 1] : g.z_level[jlev];
            if (zt > zup) return GOM_ELM_Z_ABOVE;
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
            if (fin) {
                *fin = ElmFinal{xt, yt, zt, zup, {0.0, 0.0, 0.0, 0.0}};
                for (int l = 0; l < tq; ++l) fin->staint[l] = sta[l];
            }
            if (nfl == 1) break;
            x0 = xt;
            y0 = yt;
            z0 = zt;
        }
        return 0;
    }
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
        const float rl2 = g.edge_len2_f[j - 1];
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
    constexpr bool MIXED = sizeof(R) == sizeof(float);
    long o = ix(k, j, L);
    int nnel = ie0, jlev = k;
    double x0 = g.x_face[j - 1], y0 = g.y_face[j - 1], z0;
    if (k == s.top_cell[nnel - 1]) z0 = s.ztop_cell[nnel - 1] - s.dz_cell[ix(k, nnel, L)] * 0.5;
    else z0 = g.z_level[k] - s.dz_cell[ix(k, nnel, L)] * 0.5;
    // the velocity at the face-layer midpoint and the walk threshold of :166 (vmag = sqrt(q) <=
    // thr), decided on q against thr^2 away from the threshold; in both paths the decision is
    // that of the FP64 arithmetic, so a face-layer at the threshold is walked or not as in the FP64
    // path.  The mixed path first tries the rotation-free FP32 norm un^2 + vn^2 + w^2 (within
    // 1e-6 of the FP64 q) and needs the FP64 q only within 1e-5 of the threshold.
    const double thr = F(1.e-4f), t2 = thr * thr;
    int decided = -1;   // 1 slow, 0 walk
    if constexpr (MIXED) {
        const float unf = s.un_face[o], vnf = s.vn_face[o];
        const float wd = (s.w_node[ix0(k - 1, n1, L)] + s.w_node[ix0(k - 1, n2, L)]) * 0.5f;
        const float wu = (s.w_node[ix0(k, n1, L)] + s.w_node[ix0(k, n2, L)]) * 0.5f;
        const float wf = (wd + wu) * 0.5f;
        const float qf = unf * unf + vnf * vnf + wf * wf, t2f = (float)t2;
        if (qf < t2f * (1.0f - 1e-5f)) decided = 1;
        else if (qf > t2f * (1.0f + 1e-5f)) decided = 0;
    }
    double uu, vv, ww;
    bool slow;
    if (decided == 1) {
        slow = true;
        uu = vv = ww = 0.0;
    } else {
        double unf = s.un_face[o], vnf = s.vn_face[o];
        if constexpr (MIXED) {
            // the walk starts from FP32 velocities (rotated with the FP32 direction cosines)
            const float ctf = g.cos_theta_f[j - 1], snf = g.sin_theta_f[j - 1];
            const float u32 = s.un_face[o], v32 = s.vn_face[o];
            uu = u32 * ctf - v32 * snf;
            vv = u32 * snf + v32 * ctf;
            const float wd = (s.w_node[ix0(k - 1, n1, L)] + s.w_node[ix0(k - 1, n2, L)]) * 0.5f;
            const float wu = (s.w_node[ix0(k, n1, L)] + s.w_node[ix0(k, n2, L)]) * 0.5f;
            ww = (wd + wu) * 0.5f;
        } else {
            uu = unf * ct - vnf * sn;
            vv = unf * sn + vnf * ct;
            double wdown = (s.w_node[ix0(k - 1, n1, L)] + s.w_node[ix0(k - 1, n2, L)]) * 0.5;
            double wup = (s.w_node[ix0(k, n1, L)] + s.w_node[ix0(k, n2, L)]) * 0.5;
            ww = (wdown + wup) * 0.5;
        }
        if (decided == 0) {
            slow = false;
        } else {
            const double u64 = unf * ct - vnf * sn, v64 = unf * sn + vnf * ct;
            const double q = u64 * u64 + v64 * v64 + ww * ww;
            if (q < t2 * (1.0 - 1e-9)) slow = true;
            else if (q > t2 * (1.0 + 1e-9)) slow = false;
            else slow = sqrt(q) <= thr;
        }
    }
    if (slow) {
        s.un_elm[o] = s.un_face[o];
        s.vn_elm[o] = s.vn_face[o];
        return;
    }
    // INT((n1 + n2) * 0.5) of two integers is their truncated integer half; dt / bt_step from the
    // table of dt / n (the same correctly rounded quotients) when n is in its range
    int bt_step = (s.num_sub_elm[ix(k, n1, L)] + s.num_sub_elm[ix(k, n2, L)]) / 2;
    double bt_dt = (bt_step >= 1 && bt_step <= GOM_BT_TABLE) ? p.bt_dt[bt_step - 1] : p.dt / bt_step;
    int near = 0;
    int e = elm_backtrace<R, MIXED>(g, s, p, bt_step, bt_dt, uu, vv, ww, x0, y0, z0, nnel, jlev, near);
    if (e) {
        record_error(st, GOM_E_ELM, e, j, k, 0.0, GOM_ENTITY_FACE);
        return;
    }
    s.elm_foot[o] = nnel;
    s.elm_near_edge[o] = near;
    if constexpr (MIXED) {
        const float ctf = g.cos_theta_f[j - 1], snf = g.sin_theta_f[j - 1], uf = (float)uu, vf = (float)vv;
        s.un_elm[o] = uf * ctf + vf * snf;
        s.vn_elm[o] = -uf * snf + vf * ctf;
    } else {
        s.un_elm[o] = (R)(uu * ct + vv * sn);
        s.vn_elm[o] = (R)(-uu * sn + vv * ct);
    }
}

template <typename R, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_elm_faces(Geom g, StateT<R> s, Params p, gom_status *st) {
    unsigned tid = flat_tid();
    if (tid >= (unsigned)g.NF) return;
    int j = column_entity<R>(g.face_order, tid);
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

template <typename R> __global__ void k_cell_z(Geom g, StateT<R> s, Params p);

template <typename R> cudaError_t launch_elm_walk_only(const LaunchT<R> &x) {
    k_cell_z<<<blocks_for(x.g.NC, 256), 256, 0, x.stream>>>(x.g, x.s, x.p);
    return launch_elm_walk(x);
}

// The cell's surface height MSL + eta and its dry test of search_straight_line.f90:37-46 and
// :363-372 (no layer, or MSL - h above MSL + eta), once per cell per step instead of at every
// substep of every face-layer; the same FP64 expressions, hence the same values.
template <typename R> __global__ void k_cell_z(Geom g, StateT<R> s, Params p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.NC) return;
    const double ztop = p.msl + s.eta_cell[i];
    s.ztop_cell[i] = ztop;
    if constexpr (sizeof(R) == 4) s.ztop_cell_f[i] = (float)ztop;
    s.dry_cell[i] = (s.top_cell[i] == 0 || g.zbot_cell[i] > ztop) ? 1 : 0;
}

template <typename R> cudaError_t launch_advection(const LaunchT<R> &x) {
    long nfl = (long)x.g.NF * x.g.L;
    if (x.p.advection_flag != 0)
        k_cell_z<<<blocks_for(x.g.NC, 256), 256, 0, x.stream>>>(x.g, x.s, x.p);
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
// solve_transport_equation_ELM_v8.f90:7-346 (transport_solver = 2).  The reference's quirks are
// kept: the horizontal sums use the face's second cell as the neighbour and go to the other
// tracer (salinity differences to temperature, :137-151), the top row's upper coefficient is
// -dt + Kv/dzhalf (:188), no clamp, dry cells and dry nodes keep their previous values, face
// values average the two nodes in every layer.  The heat source term of :120 is left out (phi_sz
// comes from the heat-balance module, not part of the core).  Work: con holds the backtracked values and
// con2 the explicit right-hand sides, tracer slot 0 temperature and 1 salinity.

// ELM_backtrace_v1.f90:216-473: temperature and salinity at the foot (FP64 geometry, tracers in R)
template <typename R>
__device__ int elm_tracer_at_foot(const Geom &g, const StateT<R> &s, const Forcing &f, const ElmFinal &fin, int nnel,
                                  int jlev, double &ttint, double &ssint) {
    const double small_06 = F(1.e-6f);
    const int L = g.L;
    const double xt = fin.xt, yt = fin.yt, zt = fin.zt, zup = fin.zup;
    const int ibnd1 = g.ob_element_flag[nnel - 1], ibnd2 = g.qb_element_flag[nnel - 1];
    ttint = 0.0;
    ssint = 0.0;
    if (ibnd1 > 0) {   // the boundary concentration, the same in every layer
        ssint = f.con_at_ob[ibnd1 - 1];
        ttint = f.con_at_ob[g.NOB + ibnd1 - 1];
        return 0;
    }
    if (ibnd2 > 0) {
        ssint = f.con_at_qb[ibnd2 - 1];
        ttint = f.con_at_qb[g.NQB + ibnd2 - 1];
        return 0;
    }
    const double zanchor = zup - (double)s.dz_cell[ix(jlev, nnel, L)] * 0.5;
    int k1, k2;
    double zrat2;
    if (jlev == s.top_cell[nnel - 1] && zt > zanchor) {
        k1 = jlev;
        k2 = jlev;
        zrat2 = 0.5;
    } else if (zt > zanchor) {
        k1 = jlev;
        k2 = jlev + 1;
        zrat2 = (zt - zanchor) / (double)s.dzhalf_cell[ix0(jlev, nnel, L)];
    } else {
        k1 = max(jlev - 1, g.bottom_cell[nnel - 1]);
        k2 = jlev;
        zrat2 = 1.0 - (zanchor - zt) / (double)s.dzhalf_cell[ix0(k1, nnel, L)];
    }
    zrat2 = fmax(0.0, fmin(1.0, zrat2));
    auto lev = [&](const R *a, int e) {
        return (double)a[ix(k1, e, L)] * (1 - zrat2) + (double)a[ix(k2, e, L)] * zrat2;
    };
    const int tq = g.tri_or_quad[nnel - 1];
    int icount = 0;
    double ta = 0.0, sa = 0.0, t_xi[4] = {0, 0, 0, 0}, s_xi[4] = {0, 0, 0, 0};
    for (int l = 1; l <= tq; ++l) {
        const int nd = g.cell_node(l, nnel);
        if (s.top_node[nd - 1] != 0) {
            icount = icount + 1;
            t_xi[l - 1] = lev(s.temp_node, nd);
            s_xi[l - 1] = lev(s.salt_node, nd);
            ta = ta + t_xi[l - 1];
            sa = sa + s_xi[l - 1];
        }
    }
    if (icount == 0) return GOM_ELM_ALL_DRY;
    ta = ta / icount;
    sa = sa / icount;
    if (icount != tq) {
        ttint = ta;
        ssint = sa;
    } else {
        ttint = 0.0;
        ssint = 0.0;
        for (int l = 1; l <= tq; ++l) {
            ttint = ttint + t_xi[l - 1] * fin.staint[l - 1];
            ssint = ssint + s_xi[l - 1] * fin.staint[l - 1];
        }
    }
    const double ar = g.area[nnel - 1];
    int index_1 = 0;
    if (tq == 3) {
        for (int l = 1; l <= 4; ++l) {
            double aa1, aa2, aa3;
            int n1 = 0, f1 = 0, f2, f3;
            if (l <= 3) {
                n1 = g.cell_node(l, nnel);
                f2 = g.cell_face(start_end_node(tq, l, 2), nnel);
                f3 = g.cell_face(start_end_node(tq, l, 1), nnel);
                aa1 = calculate_area(xt, g.x_face[f2 - 1], g.x_face[f3 - 1], yt, g.y_face[f2 - 1], g.y_face[f3 - 1]);
                aa2 = calculate_area(g.x_node[n1 - 1], xt, g.x_face[f3 - 1], g.y_node[n1 - 1], yt, g.y_face[f3 - 1]);
                aa3 = calculate_area(g.x_node[n1 - 1], g.x_face[f2 - 1], xt, g.y_node[n1 - 1], g.y_face[f2 - 1], yt);
            } else {
                f1 = g.cell_face(1, nnel);
                f2 = g.cell_face(2, nnel);
                f3 = g.cell_face(3, nnel);
                aa1 = calculate_area(xt, g.x_face[f2 - 1], g.x_face[f3 - 1], yt, g.y_face[f2 - 1], g.y_face[f3 - 1]);
                aa2 = calculate_area(g.x_face[f1 - 1], xt, g.x_face[f3 - 1], g.y_face[f1 - 1], yt, g.y_face[f3 - 1]);
                aa3 = calculate_area(g.x_face[f1 - 1], g.x_face[f2 - 1], xt, g.y_face[f1 - 1], g.y_face[f2 - 1], yt);
            }
            const double aa = fabs(aa1) + fabs(aa2) + fabs(aa3);
            const double subrat = fabs(aa - ar / 4) * 4 / ar;
            if (subrat < 100 * small_06) {
                index_1 = 1;
                double sig[3];
                sig[0] = aa1 * 4 / ar;
                sig[1] = aa2 * 4 / ar;
                sig[0] = fmax(0.0, fmin(1.0, sig[0]));
                sig[1] = fmax(0.0, fmin(1.0, sig[1]));
                if (sig[0] + sig[1] > 1) {
                    sig[2] = 0;
                    sig[1] = 1 - sig[0];
                } else {
                    sig[2] = 1 - sig[0] - sig[1];
                }
                const bool wet = l <= 3 ? (s.top_node[n1 - 1] != 0 && s.top_face[f2 - 1] != 0 && s.top_face[f3 - 1] != 0)
                                        : (s.top_face[f1 - 1] != 0 && s.top_face[f2 - 1] != 0 && s.top_face[f3 - 1] != 0);
                if (wet) {
                    const double t0 = l <= 3 ? lev(s.temp_node, n1) : lev(s.temp_face, f1);
                    const double s0 = l <= 3 ? lev(s.salt_node, n1) : lev(s.salt_face, f1);
                    ttint = t0 * sig[0] + lev(s.temp_face, f2) * sig[1] + lev(s.temp_face, f3) * sig[2];
                    ssint = s0 * sig[0] + lev(s.salt_face, f2) * sig[1] + lev(s.salt_face, f3) * sig[2];
                    break;
                }
            }
        }
    } else {
        const double xc = g.x_cell[nnel - 1], yc = g.y_cell[nnel - 1];
        for (int l = 1; l <= 4; ++l) {
            const int n1 = g.cell_node(l, nnel);
            const int f2 = g.cell_face(start_end_node(tq, l, 3), nnel), f4 = g.cell_face(start_end_node(tq, l, 2), nnel);
            const double xn = g.x_node[n1 - 1], yn = g.y_node[n1 - 1];
            const double x2 = g.x_face[f2 - 1], y2 = g.y_face[f2 - 1], x4 = g.x_face[f4 - 1], y4 = g.y_face[f4 - 1];
            const double aa1 = calculate_area(xn, x2, xt, yn, y2, yt);
            const double aa2 = calculate_area(x2, xc, xt, y2, yc, yt);
            const double aa3 = calculate_area(xc, x4, xt, yc, y4, yt);
            const double aa4 = calculate_area(x4, xn, xt, y4, yn, yt);
            const double bb1 = calculate_area(xn, x2, x4, yn, y2, y4);
            const double bb2 = calculate_area(x2, xc, x4, y2, yc, y4);
            if (bb1 <= 0 || bb2 <= 0) return GOM_ELM_NEG_SUBELEMENT;
            const double bb = bb1 + bb2;
            const double aa = fabs(aa1) + fabs(aa2) + fabs(aa3) + fabs(aa4);
            const double subrat = fabs(aa - bb) / bb;
            if (subrat < 4.0 * small_06) {
                index_1 = 1;
                double st4[4];
                const int b = bilinear_interpolation<double>(xn, x2, xc, x4, yn, y2, yc, y4, xt, yt, st4);
                if (b) return b;
                if (s.top_node[n1 - 1] != 0 && s.top_face[f2 - 1] != 0 && s.top_face[f4 - 1] != 0) {
                    const double tx[4] = {lev(s.temp_node, n1), lev(s.temp_face, f2), ta, lev(s.temp_face, f4)};
                    const double sx[4] = {lev(s.salt_node, n1), lev(s.salt_face, f2), sa, lev(s.salt_face, f4)};
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

// :59-125, one thread per (cell, layer)
template <typename R> __global__ void k_elmtr_backtrack(Geom g, StateT<R> s, Forcing f, Params p, R *con, gom_status *st) {
    constexpr bool MIXED = sizeof(R) == sizeof(float);
    unsigned t = flat_tid();
    const int L = g.L, NC = g.NC;
    if (t >= (unsigned)NC * L) return;
    int i, k;
    split_index(t, L, i, k);
    i += 1;
    k += 1;
    const long oT = (long)(i - 1) * L + (k - 1), oS = (long)NC * L + oT;
    const int top = s.top_cell[i - 1];
    if (top == 0) {
        con[oT] = R(0);
        con[oS] = R(0);
        return;
    }
    if (k < g.bottom_cell[i - 1] || k > top) return;
    int nnel = i, jlev = k;
    const double x0 = g.x_cell[i - 1], y0 = g.y_cell[i - 1];
    double z0;
    if (k == top) z0 = s.ztop_cell[i - 1] - (double)s.dz_cell[ix(k, i, L)] * 0.5;
    else z0 = g.z_level[k] - (double)s.dz_cell[ix(k, i, L)] * 0.5;
    double u_temp = 0.0, v_temp = 0.0;
    int bt_step = 0;
    const int tq = g.tri_or_quad[i - 1];
    for (int l = 1; l <= tq; ++l) {
        const int nd = g.cell_node(l, i);
        u_temp = u_temp + ((double)s.u_node[ix0(k, nd, L)] + (double)s.u_node[ix0(k - 1, nd, L)]) * 0.5;
        v_temp = v_temp + ((double)s.v_node[ix0(k, nd, L)] + (double)s.v_node[ix0(k - 1, nd, L)]) * 0.5;
        bt_step = bt_step + s.num_sub_elm[ix(k, nd, L)];
    }
    u_temp = u_temp / tq;
    v_temp = v_temp / tq;
    bt_step = bt_step / tq;
    double uu = u_temp, vv = v_temp;
    double ww = ((double)s.wn_cell[ix0(k, i, L)] + (double)s.wn_cell[ix0(k - 1, i, L)]) * 0.5;
    double tc, sc;
    if (sqrt(uu * uu + vv * vv + ww * ww) <= F(1.e-4f)) {
        tc = s.temp_cell[ix(k, i, L)];
        sc = s.salt_cell[ix(k, i, L)];
    } else {
        const double bt_dt = (bt_step >= 1 && bt_step <= GOM_BT_TABLE) ? p.bt_dt[bt_step - 1] : p.dt / bt_step;
        int near = 0;
        ElmFinal fin;
        int e = elm_backtrace<R, MIXED>(g, s, p, bt_step, bt_dt, uu, vv, ww, x0, y0, z0, nnel, jlev, near, &fin);
        if (!e) e = elm_tracer_at_foot(g, s, f, fin, nnel, jlev, tc, sc);
        if (e) {
            record_error(st, GOM_E_ELM, e, i, k, 0.0, GOM_ENTITY_CELL);
            return;
        }
    }
    // :120 the per-layer heat source (zero unless the host's heat-balance model sets phi_sz)
    tc = tc + p.dt * f.phi_sz[ix(k, i, L)] / (p.rho_o * 4186.0 * (double)s.dz_cell[ix(k, i, L)]);
    con[oT] = (R)tc;
    con[oS] = (R)sc;
}

// :133-154, one thread per (cell, layer)
template <typename R> __global__ void k_elmtr_hdiff(Geom g, StateT<R> s, Params p, const R *con, R *rhs) {
    unsigned t = flat_tid();
    const int L = g.L, NC = g.NC;
    if (t >= (unsigned)NC * L) return;
    int i, k;
    split_index(t, L, i, k);
    i += 1;
    k += 1;
    const int top = s.top_cell[i - 1];
    if (top == 0 || k < g.bottom_cell[i - 1] || k > top) return;
    R sum1 = R(0), sum2 = R(0);
    for (int l = 1; l <= g.tri_or_quad[i - 1]; ++l) {
        const int j = g.cell_face(l, i);
        const int ie = g.face_cell(2, j);
        if (ie != 0) {
            const R rtemp1 = geo<R>(g.face_length, g.face_length_f, j - 1) * s.dz_face[ix(k, j, L)] *
                             s.kh[ix(k, j, L)] / geo<R>(g.delta_j, g.delta_j_f, j - 1);
            sum1 = sum1 + rtemp1 * (s.salt_cell[ix(k, ie, L)] - s.salt_cell[ix(k, i, L)]);
            sum2 = sum2 + rtemp1 * (s.temp_cell[ix(k, ie, L)] - s.temp_cell[ix(k, i, L)]);
        }
    }
    const R dtR = (R)p.dt, den = geo<R>(g.area, g.area_f, i - 1) * s.dz_cell[ix(k, i, L)];
    sum1 = sum1 * dtR / den;
    sum2 = sum2 * dtR / den;
    const long oT = (long)(i - 1) * L + (k - 1), oS = (long)NC * L + oT;
    rhs[oT] = con[oT] + sum1;
    rhs[oS] = con[oS] + sum2;
}

// :163-236, one thread per cell column: implicit vertical diffusion, extension below and above
template <typename R> __global__ void k_elmtr_vsolve(Geom g, StateT<R> s, Params p, const R *rhs, gom_status *st) {
    unsigned tid = flat_tid();
    if (tid >= (unsigned)g.NC) return;
    const int i = column_entity<R>(g.cell_order, tid);
    const int L = g.L, NC = g.NC;
    const int t = s.top_cell[i - 1], b = g.bottom_cell[i - 1];
    if (t == 0) return;   // dry cells keep their previous values
    const int nvl = t - b + 1;
    const R dtR = (R)p.dt;
    R am[GOM_MAXL], bm[GOM_MAXL], cm[GOM_MAXL], gm[GOM_MAXL], rr[GOM_MAXL][2];
    for (int k = b + 1; k <= t - 1; ++k) {
        const int kk = t - k + 1;
        am[kk - 1] = -dtR * s.kv[ix0(k, i, L)] / s.dzhalf_cell[ix0(k, i, L)];
        cm[kk - 1] = -dtR * s.kv[ix0(k - 1, i, L)] / s.dzhalf_cell[ix0(k - 1, i, L)];
        bm[kk - 1] = -am[kk - 1] + s.dz_cell[ix(k, i, L)] - cm[kk - 1];
    }
    if (t == b) {
        bm[0] = s.dz_cell[ix(t, i, L)];
    } else {
        cm[0] = -dtR + s.kv[ix0(t - 1, i, L)] / s.dzhalf_cell[ix0(t - 1, i, L)];
        bm[0] = s.dz_cell[ix(t, i, L)] - cm[0];
        am[nvl - 1] = -dtR * s.kv[ix0(b, i, L)] / s.dzhalf_cell[ix0(b, i, L)];
        bm[nvl - 1] = -am[nvl - 1] + s.dz_cell[ix(b, i, L)];
    }
    for (int k = 1; k <= nvl; ++k) {
        const int kk = t - k + 1;
        const long oT = (long)(i - 1) * L + (kk - 1);
        rr[k - 1][0] = s.dz_cell[ix(kk, i, L)] * rhs[oT];
        rr[k - 1][1] = s.dz_cell[ix(kk, i, L)] * rhs[(long)NC * L + oT];
    }
    if (!thomas<2>(nvl, am, bm, cm, rr, gm)) {
        record_error(st, GOM_E_ZERO_PIVOT, 210, i, 0, 0.0, GOM_ENTITY_CELL);
        return;
    }
    for (int k = 1; k <= L; ++k) {
        const int kq = k < b ? b : (k > t ? t : k);
        const int row = t + 1 - kq;
        s.temp_cell_new[ix(k, i, L)] = rr[row - 1][0];
        s.salt_cell_new[ix(k, i, L)] = rr[row - 1][1];
    }
}

// :262-330, one thread per node column: averages with the fill from above, extension of wet nodes
template <typename R> __global__ void k_elmtr_nodes(Geom g, StateT<R> s) {
    unsigned tid = flat_tid();
    if (tid >= (unsigned)g.NN) return;
    const int i = column_entity<R>(g.node_order, tid);
    const int L = g.L;
    const int tn = s.top_node[i - 1], bn = g.bottom_node[i - 1];
    if (tn == 0) return;   // dry nodes keep their previous values
    const int na = g.adj_cells_at_node[i - 1];
    for (int k = tn; k >= bn; --k) {
        R sum0 = R(0), sum1 = R(0), sum2 = R(0);
        int icount = 0;
        for (int l = 1; l <= na; ++l) {
            const int ie = g.node_cell(l, i);
            if (k >= g.bottom_cell[ie - 1] && k <= s.top_cell[ie - 1]) {
                const R ar = geo<R>(g.area, g.area_f, ie - 1), dzn = s.dz_cell_new[ix(k, ie, L)];
                sum0 = sum0 + ar * dzn;
                sum1 = sum1 + ar * dzn * s.temp_cell_new[ix(k, ie, L)];
                sum2 = sum2 + ar * dzn * s.salt_cell_new[ix(k, ie, L)];
            } else {
                icount = icount + 1;
            }
        }
        R tv, sv;
        if (sum0 == R(0)) {
            tv = R(0);
            sv = R(0);
        } else {
            tv = sum1 / sum0;
            sv = sum2 / sum0;
        }
        if (icount == na && k != tn) {
            tv = s.temp_node[ix(k + 1, i, L)];
            sv = s.salt_node[ix(k + 1, i, L)];
        }
        s.temp_node[ix(k, i, L)] = tv;
        s.salt_node[ix(k, i, L)] = sv;
    }
    for (int k = 1; k <= bn - 1; ++k) {
        s.temp_node[ix(k, i, L)] = s.temp_node[ix(bn, i, L)];
        s.salt_node[ix(k, i, L)] = s.salt_node[ix(bn, i, L)];
    }
    for (int k = tn + 1; k <= L; ++k) {
        s.temp_node[ix(k, i, L)] = s.temp_node[ix(tn, i, L)];
        s.salt_node[ix(k, i, L)] = s.salt_node[ix(tn, i, L)];
    }
}

// :332-339, one thread per (face, layer)
template <typename R> __global__ void k_elmtr_faces(Geom g, StateT<R> s) {
    unsigned t = flat_tid();
    const int L = g.L;
    if (t >= (unsigned)g.NF * L) return;
    int j, k;
    split_index(t, L, j, k);
    j += 1;
    k += 1;
    const int n1 = g.face_node(1, j), n2 = g.face_node(2, j);
    s.salt_face[t] = (s.salt_node[ix(k, n1, L)] + s.salt_node[ix(k, n2, L)]) * R(0.5);
    s.temp_face[t] = (s.temp_node[ix(k, n1, L)] + s.temp_node[ix(k, n2, L)]) * R(0.5);
}

template <typename R> __global__ void k_cell_z(Geom g, StateT<R> s, Params p);

template <typename R> cudaError_t launch_transport_elm(const LaunchT<R> &x) {
    const Geom &g = x.g;
    const long ncl = (long)g.NC * g.L;
    k_cell_z<<<blocks_for(g.NC, 256), 256, 0, x.stream>>>(g, x.s, x.p);
    k_elmtr_backtrack<<<blocks_for(ncl, 64), 64, 0, x.stream>>>(g, x.s, x.f, x.p, x.w.con, x.status);
    k_elmtr_hdiff<<<blocks_for(ncl, 256), 256, 0, x.stream>>>(g, x.s, x.p, x.w.con, x.w.con2);
    k_elmtr_vsolve<<<blocks_for(g.NC, 128), 128, 0, x.stream>>>(g, x.s, x.p, x.w.con2, x.status);
    k_elmtr_nodes<<<blocks_for(g.NN, 128), 128, 0, x.stream>>>(g, x.s);
    k_elmtr_faces<<<blocks_for((long)g.NF * g.L, 256), 256, 0, x.stream>>>(g, x.s);
    return cudaGetLastError();
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
// Per-face quantities of a momentum column, formed once per face.
template <typename R> struct MomFace {
    int j, tj, bj, nvl, node1, node2, a1, a2, btype, ibnd, tq1, tq2, ba1, ta1, ba2, ta2, bn1, tn1, bn2, tn2;
    int cn1[4], cn2[4];   // nodes of the two adjacent cells
    bool wet_nodes;
    R dtR, cordt, ctR, snR, ct2R, sn2R, bt1, along, air1, air2, bc_dj, bc_fl, djR, flR, fl2, gdt0, wsn, wst, qub,
        smag, ah0, kh0, area1, rl1, rl2, inv_tq1, inv_tq2, spin, c069, gbdt, gtdt;
};

// false for a dry face (no column)
template <typename R>
__device__ bool momentum_setup(const Geom &g, const StateT<R> &s, const Forcing &f, const Params &p, int j,
                               MomFace<R> &m) {
    const int tj = s.top_face[j - 1];
    m.j = j;
    m.tj = tj;
    if (tj == 0) return false;
    const double dt = p.dt, gravity = p.gravity, theta = p.theta;
    const R dtR = (R)dt;
    m.dtR = dtR;
    const int bj = g.bottom_face[j - 1];
    m.bj = bj;
    m.nvl = tj - bj + 1;
    const int node1 = g.face_node(1, j), node2 = g.face_node(2, j);
    const int a1 = g.face_cell(1, j), a2 = g.face_cell(2, j);
    const int btype = g.boundary_type_of_face[j - 1];
    m.node1 = node1;
    m.node2 = node2;
    m.a1 = a1;
    m.a2 = a2;
    m.btype = btype;
    const double dj = g.delta_j[j - 1], fl = g.face_length[j - 1];
    const double ct = g.cos_theta[j - 1], sn = g.sin_theta[j - 1], ct2 = g.cos_theta2[j - 1], sn2 = g.sin_theta2[j - 1];
    m.ctR = (R)ct;
    m.snR = (R)sn;
    m.ct2R = (R)ct2;
    m.sn2R = (R)sn2;
    const R ct2R = m.ct2R, sn2R = m.sn2R;
    m.cordt = (R)(g.coriolis_factor[j - 1] * dt);
    m.gbdt = s.gamma_b[j - 1] * dtR;
    m.gtdt = (R)f.gamma_t[j - 1] * dtR;
    const bool wet_nodes = s.wetdry_node[node1 - 1] == 0 && s.wetdry_node[node2 - 1] == 0;
    m.wet_nodes = wet_nodes;
    const double eta_n1 = s.eta_node[node1 - 1], eta_n2 = s.eta_node[node2 - 1];
    m.c069 = (R)F(0.69f);
    m.ibnd = g.isflowside3[j - 1];
    const double eta1 = s.eta_cell[a1 - 1];
    const double eta2 = a2 != 0 ? s.eta_cell[a2 - 1] : 0.0;
    m.ba1 = g.bottom_cell[a1 - 1];
    m.ta1 = s.top_cell[a1 - 1];
    m.ba2 = a2 != 0 ? g.bottom_cell[a2 - 1] : 0;
    m.ta2 = a2 != 0 ? s.top_cell[a2 - 1] : 0;
    m.bn1 = g.bottom_node[node1 - 1];
    m.tn1 = s.top_node[node1 - 1];
    m.bn2 = g.bottom_node[node2 - 1];
    m.tn2 = s.top_node[node2 - 1];
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
        m.bt1 = bt_rtemp1;
        m.along = (btype == 0) ? (along0 + bt_rtemp2) : along0;
        m.air1 = rt0_air * ct2R;
        m.air2 = rtemp3_air + rt0_air * sn2R;
        m.bc_dj = -(gdt / (float)p.rho_o) * inv_dj;
        m.bc_fl = -(gdt / (float)p.rho_o) * inv_fl;
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
        m.bt1 = (R)bt_rtemp1;
        m.along = (R)((btype == 0) ? (along_rtemp0 + bt_rtemp2) : along_rtemp0);
        m.air1 = (R)(rt0_air * ct2);
        m.air2 = (R)(rtemp3_air + rt0_air * sn2);
        m.bc_dj = (R)(-gravity * dt / (p.rho_o * dj));
        m.bc_fl = (R)(-gravity * dt / (p.rho_o * fl));
    }
    m.djR = (R)dj;
    m.flR = (R)fl;
    m.fl2 = (R)(fl * fl);
    m.gdt0 = (R)(gravity * dt);
    m.wsn = (R)(dt * f.wind_stress_normal[j - 1]);
    m.wst = (R)(dt * f.wind_stress_tangnt[j - 1]);
    m.qub = m.ibnd > 0 ? (R)s.qu_boundary[m.ibnd - 1] : R(0);
    m.smag = (R)p.smagorinsky;
    m.ah0 = (R)p.ah_0;
    m.kh0 = (R)p.kh_0;
    m.area1 = (R)g.area[a1 - 1];
    m.rl1 = R(0);
    m.rl2 = R(0);
    m.inv_tq1 = R(0);
    m.inv_tq2 = R(0);
    m.tq1 = 0;
    m.tq2 = 0;
    if (a2 != 0) {
        double ddx = g.x_cell[a1 - 1] - g.x_face[j - 1], ddy = g.y_cell[a1 - 1] - g.y_face[j - 1];
        double ddx2 = g.x_cell[a2 - 1] - g.x_face[j - 1], ddy2 = g.y_cell[a2 - 1] - g.y_face[j - 1];
        if constexpr (sizeof(R) == sizeof(float)) {
            m.rl1 = sqrtf((float)ddx * (float)ddx + (float)ddy * (float)ddy);
            m.rl2 = sqrtf((float)ddx2 * (float)ddx2 + (float)ddy2 * (float)ddy2);
        } else {
            m.rl1 = (R)sqrt(ddx * ddx + ddy * ddy);
            m.rl2 = (R)sqrt(ddx2 * ddx2 + ddy2 * ddy2);
        }
        m.tq1 = g.tri_or_quad[a1 - 1];
        m.tq2 = g.tri_or_quad[a2 - 1];
        m.inv_tq1 = m.tq1 == 4 ? R(0.25) : R(0);   // x/4 == x*0.25 exactly; triangles divide
        m.inv_tq2 = m.tq2 == 4 ? R(0.25) : R(0);
#pragma unroll
        for (int ll = 1; ll <= 4; ++ll) {
            m.cn1[ll - 1] = ll <= m.tq1 ? g.cell_node(ll, a1) : 0;
            m.cn2[ll - 1] = ll <= m.tq2 ? g.cell_node(ll, a2) : 0;
        }
    }
    m.spin = (R)f.scal[2];
    return true;
}

// :120-169, row r (0 = top) of the column's tridiagonal matrix
template <typename R>
__device__ __forceinline__ void momentum_matrix_row(const StateT<R> &s, const MomFace<R> &m, int L, int r, R &a,
                                                    R &bd, R &cu) {
    const int j = m.j, tj = m.tj, bj = m.bj;
    if (m.nvl == 1) {
        bd = s.dz_face[ix(tj, j, L)] + m.gbdt;
    } else if (r == 0) {
        cu = -m.dtR * s.av[ix0(tj - 1, j, L)] / s.dzhalf_face[ix0(tj - 1, j, L)];
        bd = m.gtdt + s.dz_face[ix(tj, j, L)] - cu;
    } else if (r == m.nvl - 1) {
        a = -m.dtR * s.av[ix0(bj, j, L)] / s.dzhalf_face[ix0(bj, j, L)];
        bd = -a + s.dz_face[ix(bj, j, L)] + m.gbdt;
    } else {
        const int k = tj - r;
        a = -m.dtR * s.av[ix0(k, j, L)] / s.dzhalf_face[ix0(k, j, L)];
        cu = -m.dtR * s.av[ix0(k - 1, j, L)] / s.dzhalf_face[ix0(k - 1, j, L)];
        bd = -a + s.dz_face[ix(k, j, L)] - cu;
    }
}

// :254-551, right-hand sides of top-down row k (1-based; layer tj - k + 1); writes Kh of the row
template <typename R>
__device__ __forceinline__ void momentum_row(const Geom &g, const StateT<R> &s, const Params &p, const MomFace<R> &m,
                                             int L, int k, R &G1o, R &G2o, R &dzo) {
    const int j = m.j, tj = m.tj;
    const int kk = tj - k + 1;
    const R half = R(0.5);
    const R ctR = m.ctR, snR = m.snR;
    const R dtR = m.dtR, cordt = m.cordt;
    R dzk = s.dz_face[ix(kk, j, L)];
    R unk = s.un_face[ix(kk, j, L)], vnk = s.vn_face[ix(kk, j, L)];
    R G1 = dzk * (s.un_elm[ix(kk, j, L)] + cordt * vnk);
    R G2 = dzk * (s.vn_elm[ix(kk, j, L)] - cordt * unk);
    if (m.a2 != 0) {
        // :269-344 Smagorinsky horizontal diffusion
        R tmp[12];
        for (int l = 1; l <= 2; ++l) {
            int nd = l == 1 ? m.node1 : m.node2;
            R ut = (s.u_node[ix0(kk, nd, L)] + s.u_node[ix0(kk - 1, nd, L)]) * half;
            R vt = (s.v_node[ix0(kk, nd, L)] + s.v_node[ix0(kk - 1, nd, L)]) * half;
            tmp[2 * l - 2] = ut * ctR + vt * snR;
            tmp[2 * l - 1] = -ut * snR + vt * ctR;
        }
        for (int l = 1; l <= 2; ++l) {
            int tq = l == 1 ? m.tq1 : m.tq2;
            R itq = l == 1 ? m.inv_tq1 : m.inv_tq2;
            R ut = R(0), vt = R(0);
#pragma unroll
            for (int ll = 1; ll <= 4; ++ll) {
                if (ll > tq) break;
                int nd = l == 1 ? m.cn1[ll - 1] : m.cn2[ll - 1];
                R uu = (s.u_node[ix0(kk, nd, L)] + s.u_node[ix0(kk - 1, nd, L)]) * half;
                R vv = (s.v_node[ix0(kk, nd, L)] + s.v_node[ix0(kk - 1, nd, L)]) * half;
                ut = ut + (itq != R(0) ? uu * itq : uu / (R)tq);
                vt = vt + (itq != R(0) ? vv * itq : vv / (R)tq);
            }
            tmp[2 * l + 2] = ut * ctR + vt * snR;
            tmp[2 * l + 3] = -ut * snR + vt * ctR;
        }
        R dudx = (tmp[6] - tmp[4]) / m.djR;
        R dvdx = (tmp[7] - tmp[5]) / m.djR;
        R dudy = (tmp[2] - tmp[0]) / m.flR;
        R dvdy = (tmp[3] - tmp[1]) / m.flR;
        R sdd = dvdx + dudy;
        R hdiff = m.smag * sqrt(dudx * dudx + dvdy * dvdy + half * (sdd * sdd));
        R khv = hdiff * m.area1;
        hdiff = hdiff + m.ah0;
        s.kh[ix(k, j, L)] = khv + m.kh0;
        R d2udy = R(4) * (tmp[2] + tmp[0] - R(2) * unk) / m.fl2;
        R d2vdy = R(4) * (tmp[3] + tmp[1] - R(2) * vnk) / m.fl2;
        tmp[8] = (tmp[4] - unk) / m.rl1;
        tmp[9] = (tmp[5] - vnk) / m.rl1;
        tmp[10] = (tmp[6] - unk) / m.rl2;
        tmp[11] = (tmp[7] - vnk) / m.rl2;
        R d2udx = R(2) * (tmp[8] + tmp[10]) / m.djR;
        R d2vdx = R(2) * (tmp[9] + tmp[11]) / m.djR;
        G1 = G1 + dzk * dtR * hdiff * (d2udx + d2udy);
        G2 = G2 + dzk * dtR * hdiff * (d2vdx + d2vdy);
    }
    // :350-397 barotropic gradients at (1-theta)
    if (m.btype >= 0) G1 = G1 - dzk * m.bt1;
    else G1 = R(0);
    if (m.wet_nodes) G2 = G2 - dzk * m.along;
    // :400-471 baroclinic pressure gradient (density differences formed in FP64)
    if (p.baroclinic_flag == 1) {
        R sum1 = R(0), sum2 = R(0);
        for (int k2 = kk; k2 <= tj; ++k2) {
            R dz2 = s.dz_face[ix(k2, j, L)];
            if (m.a2 != 0 && k2 >= m.ba1 && k2 <= m.ta1 && k2 >= m.ba2 && k2 <= m.ta2) {
                R dr = (R)(s.rho_cell[ix(k2, m.a2, L)] - s.rho_cell[ix(k2, m.a1, L)]);
                sum1 = sum1 + (k2 == kk ? half * dr : dr) * dz2;
            }
            if (k2 >= m.bn1 && k2 <= m.tn1 && k2 >= m.bn2 && k2 <= m.tn2) {
                R dr = (R)(s.rho_node[ix(k2, m.node2, L)] - s.rho_node[ix(k2, m.node1, L)]);
                sum2 = sum2 + (k2 == kk ? half * dr : dr) * dz2;
            }
        }
        R dzrow = s.dz_face[ix(k, j, L)];   // the reference uses the top-down row here
        R rtemp1 = dzrow * m.bc_dj * sum1;
        R rtemp2 = dzrow * m.bc_fl * sum2;
        R rtemp3 = rtemp1 * m.ct2R;
        R rtemp4 = rtemp1 * m.sn2R;
        G1 = G1 + rtemp3 * m.spin;
        G2 = G2 + (rtemp2 + rtemp4) * m.spin;
    }
    if (k == 1) {
        G1 = G1 + m.wsn;
        G2 = G2 + m.wst;
    }
    // :485-486 tide-generating potential, zero in this build (kept for the signed-zero result)
    G1 = G1 + m.c069 * dzk * m.gdt0 * R(0);
    G2 = G2 + m.c069 * dzk * m.gdt0 * R(0);
    // :490-509 air pressure
    G1 = G1 + dzk * m.air1;
    G2 = G2 + dzk * m.air2;
    if (m.btype == -1) G1 = R(0);
    if (m.ibnd > 0) G1 = G1 + dzk * m.qub;
    G1o = G1;
    G2o = G2;
    dzo = dzk;
}

// SH: the elimination factors and partial solutions in dynamic shared memory, entry (q, r) of
// thread t at (q L + r) blockDim + t (q = 0 factor, 1..3 solutions), instead of per-thread
// local arrays that the resident columns push out of L1 (same operations, same results)
template <typename R, bool SH = false>
__global__ void __launch_bounds__(256) k_momentum(Geom g, StateT<R> s, Forcing f, Params p, gom_status *st) {
    unsigned tid = flat_tid();
    if (tid >= (unsigned)g.NF) return;
    const int j = column_entity<R>(g.face_order, tid);
    const int L = g.L;
    MomFace<R> m;
    if (!momentum_setup(g, s, f, p, j, m)) return;
    const int nvl = m.nvl;
    // thomas<3> with each row's matrix entries and right-hand sides formed as its forward
    // elimination step reaches it (the same operations in the same order; only the elimination
    // factors and partial solutions are kept)
    extern __shared__ __align__(16) unsigned char mom_smem[];
    R *const shm = reinterpret_cast<R *>(mom_smem) + threadIdx.x;
    const int bs = blockDim.x;
    R gam_l[SH ? 1 : GOM_MAXL], sol_l[SH ? 1 : GOM_MAXL][3];
    auto gam = [&](int r) -> R & {
        if constexpr (SH) return shm[r * bs];
        else return gam_l[r];
    };
    auto sol = [&](int r, int c) -> R & {
        if constexpr (SH) return shm[((c + 1) * L + r) * bs];
        else return sol_l[r][c];
    };
    R den = R(0), cu_prev = R(0);
    for (int r = 0; r < nvl; ++r) {
        R a_r = R(0), bd_r = R(0), cu_r = R(0), g1, g2, dzr;
        momentum_matrix_row(s, m, L, r, a_r, bd_r, cu_r);
        momentum_row(g, s, p, m, L, r + 1, g1, g2, dzr);
        if (r == 0) {
            if (bd_r == R(0)) {
                record_error(st, GOM_E_ZERO_PIVOT, 587, j, 0, 0.0, GOM_ENTITY_FACE);
                return;
            }
            den = bd_r;
            sol(0, 0) = g1 / den;
            sol(0, 1) = g2 / den;
            sol(0, 2) = dzr / den;
        } else {
            const R gr = cu_prev / den;
            gam(r) = gr;
            den = bd_r - a_r * gr;
            if (den == R(0)) {
                record_error(st, GOM_E_ZERO_PIVOT, 587, j, 0, 0.0, GOM_ENTITY_FACE);
                return;
            }
            sol(r, 0) = (g1 - a_r * sol(r - 1, 0)) / den;
            sol(r, 1) = (g2 - a_r * sol(r - 1, 1)) / den;
            sol(r, 2) = (dzr - a_r * sol(r - 1, 2)) / den;
        }
        cu_prev = cu_r;
    }
    for (int r = nvl - 2; r >= 0; --r) {
        const R gn = gam(r + 1);
        sol(r, 0) = sol(r, 0) - gn * sol(r + 1, 0);
        sol(r, 1) = sol(r, 1) - gn * sol(r + 1, 1);
        sol(r, 2) = sol(r, 2) - gn * sol(r + 1, 2);
    }
    const bool zero_g1 = (m.btype == -1 && m.ibnd == 0);
    const bool zero_dz1 = (m.btype == -1);
    for (int k = 1; k <= L; ++k) {
        long o = ix(k, j, L);
        if (k <= nvl) {
            s.ainvg1[o] = zero_g1 ? R(0) : sol(k - 1, 0);
            s.ainvg2[o] = sol(k - 1, 1);
            s.ainvdz1[o] = zero_dz1 ? R(0) : sol(k - 1, 2);
            s.ainvdz2[o] = sol(k - 1, 2);
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

// variants: one thread per column with 128 / 64 / 256 threads per block (local arrays), or 3:
// the shared-memory form with the largest of 64 / 32 threads whose 4 L entries per thread fit
// in 48 KB (the local form where none does)
template <typename R> cudaError_t launch_momentum_columns_only(const LaunchT<R> &x) {
    const int v = x.tune[TUNE_MOMENTUM];
    if (v == 3) {
        const size_t per_thread = 4 * (size_t)x.g.L * sizeof(R);
        for (int bs : {64, 32}) {
            const size_t smem = per_thread * bs;
            if (smem > 48 * 1024) continue;
            k_momentum<R, true><<<blocks_for(x.g.NF, bs), bs, smem, x.stream>>>(x.g, x.s, x.f, x.p, x.status);
            return cudaGetLastError();
        }
    }
    const int bs = v == 1 ? 64 : v == 2 ? 256 : 128;
    k_momentum<R, false><<<blocks_for(x.g.NF, bs), bs, 0, x.stream>>>(x.g, x.s, x.f, x.p, x.status);
    return cudaGetLastError();
}

template <typename R> cudaError_t launch_momentum(const LaunchT<R> &x) {
    long nfl = (long)x.g.NF * x.g.L;
    k_zero_face_columns<<<blocks_for(nfl, 256), 256, 0, x.stream>>>(x.g, x.s);
    return launch_momentum_columns_only(x);
}

GOM_INSTANTIATE_LAUNCH(launch_bottom_friction)
GOM_INSTANTIATE_LAUNCH(launch_boundary_velocity)
GOM_INSTANTIATE_LAUNCH(launch_advection)
GOM_INSTANTIATE_LAUNCH(launch_momentum)
GOM_INSTANTIATE_LAUNCH(launch_elm_walk_only)
GOM_INSTANTIATE_LAUNCH(launch_momentum_columns_only)
GOM_INSTANTIATE_LAUNCH(launch_transport_elm)

}  // namespace gom
