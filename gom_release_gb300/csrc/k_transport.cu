// k_transport.cu -- TVD salinity/temperature transport with flux limiter and implicit vertical
// diffusion, node/face tracer averages, equation of state and conservation sums, for sm_103a.
//
// References (GOM_Rv1.1.0/source):
//   solve_transport_equation_v19.f90:7-1482, calculate_density_full.f90:13-246,
//   calculate_density_linear.f90:10-140, check_conservation.f90:28-57 (specification).
//
// The reference's automatic work arrays are read in places where the call never assigned them
// (face layers outside a face's wet range, Q_ik_theta at the bottom and top interfaces); those
// reads are defined here as 0, i.e. no flux, exactly like the CPU restatement.
#include "gom_launch.h"
#include "gom_scan.cuh"

namespace gom {

// con (0:L+1, NC, ntr): element (k, i, tracer t) with t = 0 (first active tracer), 1
__device__ __forceinline__ long ic(int k, int i, int t, int L, int NC) {
    return ((long)t * NC + (i - 1)) * (L + 2) + k;
}

// exact shortcuts (identical IEEE results, fewer FP64 instructions):
//   q * sign with sign = +-1            -> sign flip
//   |0.5*(q + |q|)|, |0.5*(q - |q|)|    -> positive / negative part selected with integer tests
//   x / Nt with Nt a power of two       -> x * (1/Nt)
__device__ __forceinline__ bool is_pos(double q) { return __double_as_longlong(q) > 0; }
__device__ __forceinline__ bool is_neg(double q) {
    long long b = __double_as_longlong(q);
    return b < 0 && b != (long long)0x8000000000000000ull;
}
__device__ __forceinline__ double pos_part(double q) { return is_pos(q) ? q : 0.0; }
__device__ __forceinline__ double neg_part(double q) { return is_neg(q) ? -q : 0.0; }
__device__ __forceinline__ bool same_bits(double a, double b) { return __double_as_longlong(a) == __double_as_longlong(b); }
__device__ __forceinline__ bool is_pos(float q) { return __float_as_int(q) > 0; }
__device__ __forceinline__ bool is_neg(float q) {
    int b = __float_as_int(q);
    return b < 0 && b != (int)0x80000000u;
}
__device__ __forceinline__ float pos_part(float q) { return is_pos(q) ? q : 0.0f; }
__device__ __forceinline__ float neg_part(float q) { return is_neg(q) ? -q : 0.0f; }
__device__ __forceinline__ bool same_bits(float a, float b) { return __float_as_int(a) == __float_as_int(b); }
template <typename R> __device__ __forceinline__ R flip(R q, int sgn) { return sgn > 0 ? q : -q; }

// R: storage and arithmetic type of the tracers and coefficients
template <typename R> struct TArgs {
    Geom g;
    StateT<R> s;
    Forcing f;
    Params p;
    WorkT<R> w;
    gom_status *st;
    int ntr;          // active tracers
    int tid[2];       // tran_id of each slot: 1 salinity, 2 temperature
    int Nt, sub;      // subcycles, current subcycle
    R sub_r, sub1_r;  // sub and sub + 1 as R (the conversion done once, not per thread)
    R dt2;
    R inv_nt;         // 1/Nt, used only when Nt is a power of two (exact)
    R theta, om_theta;  // theta and 1 - theta
    bool pow2;
    bool changed_only;  // coefficient kernels: refresh only entries whose thickness changes
    const R *con;       // current concentrations
    R *con_new;         // next concentrations (full columns, zero outside the wet range)
};

template <typename R> __device__ __forceinline__ R divnt(R x, const TArgs<R> &a) {
    return a.pow2 ? x * a.inv_nt : x / (R)a.Nt;
}

// :1294-1300 assigns con_cell_new only for a solution in [0, 50] or outside it, so a NaN solution
// leaves the previous subcycle's value, which the copy-back of :1352-1357 also put into con
// (the current concentrations), and on the first subcycle the 0 of :80
template <typename R> __device__ __forceinline__ R nan_keep(const TArgs<R> &a, int k, int i, int tr) {
    return a.sub == 0 ? R(0) : a.con[ic(k, i, tr, a.g.L, a.g.NC)];
}

// Margin of the exact quotient filters below: far larger than one rounding of R, far smaller
// than any value the limiter distinguishes.
template <typename R> __device__ __forceinline__ R filter_margin();
template <> __device__ __forceinline__ double filter_margin<double>() { return 1e-9; }
template <> __device__ __forceinline__ float filter_margin<float>() { return 1e-5f; }

// fmin(1, 2 D / |Q|) for Q != 0, the quotient formed only when it can be below 1
template <typename R> __device__ __forceinline__ R diffusive_share(R D, R Q) {
    const R aq = fabs(Q);
    if (gt_nonneg(R(2) * D, aq * (R(1) + filter_margin<R>()))) return R(1);   // aq > 0 or NaN
    return fmin(R(1), R(2) * D / aq);
}

// :88-173 load tracers into con (0:L+1) with the heat_option 1 per-layer source or the heat_option 2
// surface term
template <typename R> __global__ void k_tr_load(TArgs<R> a) {
    unsigned t = flat_tid();
    const Geom &g = a.g;
    const int L = g.L;
    if (t >= (unsigned)g.NC * (L + 2)) return;
    int i, k;
    split_index(t, L + 2, i, k);
    i += 1;
    for (int tr = 0; tr < a.ntr; ++tr) {
        R v = R(0);
        if (k >= 1 && k <= L) {
            v = a.tid[tr] == 1 ? a.s.salt_cell[ix(k, i, L)] : a.s.temp_cell[ix(k, i, L)];
            if (a.tid[tr] == 2 && a.p.heat_option == 2) {
                int tl = a.s.top_cell[i - 1];
                if (tl > 0)
                    v = v + (R)(a.p.dt * a.f.phi_sw[i - 1]) / ((R)(a.p.rho_o * 4186.0) * a.s.dz_cell[ix(tl, i, L)]);
            } else if (a.tid[tr] == 2 && a.p.heat_option == 1) {
                // :109-131 the per-layer source over the wet layers
                if (k >= a.g.bottom_cell[i - 1] && k <= a.s.top_cell[i - 1])
                    v = v + (R)(a.p.dt * a.f.phi_sz[ix(k, i, L)]) / ((R)(a.p.rho_o * 4186.0) * a.s.dz_cell[ix(k, i, L)]);
            }
        }
        ((R *)a.con)[ic(k, i, tr, L, g.NC)] = v;
    }
}

// :232-397 boundary concentrations of the open-boundary and river cells for this subcycle
template <typename R> __global__ void k_tr_bc(TArgs<R> a) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    const Geom &g = a.g;
    const int L = g.L;
    if (t < g.NOB) {
        int i = t + 1;
        int i2 = g.ob_cell_id[i - 1];
        int tl = a.s.top_cell[i2 - 1], b = g.bottom_cell[i2 - 1];
        for (int k = 1; k <= L; ++k)
            for (int tr = 0; tr < a.ntr; ++tr) a.w.obk[((long)tr * g.NOB + i - 1) * L + k - 1] = R(0);
        int tq = g.tri_or_quad[i2 - 1];
        for (int l = 1; l <= tq; ++l) {
            int j2 = g.cell_face(l, i2);
            if (g.boundary_type_of_face[j2 - 1] <= 0) continue;
            int sg = g.cell_sign(l, i2);
            for (int k = b; k <= tl; ++k) {
                R dzf = a.s.dz_face[ix(k, j2, L)];
                R dz_old = dzf + divnt((a.s.dz_face_new[ix(k, j2, L)] - dzf) * a.sub_r, a);
                R q2 = (R)g.face_length[j2 - 1] * dz_old *
                       (flip(a.om_theta * a.s.un_face[ix(k, j2, L)], sg) + flip(a.theta * a.s.un_face_new[ix(k, j2, L)], sg));
                for (int tr = 0; tr < a.ntr; ++tr) {
                    R bc = (R)a.f.con_at_ob[((long)a.sub * 2 + (a.tid[tr] - 1)) * g.NOB + (i - 1)];
                    a.w.obk[((long)tr * g.NOB + i - 1) * L + k - 1] =
                        !is_pos(q2) ? bc : a.con[ic(k, i2, tr, L, g.NC)];
                }
            }
        }
    } else if (t < g.NOB + g.NQB) {
        int i = t - g.NOB + 1;
        int i2 = g.qb_cell[i - 1];
        int tl = a.s.top_cell[i2 - 1], b = g.bottom_cell[i2 - 1];
        for (int k = 1; k <= L; ++k)
            for (int tr = 0; tr < a.ntr; ++tr) {
                R v = R(0);
                if (k >= b && k <= tl) v = (R)a.f.con_at_qb[((long)a.sub * 2 + (a.tid[tr] - 1)) * g.NQB + (i - 1)];
                a.w.qbk[((long)tr * g.NQB + i - 1) * L + k - 1] = v;
            }
    }
}

// :551-581 face coefficients.  One thread per face walks its wet layers, so the FP64 work of a
// warp is spread over 32 wet faces (GB300 issues an FP64 warp instruction at the same cost however
// few lanes are active).  Later subcycles refresh only layers whose thickness changes.
template <typename R> __device__ __forceinline__ void face_coef_at(const TArgs<R> &a, int j, int k, long t) {
    R dzf = a.s.dz_face[t];
    R dz_old = dzf + divnt((a.s.dz_face_new[t] - dzf) * a.sub_r, a);
    R fl = geo<R>(a.g.face_length, a.g.face_length_f, j - 1);
    R Q = fl * dz_old * (a.om_theta * a.s.un_face[t] + a.theta * a.s.un_face_new[t]);
    R D = fl * dz_old * a.s.kh[t] / geo<R>(a.g.delta_j, a.g.delta_j_f, j - 1);
    R d = fmax(R(0), D - R(0.5) * fabs(Q));
    R phi = is_zero(Q) ? R(1) : diffusive_share(D, Q);
    a.w.qj[t] = Q;
    a.w.dj[t] = d;
    a.w.phij[t] = phi;
}

template <typename R> __global__ void k_tr_face_coef(TArgs<R> a) {
    unsigned tid = flat_tid();
    const Geom &g = a.g;
    if (tid >= (unsigned)g.NF) return;
    int j = g.face_order[tid];
    const int L = g.L;
    int b = g.bottom_face[j - 1], tf = a.s.top_face[j - 1];
    if (!a.changed_only) {
        for (int k = 1; k <= L; ++k) {
            long t = ix(k, j, L);
            if (k >= b && k <= tf) {
                face_coef_at(a, j, k, t);
            } else {
                a.w.qj[t] = R(0);
                a.w.dj[t] = R(0);
                a.w.phij[t] = R(0);
            }
        }
        return;
    }
    for (int k = b; k <= tf; ++k) {
        long t = ix(k, j, L);
        if (!same_bits(a.s.dz_face[t], a.s.dz_face_new[t])) face_coef_at(a, j, k, t);
    }
}

// :585-610 vertical coefficients, one thread per cell column (interfaces b..t-1)
template <typename R> __device__ __forceinline__ void cell_coef_at(const TArgs<R> &a, int i, long t) {
    R ar = geo<R>(a.g.area, a.g.area_f, i - 1);
    R Q = ar * (a.om_theta * a.s.wn_cell[t] + a.theta * a.s.wn_cell_new[t]);
    R dzh = a.s.dzhalf_cell[t];
    R dz_old = dzh + divnt((a.s.dzhalf_cell_new[t] - dzh) * a.sub_r, a);
    R D = ar * a.s.kv[t] / dz_old;
    a.w.qi[t] = Q;
    a.w.di[t] = fmax(R(0), D - R(0.5) * fabs(Q));
    a.w.phii[t] = is_zero(Q) ? R(1) : diffusive_share(D, Q);
}

template <typename R> __global__ void k_tr_cell_coef(TArgs<R> a) {
    unsigned tid = flat_tid();
    const Geom &g = a.g;
    if (tid >= (unsigned)g.NC) return;
    int i = g.cell_order[tid];
    const int L = g.L;
    int b = g.bottom_cell[i - 1], tl = a.s.top_cell[i - 1];
    if (!a.changed_only) {
        for (int k = 0; k <= L; ++k) {
            long t = ix0(k, i, L);
            if (k >= b && k <= tl - 1) {
                cell_coef_at(a, i, t);
            } else {
                a.w.qi[t] = R(0);
                a.w.di[t] = R(0);
                a.w.phii[t] = R(0);
            }
        }
        return;
    }
    for (int k = b; k <= tl - 1; ++k) {
        long t = ix0(k, i, L);
        if (!same_bits(a.s.dzhalf_cell[t], a.s.dzhalf_cell_new[t])) cell_coef_at(a, i, t);
    }
}

__device__ __forceinline__ bool face_open(const Geom &g, int j) {
    return g.boundary_type_of_face[j - 1] != -1 || g.isflowside3[j - 1] > 0;
}

// boundary concentration seen through a boundary face of cell i at layer k
template <typename R> __device__ __forceinline__ R oqb_value(const TArgs<R> &a, int i, int k, int tr) {
    const Geom &g = a.g;
    int ith_qb = g.qb_element_flag[i - 1];
    if (ith_qb > 0) return a.w.qbk[((long)tr * g.NQB + ith_qb - 1) * g.L + k - 1];
    int ith_ob = g.ob_element_flag[i - 1];
    if (ith_ob > 0) return a.w.obk[((long)tr * g.NOB + ith_ob - 1) * g.L + k - 1];
    return R(0);
}

template <typename R> __device__ __forceinline__ R phi_limit(int code, R small_phi, R r) {
    switch (code) {
    case 1: return fmax(small_phi, fmin(R(1), r)) - small_phi;
    case 2: return fmax(small_phi, (r + fabs(r)) / (R(1) + fabs(r))) - small_phi;
    case 3: return fmax(fmax(small_phi, fmin(R(1), R(2) * r)), fmin(R(2), r)) - small_phi;
    default: return R(0);
    }
}

// phi_limit(code, small_phi, r) with r = num / den (r = 1 when den = 0, as the reference sets
// it): where the ratio lies clearly below 0, below small_phi, or above the limiter's flat top
// (1 for codes 1 and 2... 2 for code 3), the result is known without the division and equals
// the reference's bit for bit; the quotient is formed only in between.
// NaN tests on the bit patterns (integer pipe): a NaN concentration (the heat_option 2 term over
// a layer of zero old thickness) reaches the limiter sums, and the sign and size filters below
// are exact only for numbers; with a NaN operand the ratio is formed, as the reference forms it

template <typename R> __device__ __forceinline__ R limited_ratio(int code, R small_phi, R num, R den) {
    if (is_zero(den)) return phi_limit(code, small_phi, R(1));
    if (code >= 1 && code <= 3 && !is_zero(num) && !nan_bits(num) && !nan_bits(den)) {
        const R m = filter_margin<R>();
        // num, den: numbers, neither zero, so a sign bit is the sign of the value
        if ((fbits(num) ^ fbits(den)) < 0) return R(0);   // r < 0: every code gives small_phi - small_phi
        const R an = fabs(num), ad = fabs(den);           // > 0; the bounds below are > 0 or +0
        if (code == 1 && gt_nonneg(an, ad * (R(1) + m))) return fmax(small_phi, R(1)) - small_phi;
        if (code == 3 && gt_nonneg(an, R(2) * ad * (R(1) + m))) return fmax(fmax(small_phi, R(1)), R(2)) - small_phi;
        if ((code == 1 || code == 3) && pos_finite_or_inf(small_phi) && lt_of_nonneg(an, small_phi * ad * (R(1) - m)) &&
            (code == 1 || lt_of_nonneg(an, R(0.5) * small_phi * ad * (R(1) - m))))
            return R(0);
    }
    return phi_limit(code, small_phi, num / den);
}

// :624-871 per cell column: upwind-weighted differences of every layer (sum1_all, sum2_all) for
// the face ratios r_jk, and the vertical ratios r_ik -> PSI_ik.
template <typename R> __device__ void limiter_column(const TArgs<R> &a, int i) {
    const Geom &g = a.g;
    const int L = g.L, NC = g.NC;
    int tl = a.s.top_cell[i - 1], b = g.bottom_cell[i - 1];
    if (tl == 0) return;
    int nvl = tl - b + 1;
    int tq = g.tri_or_quad[i - 1];
    int fj[4] = {0, 0, 0, 0}, nb[4] = {0, 0, 0, 0}, sg[4] = {0, 0, 0, 0};
    bool open[4] = {false, false, false, false};
#pragma unroll
    for (int l = 0; l < 4; ++l) {   // unrolled: the face arrays stay in registers
        if (l >= tq) break;
        fj[l] = g.cell_face(l + 1, i);
        nb[l] = g.cell_adj(l + 1, i);
        sg[l] = g.cell_sign(l + 1, i);
        open[l] = face_open(g, fj[l]);
    }
    R last1[2] = {R(0.0), R(0.0)}, last2[2] = {R(0.0), R(0.0)};
    for (int k = b; k <= tl; ++k) {
        R s1a[2] = {R(0.0), R(0.0)}, s2a[2] = {R(0.0), R(0.0)}, s1[2] = {R(0.0), R(0.0)}, s2[2] = {R(0.0), R(0.0)};
        // every operand of the layer is loaded before any is used: the neighbours' concentrations
        // whatever the sign of their flux (the selection below reads only those of inflow faces),
        // so the loads of a layer overlap instead of waiting on the flux test
        R ckv[2] = {R(0), R(0)}, cdn[2] = {R(0), R(0)}, cup[2] = {R(0), R(0)}, cnb[4][2], q2v[4];
        const R qlo = k > b ? a.w.qi[ix0(k - 1, i, L)] : R(0), qhi = k < tl ? a.w.qi[ix0(k, i, L)] : R(0);
#pragma unroll
        for (int tr = 0; tr < 2; ++tr) {
            if (tr >= a.ntr) break;
            ckv[tr] = a.con[ic(k, i, tr, L, NC)];
            if (k > b) cdn[tr] = a.con[ic(k - 1, i, tr, L, NC)];
            if (k < tl) cup[tr] = a.con[ic(k + 1, i, tr, L, NC)];
        }
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            q2v[l] = R(0);
            cnb[l][0] = cnb[l][1] = R(0);
            if (l < tq && open[l]) {
                q2v[l] = flip(a.w.qj[ix(k, fj[l], L)], sg[l]);
#pragma unroll
                for (int tr = 0; tr < 2; ++tr)
                    if (tr < a.ntr) cnb[l][tr] = nb[l] > 0 ? a.con[ic(k, nb[l], tr, L, NC)] : oqb_value(a, i, k, tr);
            }
        }
#pragma unroll
        for (int tr = 0; tr < 2; ++tr) {
            if (tr >= a.ntr) break;
            R ck = ckv[tr];
            if (nvl != 1) {
                if (k == b) {
                    R rt2 = pos_part(qhi);
                    s1a[tr] = rt2 * (ck - cup[tr]);
                    s2a[tr] = rt2;
                } else if (k == tl) {
                    R rt1 = pos_part(qlo);
                    s1a[tr] = rt1 * (ck - cdn[tr]);
                    s2a[tr] = rt1;
                } else {
                    R rt1 = pos_part(qlo);
                    R rt2 = pos_part(qhi);
                    s1a[tr] = rt1 * (ck - cdn[tr]) + rt2 * (ck - cup[tr]);
                    s2a[tr] = rt1 + rt2;
                }
            }
        }
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            if (l >= tq || !open[l]) continue;
            R q2 = q2v[l];
            if (is_neg(q2)) {
#pragma unroll
                for (int tr = 0; tr < 2; ++tr) {
                    if (tr >= a.ntr) break;
                    s1[tr] = s1[tr] + fabs(q2) * (ckv[tr] - cnb[l][tr]);
                    s2[tr] = s2[tr] + fabs(q2);
                }
            }
        }
#pragma unroll
        for (int tr = 0; tr < 2; ++tr) {
            if (tr >= a.ntr) break;
            s1a[tr] = s1a[tr] + s1[tr];
            s2a[tr] = s2a[tr] + s2[tr];
            a.w.sa1[((long)tr * NC + i - 1) * L + k - 1] = s1a[tr];
            a.w.sa2[((long)tr * NC + i - 1) * L + k - 1] = s2a[tr];
            last1[tr] = s1[tr];
            last2[tr] = s2[tr];
        }
    }
    // :806-840 (Q_ik_theta at the top interface is never assigned: 0 -> first branch)
#pragma unroll
    for (int tr = 0; tr < 2; ++tr) {
        if (tr >= a.ntr) break;
        R *psi = a.w.psii + (long)tr * NC * (L + 1);
        for (int k = b; k <= tl - 1; ++k) {
            R qm = (k - 1 >= b) ? a.w.qi[ix0(k - 1, i, L)] : R(0.0);
            R ck = a.con[ic(k, i, tr, L, NC)];
            R rt1 = last1[tr] + fabs(qm) * (ck - a.con[ic(k - 1, i, tr, L, NC)]);
            R rt2 = last2[tr] + fabs(qm);
            R rtemp = (a.con[ic(k + 1, i, tr, L, NC)] - ck) * rt2;
            psi[ix0(k, i, L)] = limited_ratio(a.p.h_flux_limiter, a.w.phii[ix0(k, i, L)], rt1, rtemp);
        }
    }
}

template <typename R> __global__ void k_tr_limiter_cells(TArgs<R> a) {
    unsigned tid = flat_tid();
    if (tid >= (unsigned)a.g.NC) return;
    limiter_column(a, a.g.cell_order[tid]);
}

// ---------------------------------------------------------------------------- wet cell-layer list
// The mixed path walks the wet (cell, layer) pairs of the step from a compact list (gom_scan.cuh)
// rebuilt after the layer update: every lane of every warp then works on a wet layer.
struct CellWetRange {
    const int *top, *bottom;
    __device__ int2 operator()(int i) const {
        const int t = top[i];
        return make_int2(bottom[i], t > 0 ? t : 0);
    }
};

cudaError_t build_cell_layer_list(const Geom &g, const int *top, int *off, int *bsum, int *list, int *count,
                                  cudaStream_t stream) {
    return build_layer_list(g.NC, CellWetRange{top, g.bottom_cell}, off, bsum, list, count, stream);
}

// :624-805 with one thread per (cell, layer): the upwind-weighted differences of the layer, and the
// top layer's horizontal sums kept for the vertical ratios.  Same expressions and order as
// limiter_column, so the FP64 list form gives the column form's results bit for bit.
template <typename R> __device__ __forceinline__ void tr_sums_at(const TArgs<R> &a, int i, int k) {
    const Geom &g = a.g;
    const int L = g.L, NC = g.NC;
    const int tl = a.s.top_cell[i - 1], b = g.bottom_cell[i - 1];
    const int nvl = tl - b + 1;
    const int tq = g.tri_or_quad[i - 1];
    R ck[2] = {R(0), R(0)}, s1a[2] = {R(0), R(0)}, s2a[2] = {R(0), R(0)}, s1[2] = {R(0), R(0)},
      s2[2] = {R(0), R(0)};
    for (int tr = 0; tr < a.ntr; ++tr) {
        ck[tr] = a.con[ic(k, i, tr, L, NC)];
        if (nvl != 1) {
            if (k == b) {
                R rt2 = pos_part(a.w.qi[ix0(k, i, L)]);
                s1a[tr] = rt2 * (ck[tr] - a.con[ic(k + 1, i, tr, L, NC)]);
                s2a[tr] = rt2;
            } else if (k == tl) {
                R rt1 = pos_part(a.w.qi[ix0(k - 1, i, L)]);
                s1a[tr] = rt1 * (ck[tr] - a.con[ic(k - 1, i, tr, L, NC)]);
                s2a[tr] = rt1;
            } else {
                R rt1 = pos_part(a.w.qi[ix0(k - 1, i, L)]);
                R rt2 = pos_part(a.w.qi[ix0(k, i, L)]);
                s1a[tr] = rt1 * (ck[tr] - a.con[ic(k - 1, i, tr, L, NC)]) +
                          rt2 * (ck[tr] - a.con[ic(k + 1, i, tr, L, NC)]);
                s2a[tr] = rt1 + rt2;
            }
        }
    }
    for (int l = 1; l <= tq; ++l) {
        const int fj = g.cell_face(l, i);
        if (!face_open(g, fj)) continue;
        const R q2 = flip(a.w.qj[ix(k, fj, L)], g.cell_sign(l, i));
        if (is_neg(q2)) {
            const int nb = g.cell_adj(l, i);
            for (int tr = 0; tr < a.ntr; ++tr) {
                R cik = nb > 0 ? a.con[ic(k, nb, tr, L, NC)] : oqb_value(a, i, k, tr);
                s1[tr] = s1[tr] + fabs(q2) * (ck[tr] - cik);
                s2[tr] = s2[tr] + fabs(q2);
            }
        }
    }
    for (int tr = 0; tr < a.ntr; ++tr) {
        a.w.sa1[((long)tr * NC + i - 1) * L + k - 1] = s1a[tr] + s1[tr];
        a.w.sa2[((long)tr * NC + i - 1) * L + k - 1] = s2a[tr] + s2[tr];
        if (k == tl) {
            a.w.tr_last[((long)tr * NC + i - 1) * 2] = s1[tr];
            a.w.tr_last[((long)tr * NC + i - 1) * 2 + 1] = s2[tr];
        }
    }
}

__global__ void __launch_bounds__(256) k_tr_sums_cl(TArgs<float> a) {
    const Geom &g = a.g;
    unsigned t = flat_tid();
    const int L = g.L, NC = g.NC;
    if (t >= (unsigned)NC * L) return;
    int i, k;
    split_index(t, L, i, k);
    i += 1;
    k += 1;
    const int tl = a.s.top_cell[i - 1], b = g.bottom_cell[i - 1];
    if (tl == 0 || k < b || k > tl) return;
    tr_sums_at(a, i, k);
}

template <typename R> __global__ void __launch_bounds__(256) k_tr_sums_list(TArgs<R> a) {
    const int n = *a.w.cl_count;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int code = a.w.cl_list[t];
        const int i = list_entity(code), k = list_layer(code);
        tr_sums_at(a, i, k);
    }
}

// :806-871 with one thread per (cell, interface), the expressions of limiter_column
template <typename R> __device__ __forceinline__ void tr_vpsi_at(const TArgs<R> &a, int i, int k) {
    const Geom &g = a.g;
    const int L = g.L, NC = g.NC;
    const int b = g.bottom_cell[i - 1];
    for (int tr = 0; tr < a.ntr; ++tr) {
        const R last1 = a.w.tr_last[((long)tr * NC + i - 1) * 2], last2 = a.w.tr_last[((long)tr * NC + i - 1) * 2 + 1];
        R *psi = a.w.psii + (long)tr * NC * (L + 1);
        R ck = a.con[ic(k, i, tr, L, NC)];
        R qm = k > b ? a.w.qi[ix0(k - 1, i, L)] : R(0.0);
        R rt1 = last1 + fabs(qm) * (ck - a.con[ic(k - 1, i, tr, L, NC)]);
        R rt2 = last2 + fabs(qm);
        R rtemp = (a.con[ic(k + 1, i, tr, L, NC)] - ck) * rt2;
        psi[ix0(k, i, L)] = limited_ratio(a.p.h_flux_limiter, a.w.phii[ix0(k, i, L)], rt1, rtemp);
    }
}

__global__ void __launch_bounds__(256) k_tr_vpsi_cl(TArgs<float> a) {
    const Geom &g = a.g;
    unsigned t = flat_tid();
    const int L = g.L, NC = g.NC;
    if (t >= (unsigned)NC * L) return;
    int i, k;
    split_index(t, L, i, k);
    i += 1;
    k += 1;
    const int tl = a.s.top_cell[i - 1], b = g.bottom_cell[i - 1];
    if (tl == 0 || k < b || k > tl - 1) return;
    tr_vpsi_at(a, i, k);
}

template <typename R> __global__ void __launch_bounds__(256) k_tr_vpsi_list(TArgs<R> a) {
    const int n = *a.w.cl_count;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int code = a.w.cl_list[t];
        const int i = list_entity(code), k = list_layer(code);
        if (k >= a.s.top_cell[i - 1]) continue;   // interfaces b .. top - 1
        tr_vpsi_at(a, i, k);
    }
}

// FP32 path: vertical coefficients of the wet interfaces from the wet cell-layer list (the FP32
// kernels never read the entries outside a column's wet interfaces, so they are not cleared)
__global__ void __launch_bounds__(256) k_tr_cell_coef_list(TArgs<float> a) {
    const int n = *a.w.cl_count;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int code = a.w.cl_list[t];
        const int i = list_entity(code), k = list_layer(code);
        if (k >= a.s.top_cell[i - 1]) continue;   // interfaces b .. top - 1
        const long o = ix0(k, i, a.g.L);
        if (!a.changed_only || !same_bits(a.s.dzhalf_cell[o], a.s.dzhalf_cell_new[o])) cell_coef_at(a, i, o);
    }
}

// :769-799 + :876-900 face ratio r_jk from its upwind cell (the last writer in cell order), PSI_jk;
// one thread per face walks its wet layers
template <typename R> __device__ __forceinline__ void limiter_face_layer(const TArgs<R> &a, int j, int k, bool open,
                                                                     int c1, int c2, int t1, int b1, int t2, int b2) {
    const Geom &g = a.g;
    const int L = g.L, NC = g.NC;
    long t = ix(k, j, L);
    R Q = a.w.qj[t];
    int writer = 0;
    if (open) {
        // a cell writes when it is wet, holds layer k and sees Q*sign >= 0; cell 2 comes later
        if (c2 != 0 && t2 != 0 && k >= b2 && k <= t2 && !is_pos(Q)) writer = c2;   // -Q >= 0
        else if (t1 != 0 && k >= b1 && k <= t1 && !is_neg(Q)) writer = c1;        // Q >= 0
    }
    const R phi = a.w.phij[t];
    // the operands of both possible writers are loaded before the writer is known, so the loads
    // overlap the flux test instead of following it
    const bool in1 = t1 != 0 && k >= b1 && k <= t1, in2 = c2 != 0 && t2 != 0 && k >= b2 && k <= t2;
    R con1[2] = {R(0), R(0)}, con2[2] = {R(0), R(0)}, s1w[2] = {R(0), R(0)}, s2w[2] = {R(0), R(0)},
      s1o[2] = {R(0), R(0)}, s2o[2] = {R(0), R(0)}, cob[2] = {R(0), R(0)};
#pragma unroll
    for (int tr = 0; tr < 2; ++tr) {
        if (tr >= a.ntr) break;
        con1[tr] = a.con[ic(k, c1, tr, L, NC)];
        if (c2 > 0) con2[tr] = a.con[ic(k, c2, tr, L, NC)];
        else cob[tr] = oqb_value(a, c1, k, tr);
        if (in1) {
            s1w[tr] = a.w.sa1[((long)tr * NC + c1 - 1) * L + k - 1];
            s2w[tr] = a.w.sa2[((long)tr * NC + c1 - 1) * L + k - 1];
        }
        if (in2) {
            s1o[tr] = a.w.sa1[((long)tr * NC + c2 - 1) * L + k - 1];
            s2o[tr] = a.w.sa2[((long)tr * NC + c2 - 1) * L + k - 1];
        }
    }
#pragma unroll
    for (int tr = 0; tr < 2; ++tr) {
        if (tr >= a.ntr) break;
        R v;
        if (writer != 0) {
            // writer c1: the other side is c2 or the boundary value; writer c2: the other is c1
            const bool w1 = writer == c1;
            const R cik = w1 ? (c2 > 0 ? con2[tr] : cob[tr]) : con1[tr];
            const R cw = w1 ? con1[tr] : con2[tr];
            R rtemp = (w1 ? s2w[tr] : s2o[tr]) * (cik - cw);
            v = limited_ratio(a.p.h_flux_limiter, phi, w1 ? s1w[tr] : s1o[tr], rtemp);
        } else {
            v = phi_limit(a.p.h_flux_limiter, phi, R(1.0));
        }
        a.w.psij[(long)tr * g.NF * L + t] = v;
    }
}

template <typename R> __global__ void k_tr_limiter_faces(TArgs<R> a) {
    unsigned tid = flat_tid();
    const Geom &g = a.g;
    if (tid >= (unsigned)g.NF) return;
    int j = g.face_order[tid];
    int b = g.bottom_face[j - 1], tf = a.s.top_face[j - 1];
    if (tf == 0) return;
    bool open = face_open(g, j);
    int c1 = g.face_cell(1, j), c2 = g.face_cell(2, j);
    int t1 = a.s.top_cell[c1 - 1], b1 = g.bottom_cell[c1 - 1];
    int t2 = c2 != 0 ? a.s.top_cell[c2 - 1] : 0, b2 = c2 != 0 ? g.bottom_cell[c2 - 1] : 0;
    for (int k = b; k <= tf; ++k) limiter_face_layer(a, j, k, open, c1, c2, t1, b1, t2, b2);
}

// FP32 path: one thread per (face, layer), layers of a face on consecutive lanes
template <typename R> __global__ void k_tr_limiter_faces_flat(TArgs<R> a) {
    unsigned t = flat_tid();
    const Geom &g = a.g;
    if (t >= (unsigned)g.NF * g.L) return;
    int j, k;
    split_index(t, g.L, j, k);
    j += 1;
    k += 1;
    int b = g.bottom_face[j - 1], tf = a.s.top_face[j - 1];
    if (k < b || k > tf) return;
    int c1 = g.face_cell(1, j), c2 = g.face_cell(2, j);
    int t1 = a.s.top_cell[c1 - 1], b1 = g.bottom_cell[c1 - 1];
    int t2 = c2 != 0 ? a.s.top_cell[c2 - 1] : 0, b2 = c2 != 0 ? g.bottom_cell[c2 - 1] : 0;
    limiter_face_layer(a, j, k, face_open(g, j), c1, c2, t1, b1, t2, b2);
}

// FP32 path: face coefficients, one thread per (face, layer)
template <typename R> __global__ void k_tr_face_coef_flat(TArgs<R> a) {
    unsigned t = flat_tid();
    const Geom &g = a.g;
    if (t >= (unsigned)g.NF * g.L) return;
    int j, k;
    split_index(t, g.L, j, k);
    j += 1;
    k += 1;
    int b = g.bottom_face[j - 1], tf = a.s.top_face[j - 1];
    if (k >= b && k <= tf) {
        if (!a.changed_only || !same_bits(a.s.dz_face[t], a.s.dz_face_new[t])) face_coef_at(a, j, k, (long)t);
    } else if (!a.changed_only) {
        a.w.qj[t] = R(0);
        a.w.dj[t] = R(0);
        a.w.phij[t] = R(0);
    }
}

// :921-1346 per cell column: explicit horizontal fluxes + limiter, implicit vertical system,
// Thomas solve, clamp to [0, 50]; writes the full next column (zero outside the wet range).
template <typename R> __device__ void tr_solve_column(const TArgs<R> &a, int i) {
    const Geom &g = a.g;
    const int L = g.L, NC = g.NC;
    int tl = a.s.top_cell[i - 1], b = g.bottom_cell[i - 1];
    const R dt2 = a.dt2;
    const int Nt = a.Nt, sub = a.sub;
    const bool lim = a.p.h_flux_limiter > 0 || a.p.v_flux_limiter > 0;
    if (tl == 0) {
        for (int k = 0; k <= L + 1; ++k)
            for (int tr = 0; tr < a.ntr; ++tr) a.con_new[ic(k, i, tr, L, NC)] = R(0.0);
        return;
    }
    int nvl = tl - b + 1;
    const R ar = geo<R>(g.area, g.area_f, i - 1);
    R am[GOM_MAXL], bm[GOM_MAXL], cm[GOM_MAXL], gm[GOM_MAXL];
    R rhs[GOM_MAXL][2];
    for (int k = b + 1; k <= tl - 1; ++k) {
        int kk = tl + 1 - k;
        am[kk - 1] = -dt2 * a.w.di[ix0(k, i, L)];
        cm[kk - 1] = -dt2 * a.w.di[ix0(k - 1, i, L)];
        R dzc = a.s.dz_cell[ix(k, i, L)];
        R dz_new = dzc + divnt((a.s.dz_cell_new[ix(k, i, L)] - dzc) * (sub + 1), a);
        bm[kk - 1] = -am[kk - 1] + ar * dz_new - cm[kk - 1];
    }
    {
        R dzc = a.s.dz_cell[ix(tl, i, L)];
        R dz_new = dzc + divnt((a.s.dz_cell_new[ix(tl, i, L)] - dzc) * (sub + 1), a);
        if (tl == b) {
            bm[0] = ar * dz_new;
        } else {
            cm[0] = -dt2 * a.w.di[ix0(tl - 1, i, L)];
            bm[0] = ar * dz_new - cm[0];
            am[nvl - 1] = -dt2 * a.w.di[ix0(b, i, L)];
            R dzb = a.s.dz_cell[ix(b, i, L)];
            R dz_newb = dzb + divnt((a.s.dz_cell_new[ix(b, i, L)] - dzb) * (sub + 1), a);
            bm[nvl - 1] = -am[nvl - 1] + ar * dz_newb;
        }
    }
    int tq = g.tri_or_quad[i - 1];
    int fj[4], nb[4], fb[4], ft[4], sg[4];
    bool open[4];
    for (int l = 1; l <= tq; ++l) {
        fj[l - 1] = g.cell_face(l, i);
        nb[l - 1] = g.cell_adj(l, i);
        sg[l - 1] = g.cell_sign(l, i);
        open[l - 1] = face_open(g, fj[l - 1]);
        fb[l - 1] = g.bottom_face[fj[l - 1] - 1];
        ft[l - 1] = a.s.top_face[fj[l - 1] - 1];
    }
    for (int k = b; k <= tl; ++k) {
        int kk = tl + 1 - k;
        R sQi[2] = {0, 0}, sQii[2] = {0, 0}, shd[2] = {0, 0}, shl[2] = {0, 0};
        R ck[2];
        for (int tr = 0; tr < a.ntr; ++tr) ck[tr] = a.con[ic(k, i, tr, L, NC)];
        for (int l = 0; l < tq; ++l) {
            if (!open[l]) continue;
            bool in_face = k >= fb[l] && k <= ft[l];
            long fo = ix(k, fj[l], L);
            R q2 = flip(in_face ? a.w.qj[fo] : R(0.0), sg[l]);
            R dface = in_face ? a.w.dj[fo] : R(0.0);
            bool qpos = is_pos(q2), qneg = is_neg(q2);
            for (int tr = 0; tr < a.ntr; ++tr) {
                R cik = nb[l] > 0 ? a.con[ic(k, nb[l], tr, L, NC)] : oqb_value(a, i, k, tr);
                if (qpos) sQi[tr] = sQi[tr] + fabs(q2) * ck[tr];
                else if (qneg) sQii[tr] = sQii[tr] + fabs(q2) * cik;
                shd[tr] = shd[tr] + dface * (cik - ck[tr]);
                R psi = (lim && in_face) ? a.w.psij[(long)tr * g.NF * L + fo] : R(0.0);
                shl[tr] = shl[tr] + psi * fabs(q2) * (ck[tr] - cik);
            }
        }
        R dzc = a.s.dz_cell[ix(k, i, L)];
        R dz_old = dzc + divnt((a.s.dz_cell_new[ix(k, i, L)] - dzc) * sub, a);
        for (int tr = 0; tr < a.ntr; ++tr) {
            R h_adv = dt2 * (sQii[tr] - sQi[tr]);
            R h_diff = dt2 * shd[tr];
            R h_flux = R(0.5) * dt2 * shl[tr];
            R v = ar * dz_old * ck[tr] + h_adv + h_diff;
            if (a.p.h_flux_limiter > 0) v = v + h_flux;
            rhs[kk - 1][tr] = v;
        }
    }
    if (nvl != 1) {
        for (int k = b; k <= tl; ++k) {
            int kk = tl + 1 - k;
            for (int tr = 0; tr < a.ntr; ++tr) {
                const R *psi = a.w.psii + (long)tr * NC * (L + 1);
                R c0 = a.con[ic(k, i, tr, L, NC)];
                R v = rhs[kk - 1][tr];
                if (k == b) {
                    R q = a.w.qi[ix0(k, i, L)];
                    R qp = pos_part(q), qm = neg_part(q);
                    R cp1 = a.con[ic(k + 1, i, tr, L, NC)];
                    v = v + dt2 * (-qp * c0 + qm * cp1);
                    if (a.p.v_flux_limiter > 0) {
                        R ps = lim ? psi[ix0(k, i, L)] : R(0.0);
                        v = v + R(0.5) * dt2 * (-ps * qp * (cp1 - c0) + ps * qm * (c0 - cp1));
                    }
                } else if (k == tl) {
                    R q = a.w.qi[ix0(k - 1, i, L)];
                    R qp = pos_part(q), qm = neg_part(q);
                    R cm1 = a.con[ic(k - 1, i, tr, L, NC)];
                    v = v + dt2 * (qp * cm1 - qm * c0);
                    if (a.p.v_flux_limiter > 0) {
                        R ps = lim ? psi[ix0(k - 1, i, L)] : R(0.0);
                        v = v + R(0.5) * dt2 * (ps * qp * (c0 - cm1) - ps * qm * (cm1 - c0));
                    }
                } else {
                    R q1 = a.w.qi[ix0(k - 1, i, L)], q = a.w.qi[ix0(k, i, L)];
                    R qp1 = pos_part(q1), qm1 = neg_part(q1);
                    R qp = pos_part(q), qm = neg_part(q);
                    R cm1 = a.con[ic(k - 1, i, tr, L, NC)], cp1 = a.con[ic(k + 1, i, tr, L, NC)];
                    v = v + dt2 * (qp1 * cm1 - qp * c0 + qm * cp1 - qm1 * c0);
                    if (a.p.v_flux_limiter > 0) {
                        R p1 = lim ? psi[ix0(k - 1, i, L)] : R(0.0), p0 = lim ? psi[ix0(k, i, L)] : R(0.0);
                        v = v + R(0.5) * dt2 *
                                    (p1 * qp1 * (c0 - cm1) - p0 * qp * (cp1 - c0) + p0 * qm * (c0 - cp1) -
                                     p1 * qm1 * (cm1 - c0));
                    }
                }
                rhs[kk - 1][tr] = v;
            }
        }
    }
    bool okp;
    if (a.ntr == 2) okp = thomas<2>(nvl, am, bm, cm, rhs, gm);
    else {
        R r1[GOM_MAXL][1];
        for (int k = 0; k < nvl; ++k) r1[k][0] = rhs[k][0];
        okp = thomas<1>(nvl, am, bm, cm, r1, gm);
        for (int k = 0; k < nvl; ++k) rhs[k][0] = r1[k][0];
    }
    if (!okp) {
        record_error(a.st, GOM_E_ZERO_PIVOT, 1285, i, 0, 0.0, GOM_ENTITY_CELL);
        return;
    }
    for (int tr = 0; tr < a.ntr; ++tr) {
        for (int k = 0; k <= L + 1; ++k) {
            R v = R(0.0);
            if (k >= b && k <= tl) {
                R sv = rhs[tl - k][tr];
                if (sv >= R(0.0) && sv <= R(50.0)) v = sv;
                else if (sv < R(0.0)) v = R(0.0);
                else if (sv > R(50.0)) v = R(50.0);
                else v = nan_keep(a, k, i, tr);
            }
            a.con_new[ic(k, i, tr, L, NC)] = v;
        }
    }
}

template <typename R> __global__ void __launch_bounds__(256) k_tr_solve(TArgs<R> a) {
    unsigned tid = flat_tid();
    if (tid >= (unsigned)a.g.NC) return;
    tr_solve_column(a, a.g.cell_order[tid]);
}

// ---------------------------------------------------------------------------- FP32 cell-layers
// The mixed-precision path forms the transport fluxes with one thread per (cell, layer): layers of
// a cell sit on consecutive lanes, so the layer-contiguous arrays are read in coalesced runs and
// the GPU holds enough threads to hide the latency of the neighbour gathers.  Each row of the
// implicit vertical system is written to work arrays, and one thread per column then runs the
// tridiagonal solve.  FP32 arithmetic is cheap on GB300, so the lanes of dry layers are simply
// idle.
template <typename R> __device__ __forceinline__ R clamp_tracer(R sv, R prev) {
    if (sv >= R(0) && sv <= R(50)) return sv;
    if (sv < R(0)) return R(0);
    if (sv > R(50)) return R(50);
    return prev;   // NaN: the reference keeps the previous value
}

// :921-1250 for one wet cell-layer: right-hand sides and the row of the implicit system
// (a couples the layer below, c the layer above)
__device__ __forceinline__ void tr_rows_at(const TArgs<float> &a, int i, int k) {
    const Geom &g = a.g;
    const int L = g.L, NC = g.NC;
    const int tl = a.s.top_cell[i - 1], b = g.bottom_cell[i - 1];
    (void)L;
    (void)NC;
    const float dt2 = a.dt2;
    const int sub = a.sub;
    const bool lim = a.p.h_flux_limiter > 0 || a.p.v_flux_limiter > 0;
    const float ar = g.area_f[i - 1];
    const int tq = g.tri_or_quad[i - 1];
    float c0[2] = {0.0f, 0.0f};
    for (int tr = 0; tr < a.ntr; ++tr) c0[tr] = a.con[ic(k, i, tr, L, NC)];
    float sQi[2] = {0, 0}, sQii[2] = {0, 0}, shd[2] = {0, 0}, shl[2] = {0, 0};
    for (int l = 1; l <= tq; ++l) {
        const int fj = g.cell_face(l, i);
        if (!face_open(g, fj)) continue;
        const int nb = g.cell_adj(l, i), sg = g.cell_sign(l, i);
        const bool in_face = k >= g.bottom_face[fj - 1] && k <= a.s.top_face[fj - 1];
        const long fo = ix(k, fj, L);
        const float q2 = flip(in_face ? a.w.qj[fo] : 0.0f, sg);
        const float dface = in_face ? a.w.dj[fo] : 0.0f;
        const bool qpos = is_pos(q2), qneg = is_neg(q2);
        for (int tr = 0; tr < a.ntr; ++tr) {
            float cik = nb > 0 ? a.con[ic(k, nb, tr, L, NC)] : oqb_value(a, i, k, tr);
            if (qpos) sQi[tr] = sQi[tr] + fabsf(q2) * c0[tr];
            else if (qneg) sQii[tr] = sQii[tr] + fabsf(q2) * cik;
            shd[tr] = shd[tr] + dface * (cik - c0[tr]);
            float psi = (lim && in_face) ? a.w.psij[(long)tr * g.NF * L + fo] : 0.0f;
            shl[tr] = shl[tr] + psi * fabsf(q2) * (c0[tr] - cik);
        }
    }
    const float dzc = a.s.dz_cell[ix(k, i, L)], dzn = a.s.dz_cell_new[ix(k, i, L)];
    const float dz_old = dzc + divnt((dzn - dzc) * (float)sub, a);
    const float dz_new = dzc + divnt((dzn - dzc) * (float)(sub + 1), a);
    const int nvl = tl - b + 1;
    const float qlo = k > b ? a.w.qi[ix0(k - 1, i, L)] : 0.0f;   // interface below layer k
    const float qhi = k < tl ? a.w.qi[ix0(k, i, L)] : 0.0f;      // interface above
    for (int tr = 0; tr < a.ntr; ++tr) {
        float v = ar * dz_old * c0[tr] + dt2 * (sQii[tr] - sQi[tr]) + dt2 * shd[tr];
        if (a.p.h_flux_limiter > 0) v = v + 0.5f * dt2 * shl[tr];
        if (nvl != 1) {
            const float *psi = a.w.psii + (long)tr * NC * (L + 1);
            const float c = c0[tr];
            if (k > b) {
                float qp1 = pos_part(qlo), qm1 = neg_part(qlo);
                float cm1 = a.con[ic(k - 1, i, tr, L, NC)];
                v = v + dt2 * (qp1 * cm1 - qm1 * c);
                if (a.p.v_flux_limiter > 0) {
                    float p1 = lim ? psi[ix0(k - 1, i, L)] : 0.0f;
                    v = v + 0.5f * dt2 * (p1 * qp1 * (c - cm1) - p1 * qm1 * (cm1 - c));
                }
            }
            if (k < tl) {
                float qp = pos_part(qhi), qm = neg_part(qhi);
                float cp1 = a.con[ic(k + 1, i, tr, L, NC)];
                v = v + dt2 * (qm * cp1 - qp * c);
                if (a.p.v_flux_limiter > 0) {
                    float p0 = lim ? psi[ix0(k, i, L)] : 0.0f;
                    v = v + 0.5f * dt2 * (-p0 * qp * (cp1 - c) + p0 * qm * (c - cp1));
                }
            }
        }
        a.w.tr_rhs[((long)tr * NC + i - 1) * L + k - 1] = v;
    }
    const float am = k > b ? -dt2 * a.w.di[ix0(k - 1, i, L)] : 0.0f;
    const float cm = k < tl ? -dt2 * a.w.di[ix0(k, i, L)] : 0.0f;
    const long o = (long)(i - 1) * L + k - 1;
    a.w.tr_a[o] = am;
    a.w.tr_b[o] = ar * dz_new - am - cm;
    a.w.tr_c[o] = cm;
}

// FP64 list form of tr_solve_column: the row of one wet (cell, layer) of the implicit vertical
// system and its right-hand sides, formed with the column kernel's expressions in its order (so
// the list-form solve gives the column form's results bit for bit), written for k_tr_thomas_col:
// tr_a couples the layer below, tr_c the layer above.
__device__ __forceinline__ void tr_rows64_at(const TArgs<double> &a, int i, int k) {
    const Geom &g = a.g;
    const int L = g.L, NC = g.NC;
    const int tl = a.s.top_cell[i - 1], b = g.bottom_cell[i - 1];
    const double dt2 = a.dt2;
    const bool lim = a.p.h_flux_limiter > 0 || a.p.v_flux_limiter > 0;
    const double ar = g.area[i - 1];
    const int nvl = tl - b + 1;
    const double dzc = a.s.dz_cell[ix(k, i, L)];
    const double dz_new = dzc + divnt((a.s.dz_cell_new[ix(k, i, L)] - dzc) * a.sub1_r, a);
    double am = 0.0, bm, cm = 0.0;   // am: the layer above, cm: the layer below
    if (tl == b) {
        bm = ar * dz_new;
    } else if (k == tl) {
        cm = -dt2 * a.w.di[ix0(tl - 1, i, L)];
        bm = ar * dz_new - cm;
    } else if (k == b) {
        am = -dt2 * a.w.di[ix0(b, i, L)];
        bm = -am + ar * dz_new;
    } else {
        am = -dt2 * a.w.di[ix0(k, i, L)];
        cm = -dt2 * a.w.di[ix0(k - 1, i, L)];
        bm = -am + ar * dz_new - cm;
    }
    const int tq = g.tri_or_quad[i - 1];
    // GB300 issues an FP64 warp instruction at the same cost however few of its lanes are active,
    // so the branches below select operands (integer work) and every lane then runs the same FP64
    // instructions; each lane's operations and their order are those of the column form.  The
    // tracer loops are unrolled so that the sums stay in registers.
    double sQi[2] = {0, 0}, sQii[2] = {0, 0}, shd[2] = {0, 0}, shl[2] = {0, 0};
    double ck[2] = {0, 0};
#pragma unroll
    for (int tr = 0; tr < 2; ++tr)
        if (tr < a.ntr) ck[tr] = a.con[ic(k, i, tr, L, NC)];
    for (int l = 1; l <= tq; ++l) {
        const int fj = g.cell_face(l, i);
        if (!face_open(g, fj)) continue;
        const int nb = g.cell_adj(l, i);
        const bool in_face = k >= g.bottom_face[fj - 1] && k <= a.s.top_face[fj - 1];
        const long fo = ix(k, fj, L);
        const double q2 = flip(in_face ? a.w.qj[fo] : 0.0, g.cell_sign(l, i));
        const double dface = in_face ? a.w.dj[fo] : 0.0;
        const bool qpos = is_pos(q2), qneg = is_neg(q2);
        const double aq = fabs(q2);
#pragma unroll
        for (int tr = 0; tr < 2; ++tr) {
            if (tr >= a.ntr) break;
            const double cik = nb > 0 ? a.con[ic(k, nb, tr, L, NC)] : oqb_value(a, i, k, tr);
            // outflow adds |q2| ck to sQi, inflow |q2| cik to sQii: one product and one sum for
            // every lane, the sum kept on the side the flux takes (neither for q2 = 0)
            const double up = aq * (qpos ? ck[tr] : cik);
            const double acc = (qpos ? sQi[tr] : sQii[tr]) + up;
            if (qpos) sQi[tr] = acc;
            else if (qneg) sQii[tr] = acc;
            shd[tr] = shd[tr] + dface * (cik - ck[tr]);
            const double psi = (lim && in_face) ? a.w.psij[(long)tr * g.NF * L + fo] : 0.0;
            shl[tr] = shl[tr] + psi * aq * (ck[tr] - cik);
        }
    }
    const double dz_old = dzc + divnt((a.s.dz_cell_new[ix(k, i, L)] - dzc) * a.sub_r, a);
    // the vertical terms: interior layers couple both interfaces; the bottom and the top layer
    // one interface each, in two expressions of the same shape, x1 x2 + y1 y2 and, with the
    // limiter, p1 d1 + p2 d2, whose operands the layer selects
    const bool interior = nvl != 1 && k != b && k != tl;
    const bool edge = nvl != 1 && (k == b || k == tl);
    const bool bot = k == b;
    double qlo = 0.0, qhi = 0.0;
    if (nvl != 1) {
        if (k > b) qlo = a.w.qi[ix0(k - 1, i, L)];
        if (k < tl) qhi = a.w.qi[ix0(k, i, L)];
    }
    const double qe = bot ? qhi : qlo;   // the one interface of the bottom / top layer
#pragma unroll
    for (int tr = 0; tr < 2; ++tr) {
        if (tr >= a.ntr) break;
        const double h_adv = dt2 * (sQii[tr] - sQi[tr]);
        const double h_diff = dt2 * shd[tr];
        const double h_flux = 0.5 * dt2 * shl[tr];
        double v = ar * dz_old * ck[tr] + h_adv + h_diff;
        if (a.p.h_flux_limiter > 0) v = v + h_flux;
        const double *psi = a.w.psii + (long)tr * NC * (L + 1);
        const double c0 = ck[tr];
        const double cm1 = k > b ? a.con[ic(k - 1, i, tr, L, NC)] : 0.0;
        const double cp1 = k < tl ? a.con[ic(k + 1, i, tr, L, NC)] : 0.0;
        double plo = 0.0, phi = 0.0;   // the limiter of the interface below / above
        if (a.p.v_flux_limiter > 0 && lim && nvl != 1) {
            plo = k > b ? psi[ix0(k - 1, i, L)] : 0.0;
            phi = k < tl ? psi[ix0(k, i, L)] : 0.0;
        }
        if (interior) {
            const double qp1 = pos_part(qlo), qm1 = neg_part(qlo);
            const double qp = pos_part(qhi), qm = neg_part(qhi);
            v = v + dt2 * (qp1 * cm1 - qp * c0 + qm * cp1 - qm1 * c0);
            if (a.p.v_flux_limiter > 0) {
                const double p1 = lim ? plo : 0.0, p0 = lim ? phi : 0.0;
                v = v + 0.5 * dt2 *
                            (p1 * qp1 * (c0 - cm1) - p0 * qp * (cp1 - c0) + p0 * qm * (c0 - cp1) -
                             p1 * qm1 * (cm1 - c0));
            }
        } else if (edge) {
            // bottom: -qp c0 + qm c(k+1); top: qp c(k-1) - qm c0 = qp c(k-1) + (-qm) c0
            const double qp = pos_part(qe), qm = neg_part(qe);
            const double cn = bot ? cp1 : cm1;
            const double x1 = bot ? -qp : qp, x2 = bot ? c0 : cn;
            const double y1 = bot ? qm : -qm, y2 = bot ? cn : c0;
            v = v + dt2 * (x1 * x2 + y1 * y2);
            if (a.p.v_flux_limiter > 0) {
                // bottom: -ps qp (c(k+1) - c0) + ps qm (c0 - c(k+1));
                // top:     ps qp (c0 - c(k-1)) - ps qm (c(k-1) - c0)
                const double ps = lim ? (bot ? phi : plo) : 0.0;
                const double u1 = bot ? cn : c0, u2 = bot ? c0 : cn;
                const double p1 = (bot ? -ps : ps) * qp;
                const double p2 = (bot ? ps : -ps) * qm;
                v = v + 0.5 * dt2 * (p1 * (u1 - u2) + p2 * (u2 - u1));
            }
        }
        a.w.tr_rhs[((long)tr * NC + i - 1) * L + k - 1] = v;
    }
    const long o = (long)(i - 1) * L + k - 1;
    a.w.tr_a[o] = cm;
    a.w.tr_b[o] = bm;
    a.w.tr_c[o] = am;
}

// The rows per listed wet cell-layer, each block taking 256 consecutive entries (the layers of
// about 28 columns) and reordering them in shared memory, interior layers first, then the bottom
// and top layers: each warp then takes one branch of the row's vertical terms (GB300 issues an
// FP64 warp instruction at the same cost however few lanes take its branch), and the two kinds of
// warps of a block work on the same columns at the same time (the neighbours' data is read once).
constexpr int ROWS_CHUNK = 256;

__global__ void __launch_bounds__(ROWS_CHUNK) k_tr_rows64_sorted(TArgs<double> a) {
    __shared__ int codes[ROWS_CHUNK];
    __shared__ int count_in[ROWS_CHUNK / 32], count_edge[ROWS_CHUNK / 32];
    const int n = *a.w.cl_count;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int base = blockIdx.x * ROWS_CHUNK; base < n; base += gridDim.x * ROWS_CHUNK) {
        const int t = base + threadIdx.x;
        int code = 0, kind = 2;   // 0 interior layer, 1 bottom or top layer, 2 past the list
        if (t < n) {
            code = a.w.cl_list[t];
            const int i = list_entity(code), k = list_layer(code);
            kind = (k == a.g.bottom_cell[i - 1] || k == a.s.top_cell[i - 1]) ? 1 : 0;
        }
        const unsigned in_mask = __ballot_sync(0xffffffffu, kind == 0);
        const unsigned edge_mask = __ballot_sync(0xffffffffu, kind == 1);
        if (lane == 0) {
            count_in[w] = __popc(in_mask);
            count_edge[w] = __popc(edge_mask);
        }
        __syncthreads();
        int in_before = 0, edge_before = 0, in_total = 0;
#pragma unroll
        for (int q = 0; q < ROWS_CHUNK / 32; ++q) {
            if (q < w) {
                in_before += count_in[q];
                edge_before += count_edge[q];
            }
            in_total += count_in[q];
        }
        const unsigned below = (1u << lane) - 1u;
        if (kind == 0) codes[in_before + __popc(in_mask & below)] = code;
        else if (kind == 1) codes[in_total + edge_before + __popc(edge_mask & below)] = code;
        __syncthreads();
        if (threadIdx.x < n - base) {
            const int c = codes[threadIdx.x];
            tr_rows64_at(a, list_entity(c), list_layer(c));
        }
        __syncthreads();   // the next chunk reuses codes and the counts
    }
}

__global__ void __launch_bounds__(256) k_tr_rows_cl(TArgs<float> a) {
    const Geom &g = a.g;
    unsigned t = flat_tid();
    const int L = g.L, NC = g.NC;
    if (t >= (unsigned)NC * L) return;
    int i, k;
    split_index(t, L, i, k);
    i += 1;
    k += 1;
    const int tl = a.s.top_cell[i - 1], b = g.bottom_cell[i - 1];
    if (tl == 0 || k < b || k > tl) return;
    tr_rows_at(a, i, k);
}

__global__ void __launch_bounds__(256) k_tr_rows_list(TArgs<float> a) {
    const int n = *a.w.cl_count;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int code = a.w.cl_list[t];
        const int i = list_entity(code), k = list_layer(code);
        tr_rows_at(a, i, k);
    }
}

// one thread per column: tridiagonal solve of the rows (top layer first, as
// tridiagonal_solver.f90 is called), clamp to [0, 50], full next column
template <typename R> __global__ void __launch_bounds__(256) k_tr_thomas_col(TArgs<R> a) {
    const Geom &g = a.g;
    unsigned tid = flat_tid();
    if (tid >= (unsigned)g.NC) return;
    const int i = column_entity<R>(g.cell_order, tid);
    const int L = g.L, NC = g.NC;
    const int tl = a.s.top_cell[i - 1], b = g.bottom_cell[i - 1];
    if (tl == 0) {
        for (int k = 0; k <= L + 1; ++k)
            for (int tr = 0; tr < a.ntr; ++tr) a.con_new[ic(k, i, tr, L, NC)] = R(0);
        return;
    }
    const int nvl = tl - b + 1;
    const long base = (long)(i - 1) * L;
    R gam[GOM_MAXL], x[GOM_MAXL][2];
    // row r = 1..nvl is layer k = tl + 1 - r: its lower neighbour (row r - 1) is the layer above;
    // the operations of thomas<> (tridiagonal_solver.f90) in the same order
    R den = a.w.tr_b[base + tl - 1];
    bool ok = den != R(0);
    for (int tr = 0; tr < a.ntr; ++tr) x[0][tr] = a.w.tr_rhs[((long)tr * NC + i - 1) * L + tl - 1] / den;
    for (int r = 2; r <= nvl && ok; ++r) {
        const int k = tl + 1 - r;
        const R lower = a.w.tr_c[base + k - 1];       // coupling to the layer above
        const R upper_prev = a.w.tr_a[base + k];       // previous row's coupling to this layer
        gam[r - 1] = upper_prev / den;
        den = a.w.tr_b[base + k - 1] - lower * gam[r - 1];
        ok = den != R(0);
        for (int tr = 0; tr < a.ntr; ++tr)
            x[r - 1][tr] = (a.w.tr_rhs[((long)tr * NC + i - 1) * L + k - 1] - lower * x[r - 2][tr]) / den;
    }
    if (!ok) {
        record_error(a.st, GOM_E_ZERO_PIVOT, 1285, i, 0, 0.0, GOM_ENTITY_CELL);
        return;
    }
    for (int r = nvl - 1; r >= 1; --r)
        for (int tr = 0; tr < a.ntr; ++tr) x[r - 1][tr] = x[r - 1][tr] - gam[r] * x[r][tr];
    for (int tr = 0; tr < a.ntr; ++tr) {
        for (int k = 0; k <= L + 1; ++k) {
            R v = R(0);
            if (k >= b && k <= tl) v = clamp_tracer(x[tl - k][tr], nan_keep(a, k, i, tr));
            a.con_new[ic(k, i, tr, L, NC)] = v;
        }
    }
}

// :1403-1454 node averages (column, top-down) and :1457-1482 face averages + write-back
template <typename R> __global__ void k_tr_nodes(TArgs<R> a) {
    unsigned tid = flat_tid();
    const Geom &g = a.g;
    if (tid >= (unsigned)g.NN) return;
    int i = column_entity<R>(g.node_order, tid);
    const int L = g.L, NC = g.NC;
    int tn = a.s.top_node[i - 1], bn = g.bottom_node[i - 1];
    int na = g.adj_cells_at_node[i - 1];
    for (int tr = 0; tr < a.ntr; ++tr) {
        R *dst = a.tid[tr] == 1 ? a.s.salt_node : a.s.temp_node;
        bool write = a.tid[tr] <= a.ntr;   // slot 1 -> salt, slot 2 -> temperature
        R above = R(0.0);
        for (int k = L; k >= 1; --k) {
            R v = R(0.0);
            if (tn != 0 && k <= tn && k >= bn) {
                R s11 = R(0.0), s22 = R(0.0);
                int count1 = 0;
                for (int l = 1; l <= na; ++l) {
                    int ii = g.node_cell(l, i);
                    if (k >= g.bottom_cell[ii - 1] && k <= a.s.top_cell[ii - 1]) {
                        R w = (R)g.area[ii - 1] * a.s.dz_cell_new[ix(k, ii, L)];
                        s11 = s11 + w;
                        s22 = s22 + w * a.con[ic(k, ii, tr, L, NC)];
                    } else {
                        count1 = count1 + 1;
                    }
                }
                v = s11 == R(0.0) ? R(0.0) : s22 / s11;
                if (count1 == na && k != tn) v = above;
            }
            if (write) dst[ix(k, i, L)] = v;
            above = v;
        }
    }
}

// FP32 path, the same per node: a block takes NT_TILE consecutive nodes, gathers each node's
// adjacent cells once into shared memory, forms every (node, layer) average in its own thread
// (neighbouring lanes read neighbouring layers of the same cells), resolves the fill from above
// per node in the column kernel's order, and writes the block's (L, node) tile coalesced.
constexpr int NT_TILE = 32;

__global__ void __launch_bounds__(256) k_tr_nodes_tile(TArgs<float> a) {
    __shared__ float col[NT_TILE][GOM_MAXL + 2];
    __shared__ unsigned char fill[NT_TILE][GOM_MAXL + 2];
    __shared__ int cell_s[NT_TILE][GOM_MAXNB], cb_s[NT_TILE][GOM_MAXNB], ct_s[NT_TILE][GOM_MAXNB];
    __shared__ float car_s[NT_TILE][GOM_MAXNB];
    __shared__ int tn_s[NT_TILE], bn_s[NT_TILE], na_s[NT_TILE];
    const Geom &g = a.g;
    const int L = g.L, NC = g.NC;
    const int i0 = blockIdx.x * NT_TILE;
    const int nn = min(NT_TILE, g.NN - i0);
    for (int c = threadIdx.x; c < nn; c += blockDim.x) {
        const int i = i0 + c + 1;
        tn_s[c] = a.s.top_node[i - 1];
        bn_s[c] = g.bottom_node[i - 1];
        const int na = g.adj_cells_at_node[i - 1];
        na_s[c] = na;
        for (int l = 1; l <= na; ++l) {
            const int ii = g.node_cell(l, i);
            cell_s[c][l - 1] = ii;
            cb_s[c][l - 1] = g.bottom_cell[ii - 1];
            ct_s[c][l - 1] = a.s.top_cell[ii - 1];
            car_s[c][l - 1] = g.area_f[ii - 1];
        }
    }
    __syncthreads();
    const long base = (long)i0 * L;
    for (int tr = 0; tr < a.ntr; ++tr) {
        if (a.tid[tr] > a.ntr) continue;   // slot 1 -> salinity, slot 2 -> temperature
        float *dst = a.tid[tr] == 1 ? a.s.salt_node : a.s.temp_node;
        for (int t = threadIdx.x; t < nn * L; t += blockDim.x) {
            const int c = t / L, k = t - c * L + 1;
            const int tn = tn_s[c];
            float v = 0.0f;
            bool f = false;
            if (tn != 0 && k <= tn && k >= bn_s[c]) {
                float s11 = 0.0f, s22 = 0.0f;
                int count1 = 0;
                const int na = na_s[c];
                for (int l = 0; l < na; ++l) {
                    const int ii = cell_s[c][l];
                    if (k >= cb_s[c][l] && k <= ct_s[c][l]) {
                        const float w = car_s[c][l] * a.s.dz_cell_new[ix(k, ii, L)];
                        s11 = s11 + w;
                        s22 = s22 + w * a.con[ic(k, ii, tr, L, NC)];
                    } else {
                        count1 = count1 + 1;
                    }
                }
                v = s11 == 0.0f ? 0.0f : s22 / s11;
                f = count1 == na && k != tn;
            }
            col[c][k] = v;
            fill[c][k] = f;
        }
        __syncthreads();
        for (int c = threadIdx.x; c < nn; c += blockDim.x)
            for (int k = tn_s[c] - 1; k >= 1; --k)
                if (fill[c][k]) col[c][k] = col[c][k + 1];
        __syncthreads();
        for (int t = threadIdx.x; t < nn * L; t += blockDim.x) {
            const int c = t / L, k = t - c * L + 1;
            dst[base + t] = col[c][k];
        }
        __syncthreads();
    }
}

template <typename R> __global__ void k_tr_faces_cells(TArgs<R> a) {
    unsigned t = flat_tid();
    const Geom &g = a.g;
    const int L = g.L, NC = g.NC;
    unsigned nfl = (unsigned)g.NF * L, ncl = (unsigned)g.NC * L;
    if (t < nfl) {
        int j, k;
        split_index(t, L, j, k);
        j += 1;
        k += 1;
        int n1 = g.face_node(1, j), n2 = g.face_node(2, j);
        bool in = k >= g.bottom_face[j - 1] && k <= a.s.top_face[j - 1];
        for (int tr = 0; tr < a.ntr; ++tr) {
            if (a.tid[tr] > a.ntr) continue;
            const R *src = a.tid[tr] == 1 ? a.s.salt_node : a.s.temp_node;
            R *dst = a.tid[tr] == 1 ? a.s.salt_face : a.s.temp_face;
            dst[t] = in ? (src[ix(k, n1, L)] + src[ix(k, n2, L)]) * R(0.5) : R(0.0);
        }
    } else if (t < nfl + ncl) {
        unsigned u = t - nfl;
        int i, k;
        split_index(u, L, i, k);
        i += 1;
        k += 1;
        for (int tr = 0; tr < a.ntr; ++tr) {
            if (a.tid[tr] > a.ntr) continue;
            R *dst = a.tid[tr] == 1 ? a.s.salt_cell_new : a.s.temp_cell_new;
            dst[u] = a.con[ic(k, i, tr, L, NC)];
        }
    }
}

template <typename R> bool transport_args(const LaunchT<R> &x, TArgs<R> &a) {
    const Params &p = x.p;
    if (!p.transport_flag) return false;
    a.g = x.g;
    a.s = x.s;
    a.f = x.f;
    a.p = x.p;
    a.w = x.w;
    a.st = x.status;
    a.ntr = 0;
    if (p.is_salt) a.tid[a.ntr++] = 1;
    if (p.is_temp) a.tid[a.ntr++] = 2;
    if (a.ntr == 0) return false;
    a.Nt = p.trans_sub_iter == 0 ? 1 : p.trans_sub_iter;
    a.dt2 = (R)(p.dt / a.Nt);
    a.pow2 = (a.Nt & (a.Nt - 1)) == 0;
    a.inv_nt = (R)(1.0 / a.Nt);
    a.theta = (R)p.theta;
    a.om_theta = (R)(1.0 - p.theta);
    a.changed_only = false;
    a.sub = 0;
    a.sub_r = R(0);
    a.sub1_r = R(1);
    a.con = x.w.con;
    a.con_new = x.w.con2;
    return true;
}

// the column solve of one subcycle alone (coefficients and limiter of the last transport call)
template <typename R> cudaError_t launch_tr_solve_only(const LaunchT<R> &x) {
    TArgs<R> a;
    if (!transport_args(x, a)) return cudaSuccess;
    const Geom &g = x.g;
    const int bs_solve = x.tune[TUNE_TR_SOLVE] == 1 ? 64 : x.tune[TUNE_TR_SOLVE] == 2 ? 256 : 128;
    if constexpr (sizeof(R) == sizeof(float)) {
        k_tr_rows_cl<<<blocks_for((long)g.NC * g.L, bs_solve), bs_solve, 0, x.stream>>>(a);
        k_tr_thomas_col<<<blocks_for(g.NC, 128), 128, 0, x.stream>>>(a);
    } else if (x.tune[TUNE_TR_SOLVE] == 3 && x.w.tr_a) {
        // rows from the wet cell-layer list the last transport call built
        k_tr_rows64_sorted<<<x.num_sms * 3, ROWS_CHUNK, 0, x.stream>>>(a);
        k_tr_thomas_col<<<blocks_for(g.NC, 128), 128, 0, x.stream>>>(a);
    } else {
        k_tr_solve<<<blocks_for(g.NC, bs_solve), bs_solve, 0, x.stream>>>(a);
    }
    return cudaGetLastError();
}

template <typename R> cudaError_t launch_transport(const LaunchT<R> &x) {
    const Params &p = x.p;
    if (!p.transport_flag) return cudaSuccess;
    if (p.transport_solver == 2) return launch_transport_elm(x);
    TArgs<R> a;
    a.g = x.g;
    a.s = x.s;
    a.f = x.f;
    a.p = x.p;
    a.w = x.w;
    a.st = x.status;
    a.ntr = 0;
    if (p.is_salt) a.tid[a.ntr++] = 1;
    if (p.is_temp) a.tid[a.ntr++] = 2;
    if (a.ntr == 0) return cudaSuccess;
    a.Nt = p.trans_sub_iter == 0 ? 1 : p.trans_sub_iter;
    a.dt2 = (R)(p.dt / a.Nt);
    a.pow2 = (a.Nt & (a.Nt - 1)) == 0;
    a.inv_nt = (R)(1.0 / a.Nt);
    a.theta = (R)p.theta;
    a.om_theta = (R)(1.0 - p.theta);
    a.changed_only = false;
    const Geom &g = x.g;
    const int L = g.L;
    a.con = x.w.con;
    a.con_new = x.w.con2;
    k_tr_load<<<blocks_for((long)g.NC * (L + 2), 256), 256, 0, x.stream>>>(a);
    // FP64 limiter variant 3: face coefficients and limiters per (entity, layer) from the wet
    // cell-layer list, as the FP32 path always runs them (same expressions, same results)
    const bool flat_lim = sizeof(R) == sizeof(float) || (x.tune[TUNE_TR_LIMITER] == 3 && x.w.cl_list);
    // FP64 limiter variants 4 and 5 mix the forms: 4 the cell sums per listed wet cell-layer with
    // the face limiter per face, 5 the cell sums per column with the face limiter per face-layer
    const bool list_sums = !flat_lim && x.tune[TUNE_TR_LIMITER] == 4 && x.w.cl_list;
    const bool flat_faces = !flat_lim && x.tune[TUNE_TR_LIMITER] == 5;
    // variant 6: the column limiter of variant 1 with the face coefficients per face-layer
    const bool flat_coef = flat_lim || x.tune[TUNE_TR_LIMITER] == 6;
    // FP64 solve variant 3: rows per listed wet cell-layer, then one thread per column
    const bool list_solve = sizeof(R) == sizeof(double) && x.tune[TUNE_TR_SOLVE] == 3 && x.w.cl_list && x.w.tr_a;
    if (flat_lim || list_solve || list_sums) {
        cudaError_t e = build_cell_layer_list(g, x.s.top_cell, x.w.cl_off, x.w.cl_bsum, x.w.cl_list, x.w.cl_count,
                                              x.stream);
        if (e != cudaSuccess) return e;
    }

    const int list_grid = x.num_sms * 8;   // grid-stride over the wet cell-layers
    bool lim = p.h_flux_limiter > 0 || p.v_flux_limiter > 0;
    const int bs_solve = x.tune[TUNE_TR_SOLVE] == 1 ? 64 : x.tune[TUNE_TR_SOLVE] == 2 ? 256 : 128;
    const int bs_lim = x.tune[TUNE_TR_LIMITER] == 1 || x.tune[TUNE_TR_LIMITER] >= 5 ? 64
                       : x.tune[TUNE_TR_LIMITER] == 2 ? 256 : 128;
    R *cur = x.w.con, *nxt = x.w.con2;
    for (int sub = 0; sub < a.Nt; ++sub) {
        a.sub = sub;
        a.sub_r = (R)sub;
        a.sub1_r = (R)(sub + 1);
        a.con = cur;
        a.con_new = nxt;
        if (g.NOB + g.NQB > 0) k_tr_bc<<<blocks_for(g.NOB + g.NQB, 128), 128, 0, x.stream>>>(a);
        a.changed_only = sub > 0;
        if (flat_coef)
            k_tr_face_coef_flat<<<blocks_for((long)g.NF * L, 256), 256, 0, x.stream>>>(a);
        else
            k_tr_face_coef<<<blocks_for(g.NF, 128), 128, 0, x.stream>>>(a);
        if constexpr (sizeof(R) == sizeof(float))
            k_tr_cell_coef_list<<<list_grid, 256, 0, x.stream>>>(a);
        else
            k_tr_cell_coef<<<blocks_for(g.NC, 128), 128, 0, x.stream>>>(a);
        if (lim) {
            if (flat_lim) {
                k_tr_sums_list<<<list_grid, bs_lim, 0, x.stream>>>(a);
                k_tr_vpsi_list<<<list_grid, bs_lim, 0, x.stream>>>(a);
                k_tr_limiter_faces_flat<<<blocks_for((long)g.NF * L, 256), 256, 0, x.stream>>>(a);
            } else {
                if (list_sums) {
                    k_tr_sums_list<<<list_grid, bs_lim, 0, x.stream>>>(a);
                    k_tr_vpsi_list<<<list_grid, bs_lim, 0, x.stream>>>(a);
                } else {
                    k_tr_limiter_cells<<<blocks_for(g.NC, bs_lim), bs_lim, 0, x.stream>>>(a);
                }
                if (flat_faces)
                    k_tr_limiter_faces_flat<<<blocks_for((long)g.NF * L, 256), 256, 0, x.stream>>>(a);
                else
                    k_tr_limiter_faces<<<blocks_for(g.NF, 128), 128, 0, x.stream>>>(a);
            }
        }
        if constexpr (sizeof(R) == sizeof(float)) {
            k_tr_rows_list<<<list_grid, bs_solve, 0, x.stream>>>(a);
            k_tr_thomas_col<<<blocks_for(g.NC, 128), 128, 0, x.stream>>>(a);
        } else if (list_solve) {
            if constexpr (sizeof(R) == sizeof(double))
                k_tr_rows64_sorted<<<x.num_sms * 3, ROWS_CHUNK, 0, x.stream>>>(a);
            k_tr_thomas_col<<<blocks_for(g.NC, 128), 128, 0, x.stream>>>(a);
        } else {
            k_tr_solve<<<blocks_for(g.NC, bs_solve), bs_solve, 0, x.stream>>>(a);
        }
        R *t = cur;
        cur = nxt;
        nxt = t;
    }
    a.con = cur;
    if constexpr (sizeof(R) == sizeof(float))
        k_tr_nodes_tile<<<blocks_for(g.NN, NT_TILE), 256, 0, x.stream>>>(a);
    else
        k_tr_nodes<<<blocks_for(g.NN, 128), 128, 0, x.stream>>>(a);
    long n = (long)g.NF * L + (long)g.NC * L;
    k_tr_faces_cells<<<blocks_for(n, 256), 256, 0, x.stream>>>(a);
    return cudaGetLastError();
}

// ============================================================================================
// calculate_density_full.f90:57-100 (default-REAL coefficients) and the linear variant
__device__ __forceinline__ double eos_surface(double rtemp, double rsalt) {
    double t2 = rtemp * rtemp, t3 = t2 * rtemp, t4 = t2 * t2, t5 = t3 * t2;
    double sq = sqrt(rsalt);
    double sq3 = sq * sq * sq;
    const double c0 = (double)(1000.0f - 0.157406f);
    return c0 + F(6.793952e-2f) * rtemp - F(9.095290e-3f) * t2 + F(1.001685e-4f) * t3 - F(1.120083e-6f) * t4 +
           F(6.536332e-9f) * t5 +
           rsalt * (F(0.824493f) - F(4.089900e-3f) * rtemp + F(7.643800e-5f) * t2 - F(8.246700e-7f) * t3 +
                    F(5.387500e-9f) * t4) +
           sq3 * (F(-5.72466e-3f) + F(1.022700e-4f) * rtemp - F(1.654600e-6f) * t2) + F(4.831400e-4f) * (rsalt * rsalt);
}

__device__ __forceinline__ double eos_bulk(double rtemp, double rsalt, double pres) {
    double t2 = rtemp * rtemp, t3 = t2 * rtemp, t4 = t2 * t2;
    double sq = sqrt(rsalt);
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

// one thread per node (kind 0) or face (kind 1) column
template <int KIND, typename R>
__global__ void k_density_col(Geom g, StateT<R> s, Params p, gom_status *st) {
    unsigned tid = flat_tid();
    int n = KIND == 0 ? g.NN : g.NF;
    if (tid >= (unsigned)n) return;
    int e = column_entity<R>(KIND == 0 ? g.node_order : g.face_order, tid);
    const int L = g.L;
    int t = KIND == 0 ? s.top_node[e - 1] : s.top_face[e - 1];
    if (t == 0) return;
    int b = KIND == 0 ? g.bottom_node[e - 1] : g.bottom_face[e - 1];
    double *rho = KIND == 0 ? s.rho_node : s.rho_face;
    const R *tt = KIND == 0 ? s.temp_node : s.temp_face;
    const R *ss = KIND == 0 ? s.salt_node : s.salt_face;
    const R *dz = KIND == 0 ? s.dz_node : s.dz_face;
    const double c981 = F(9.81f), c1e5h = (double)(1.0e-5f * 0.5f), c1e5 = F(1.0e-5f);
    for (int k = b; k <= t; ++k) {
        double rtemp = tt[ix(k, e, L)], rsalt = ss[ix(k, e, L)];
        if (rtemp < -5.0 || rtemp > 100.0 || rsalt < -5.0 || rsalt > 100.0) {
            record_error(st, GOM_E_DENSITY, KIND == 0 ? 43 : 130, e, k, (rtemp < -5.0 || rtemp > 100.0) ? rtemp : rsalt, KIND == 0 ? GOM_ENTITY_NODE : GOM_ENTITY_FACE);
            return;
        }
        double r;
        if (p.ana_density == 1) {
            r = F(1000.0f) + F(0.7f) * rsalt;
        } else {
            r = eos_surface(rtemp, rsalt);
            rho[ix(k, e, L)] = r;
            if (p.msl - g.z_level[k] > F(100.0f)) {
                double pres = 0.0;
                for (int kk = k; kk <= t; ++kk) {
                    double ptmp = c981 * rho[ix(kk, e, L)] * (double)dz[ix(kk, e, L)];
                    pres = pres + (kk == k ? c1e5h : c1e5) * ptmp;
                }
                double sbm = eos_bulk(rtemp, rsalt, pres);
                r = r * (1.0 / (1.0 - pres / sbm));
            }
        }
        rho[ix(k, e, L)] = r;
        if (r < F(980.0f)) {
            record_error(st, GOM_E_DENSITY, KIND == 0 ? 103 : 188, e, k, r, KIND == 0 ? GOM_ENTITY_NODE : GOM_ENTITY_FACE);
            return;
        }
    }
    double rb = rho[ix(b, e, L)], rt = rho[ix(t, e, L)];
    for (int k = 1; k <= b - 1; ++k) rho[ix(k, e, L)] = rb;
    for (int k = t + 1; k <= L; ++k) rho[ix(k, e, L)] = rt;
}

// :207-238 cell density = mean of its wet nodes
template <typename R> __global__ void k_density_cells(Geom g, StateT<R> s, gom_status *st) {
    unsigned tid = flat_tid();
    if (tid >= (unsigned)g.NC) return;
    int i = column_entity<R>(g.cell_order, tid);
    const int L = g.L;
    int t = s.top_cell[i - 1];
    if (t == 0) return;
    int b = g.bottom_cell[i - 1];
    int tq = g.tri_or_quad[i - 1];
    for (int k = b; k <= t; ++k) {
        double r = 0.0;
        int icount = 0;
        for (int l = 1; l <= tq; ++l) {
            int nd = g.cell_node(l, i);
            if (s.top_node[nd - 1] != 0) {
                icount = icount + 1;
                r = r + s.rho_node[ix(k, nd, L)];
            }
        }
        if (icount == 0) {
            record_error(st, GOM_E_DRY, 224, i, k, 0.0, GOM_ENTITY_CELL);
            return;
        }
        s.rho_cell[ix(k, i, L)] = r / icount;
    }
    double rb = s.rho_cell[ix(b, i, L)], rt = s.rho_cell[ix(t, i, L)];
    for (int k = 1; k <= b - 1; ++k) s.rho_cell[ix(k, i, L)] = rb;
    for (int k = t + 1; k <= L; ++k) s.rho_cell[ix(k, i, L)] = rt;
}

template <typename R> cudaError_t launch_density(const LaunchT<R> &x) {
    if (x.p.baroclinic_flag != 1) return cudaSuccess;
    k_density_col<0, R><<<blocks_for(x.g.NN, 128), 128, 0, x.stream>>>(x.g, x.s, x.p, x.status);
    if (x.p.ana_density == 0) k_density_col<1, R><<<blocks_for(x.g.NF, 128), 128, 0, x.stream>>>(x.g, x.s, x.p, x.status);
    k_density_cells<<<blocks_for(x.g.NC, 128), 128, 0, x.stream>>>(x.g, x.s, x.status);
    return cudaGetLastError();
}

// ============================================================================================
// turbulence_closure_v1.f90:72-138, schemes 1 (step function of Ri) and 2 (Pacanowski-Philander).
// The routine names another model's arrays; here srho -> rho_face, velocity_normal/tangnt ->
// un/vn_face_new, dzhalf -> dzhalf_face_new, h_at_face_center -> h_face, ref_water_density ->
// rho_o.  Interface k of a face (top of layer k) gets Av(k) and a face diffusivity; a cell's Kv(k)
// is the mean of its wet faces' diffusivities at the level clamped to each face's wet range
// (the nodal averaging of :446-470 applied to cells), 1e-2 where no face is wet.
// One thread per face column; Ri differences densities in FP64, the rest runs in R.
template <typename R> __global__ void k_turbulence_faces(Geom g, StateT<R> s, Params p, R *kvf) {
    unsigned tid = flat_tid();
    if (tid >= (unsigned)g.NF) return;
    int i = column_entity<R>(g.face_order, tid);
    const int L = g.L;
    int t = s.top_face[i - 1];
    if (t == 0) return;
    int b = g.bottom_face[i - 1];
    R vmax = R(0), vmin = R(0);
    if (p.turbulence_flag == 2) {
        double h = g.h_face[i - 1];
        if (h <= p.pp_h1) {
            vmax = (R)p.pp_vdmax1;
            vmin = (R)p.pp_vdmin1;
        } else if (h < p.pp_h2) {
            vmax = (R)(p.pp_vdmax1 + (p.pp_vdmax2 - p.pp_vdmax1) * (h - p.pp_h1) / (p.pp_h2 - p.pp_h1));
            vmin = (R)(p.pp_vdmin1 + (p.pp_vdmin2 - p.pp_vdmin1) * (h - p.pp_h1) / (p.pp_h2 - p.pp_h1));
        } else {
            vmax = (R)p.pp_vdmax2;
            vmin = (R)p.pp_vdmin2;
        }
    }
    const R gR = (R)p.gravity, rho_o = (R)p.rho_o;
    const R gsound = (R)(p.gravity / (double)(1.5e3f * 1.5e3f));
    const R tdmin = (R)p.pp_tdmin;
    for (int k = b; k <= t; ++k) {
        R ri = R(0);
        if (k != t) {
            R dzh = s.dzhalf_face_new[ix0(k, i, L)];
            R drhodz = (R)(s.rho_face[ix(k + 1, i, L)] - s.rho_face[ix(k, i, L)]) / dzh;
            R bvf = -gR * (drhodz / rho_o + gsound);
            R dundz = (s.un_face_new[ix(k + 1, i, L)] - s.un_face_new[ix(k, i, L)]) / dzh;
            R dutdz = (s.vn_face_new[ix(k + 1, i, L)] - s.vn_face_new[ix(k, i, L)]) / dzh;
            R shear2 = dundz * dundz + dutdz * dutdz;
            shear2 = fmax(shear2, (R)1.0e-10);
            ri = fmax(bvf / shear2, R(0));
        }
        R a, d;
        if (p.turbulence_flag == 1) {
            if (ri < R(0.25)) {
                a = (R)1.0e-3;
                d = (R)1.0e-3;
            } else {
                a = (R)1.0e-5;
                d = (R)1.0e-5;
            }
        } else {
            R x = R(1) + R(5) * ri;
            a = vmax / (x * x) + vmin;
            d = a / (R(1) + R(5) * ri) + tdmin;
        }
        s.av[ix0(k, i, L)] = a;
        kvf[ix0(k, i, L)] = d;
    }
}

template <typename R> __global__ void k_turbulence_cells(Geom g, StateT<R> s, const R *kvf) {
    unsigned tid = flat_tid();
    if (tid >= (unsigned)g.NC) return;
    int i = column_entity<R>(g.cell_order, tid);
    const int L = g.L;
    int t = s.top_cell[i - 1];
    if (t == 0) return;
    int tq = g.tri_or_quad[i - 1];
    int fj[4], fb[4], ft[4];
    for (int l = 1; l <= tq; ++l) {
        fj[l - 1] = g.cell_face(l, i);
        fb[l - 1] = g.bottom_face[fj[l - 1] - 1];
        ft[l - 1] = s.top_face[fj[l - 1] - 1];
    }
    for (int k = g.bottom_cell[i - 1]; k <= t; ++k) {
        R sum = R(0);
        int icount = 0;
        for (int l = 0; l < tq; ++l) {
            if (ft[l] != 0) {
                icount = icount + 1;
                int klev = min(max(k, fb[l]), ft[l]);
                sum = sum + kvf[ix0(klev, fj[l], L)];
            }
        }
        s.kv[ix0(k, i, L)] = icount == 0 ? (R)F(1.0e-2f) : sum / (R)icount;
    }
}

template <typename R> cudaError_t launch_turbulence(const LaunchT<R> &x) {
    if (x.p.turbulence_flag != 1 && x.p.turbulence_flag != 2) return cudaSuccess;
    k_turbulence_faces<<<blocks_for(x.g.NF, 128), 128, 0, x.stream>>>(x.g, x.s, x.p, x.w.kvf);
    k_turbulence_cells<<<blocks_for(x.g.NC, 128), 128, 0, x.stream>>>(x.g, x.s, (const R *)x.w.kvf);
    return cudaGetLastError();
}

// ============================================================================================
// volume and salt mass in FP64: per-block sums, then one block adds the block sums in order.
// A mixed-precision context stores thicknesses in FP32; its sums use the FP64 thickness of each
// wet layer recomputed from the FP64 elevation as update_vertical_layers_1.f90:42-133 forms it,
// so the volume is conserved to the free-surface solve's accuracy, not to FP32 rounding.
template <typename R>
__device__ __forceinline__ double layer_dz64(const Geom &g, const StateT<R> &s, const Params &p, int i, int k, int b,
                                              int t) {
    if (sizeof(R) == sizeof(double)) return (double)s.dz_cell[ix(k, i, g.L)];
    double h = g.h_cell[i - 1], eta = s.eta_cell[i - 1];
    if (t == b) return h + eta;
    if (k == t) return (p.msl + eta) - g.z_level[t - 1];
    if (k == b) return g.z_level[b] - (p.msl - h);
    return g.delta_z[k - 1];
}

template <typename R> __global__ void k_conservation_partial(Geom g, StateT<R> s, Params p, double *part) {
    __shared__ double sv[256], ss[256];
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int L = g.L;
    double v = 0.0, m = 0.0;
    if (i <= g.NC) {
        int t = s.top_cell[i - 1], b = g.bottom_cell[i - 1];
        for (int k = b; k <= t; ++k) {
            double vv = g.area[i - 1] * layer_dz64(g, s, p, i, k, b, t);
            v = v + vv;
            m = m + vv * (double)s.salt_cell[ix(k, i, L)];
        }
    }
    sv[threadIdx.x] = v;
    ss[threadIdx.x] = m;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            sv[threadIdx.x] += sv[threadIdx.x + o];
            ss[threadIdx.x] += ss[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 + 2 * blockIdx.x] = sv[0];
        part[3 + 2 * blockIdx.x] = ss[0];
    }
}

__global__ void k_conservation_final(double *part, int nblocks) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double v = 0.0, m = 0.0;
    for (int b = 0; b < nblocks; ++b) {
        v += part[2 + 2 * b];
        m += part[3 + 2 * b];
    }
    part[0] = v;
    part[1] = m;
}

template <typename R> cudaError_t launch_conservation(const LaunchT<R> &x) {
    int nb = blocks_for(x.g.NC, 256);
    k_conservation_partial<<<nb, 256, 0, x.stream>>>(x.g, x.s, x.p, x.w.cons);
    k_conservation_final<<<1, 32, 0, x.stream>>>(x.w.cons, nb);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------- station series
// write_tser_out_files.f90:9-330: one thread per station forms the station's record
// [eta, H, ubar, u(1:L), vbar, v(1:L), sbar, salt(1:L), tbar, temp(1:L), air pressure] in the
// reference's order of operations (the means are serial sums over the layers, as there), so the
// FP64 path writes the same bits as the reference formulas.
template <typename R>
__global__ void k_station_series(Geom g, StateT<R> s, Forcing f, int hloc, int n, const int *ids, double *out) {
    const int is = blockIdx.x * blockDim.x + threadIdx.x;
    if (is >= n) return;
    const int L = g.L;
    double *o = out + (long)is * (7 + 4 * L);
    double *ou = o + 2, *ov = o + 3 + L, *os = o + 4 + 2 * L, *ot = o + 5 + 3 * L;
    const int e = ids[is];
    if (hloc == 1) {
        const int ie = e;
        const double eta = s.eta_cell[ie - 1];
        o[0] = eta;
        o[1] = g.h_cell[ie - 1] + eta;
        const int t = s.top_cell[ie - 1], b = g.bottom_cell[ie - 1];
        for (int k = 0; k <= L; ++k) ou[k] = ov[k] = 0.0;
        double sb = 0.0, tb = 0.0;
        if (t != 0) {
            // :100-117 (u), :145-162 (v): cell velocity from the node columns, then the depth mean
            const int tq = g.tri_or_quad[ie - 1];
            const int nvl = t - b + 1;
            double ub = 0.0, vb = 0.0;
            for (int k = b; k <= t; ++k) {
                double uc = 0.0, vc = 0.0;
                for (int l = 1; l <= tq; ++l) {
                    const int nd = g.cell_node(l, ie);
                    uc = uc + (double)s.u_node[ix0(k - 1, nd, L)] + (double)s.u_node[ix0(k, nd, L)];
                    vc = vc + (double)s.v_node[ix0(k - 1, nd, L)] + (double)s.v_node[ix0(k, nd, L)];
                }
                uc = uc / (double)(tq * 2);
                vc = vc / (double)(tq * 2);
                ou[k] = uc;
                ov[k] = vc;
            }
            for (int k = b; k <= t; ++k) ub = ub + ou[k];
            for (int k = b; k <= t; ++k) vb = vb + ov[k];
            ou[0] = ub / (double)nvl;
            ov[0] = vb / (double)nvl;
            // :189-195, :239-245
            for (int k = b; k <= t; ++k) sb = sb + (double)s.salt_cell[ix(k, ie, L)];
            for (int k = b; k <= t; ++k) tb = tb + (double)s.temp_cell[ix(k, ie, L)];
            sb = sb / (double)nvl;
            tb = tb / (double)nvl;
        }
        os[0] = sb;
        ot[0] = tb;
        for (int k = 1; k <= L; ++k) {
            os[k] = (double)s.salt_cell[ix(k, ie, L)];
            ot[k] = (double)s.temp_cell[ix(k, ie, L)];
        }
        // :312 reads the node array air_p1 at the cell id
        o[6 + 4 * L] = (ie <= g.NN && f.air_p) ? f.air_p[ie - 1] : 0.0;
    } else {
        const int nd = e;
        const double eta = s.eta_node[nd - 1];
        o[0] = eta;
        o[1] = g.h_node[nd - 1] + eta;
        // update_variables.f90:36-72: depth means of the node columns
        const int t = s.top_node[nd - 1], b = g.bottom_node[nd - 1];
        const int nvl = t - b + 1;
        double ub = 0.0, vb = 0.0, sb = 0.0, tb = 0.0;
        if (nvl != 0) {
            for (int k = b - 1; k <= t; ++k) {
                ub = ub + (double)s.u_node[ix0(k, nd, L)];
                vb = vb + (double)s.v_node[ix0(k, nd, L)];
            }
            ub = ub / (double)(nvl + 1);
            vb = vb / (double)(nvl + 1);
            for (int k = b; k <= t; ++k) {
                sb = sb + (double)s.salt_node[ix(k, nd, L)];
                tb = tb + (double)s.temp_node[ix(k, nd, L)];
            }
            sb = sb / (double)nvl;
            tb = tb / (double)nvl;
        }
        ou[0] = ub;
        ov[0] = vb;
        os[0] = sb;
        ot[0] = tb;
        for (int k = 1; k <= L; ++k) {
            ou[k] = (double)s.u_node[ix0(k, nd, L)];
            ov[k] = (double)s.v_node[ix0(k, nd, L)];
            os[k] = (double)s.salt_node[ix(k, nd, L)];
            ot[k] = (double)s.temp_node[ix(k, nd, L)];
        }
        o[6 + 4 * L] = f.air_p ? f.air_p[nd - 1] : 0.0;
    }
}

template <typename R>
cudaError_t launch_station_series(const LaunchT<R> &x, int hloc, int n, const int *ids, double *out) {
    if (n <= 0) return cudaSuccess;
    k_station_series<<<blocks_for(n, 64), 64, 0, x.stream>>>(x.g, x.s, x.f, hloc, n, ids, out);
    return cudaGetLastError();
}
template cudaError_t launch_station_series<double>(const LaunchT<double> &, int, int, const int *, double *);
template cudaError_t launch_station_series<float>(const LaunchT<float> &, int, int, const int *, double *);

GOM_INSTANTIATE_LAUNCH(launch_transport)
GOM_INSTANTIATE_LAUNCH(launch_tr_solve_only)
GOM_INSTANTIATE_LAUNCH(launch_density)
GOM_INSTANTIATE_LAUNCH(launch_turbulence)
GOM_INSTANTIATE_LAUNCH(launch_conservation)

}  // namespace gom
