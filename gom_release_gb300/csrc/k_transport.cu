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
__device__ __forceinline__ double flip(double q, int sgn) { return sgn > 0 ? q : -q; }
__device__ __forceinline__ bool same_bits(double a, double b) { return __double_as_longlong(a) == __double_as_longlong(b); }

struct TArgs;
__device__ __forceinline__ double divnt(double x, const TArgs &a);

struct TArgs {
    Geom g;
    State s;
    Forcing f;
    Params p;
    Work w;
    gom_status *st;
    int ntr;          // active tracers
    int tid[2];       // tran_id of each slot: 1 salinity, 2 temperature
    int Nt, sub;      // subcycles, current subcycle
    double dt2;
    double inv_nt;    // 1/Nt, used only when Nt is a power of two (exact)
    bool pow2;
    bool changed_only;  // coefficient kernels: refresh only entries whose thickness changes
    const double *con;  // current concentrations
    double *con_new;    // next concentrations (full columns, zero outside the wet range)
};

__device__ __forceinline__ double divnt(double x, const TArgs &a) { return a.pow2 ? x * a.inv_nt : x / a.Nt; }

// :88-173 load tracers into con (0:L+1) with the heat_option 2 surface term
__global__ void k_tr_load(TArgs a) {
    unsigned t = flat_tid();
    const Geom &g = a.g;
    const int L = g.L;
    if (t >= (unsigned)g.NC * (L + 2)) return;
    int i, k;
    split_index(t, L + 2, i, k);
    i += 1;
    for (int tr = 0; tr < a.ntr; ++tr) {
        double v = 0.0;
        if (k >= 1 && k <= L) {
            v = a.tid[tr] == 1 ? a.s.salt_cell[ix(k, i, L)] : a.s.temp_cell[ix(k, i, L)];
            if (a.tid[tr] == 2 && a.p.heat_option == 2) {
                int tl = a.s.top_cell[i - 1];
                if (tl > 0)
                    v = v + a.p.dt * a.f.phi_sw[i - 1] / (a.p.rho_o * 4186.0 * a.s.dz_cell[ix(tl, i, L)]);
            }
        }
        ((double *)a.con)[ic(k, i, tr, L, g.NC)] = v;
    }
}

// :232-397 boundary concentrations of the open-boundary and river cells for this subcycle
__global__ void k_tr_bc(TArgs a) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    const Geom &g = a.g;
    const int L = g.L;
    const double theta = a.p.theta;
    if (t < g.NOB) {
        int i = t + 1;
        int i2 = g.ob_cell_id[i - 1];
        int tl = a.s.top_cell[i2 - 1], b = g.bottom_cell[i2 - 1];
        for (int k = 1; k <= L; ++k)
            for (int tr = 0; tr < a.ntr; ++tr) a.w.obk[((long)tr * g.NOB + i - 1) * L + k - 1] = 0.0;
        int tq = g.tri_or_quad[i2 - 1];
        for (int l = 1; l <= tq; ++l) {
            int j2 = g.cell_face(l, i2);
            if (g.boundary_type_of_face[j2 - 1] <= 0) continue;
            int sg = g.cell_sign(l, i2);
            for (int k = b; k <= tl; ++k) {
                double dzf = a.s.dz_face[ix(k, j2, L)];
                double dz_old = dzf + divnt((a.s.dz_face_new[ix(k, j2, L)] - dzf) * a.sub, a);
                double q2 = g.face_length[j2 - 1] * dz_old *
                            (flip((1.0 - theta) * a.s.un_face[ix(k, j2, L)], sg) + flip(theta * a.s.un_face_new[ix(k, j2, L)], sg));
                for (int tr = 0; tr < a.ntr; ++tr) {
                    double bc = a.f.con_at_ob[((long)a.sub * 2 + (a.tid[tr] - 1)) * g.NOB + (i - 1)];
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
                double v = 0.0;
                if (k >= b && k <= tl) v = a.f.con_at_qb[((long)a.sub * 2 + (a.tid[tr] - 1)) * g.NQB + (i - 1)];
                a.w.qbk[((long)tr * g.NQB + i - 1) * L + k - 1] = v;
            }
    }
}

// :551-581 face coefficients.  One thread per face walks its wet layers, so the FP64 work of a
// warp is spread over 32 wet faces (GB300 issues an FP64 warp instruction at the same cost however
// few lanes are active).  Later subcycles refresh only layers whose thickness changes.
__device__ __forceinline__ void face_coef_at(const TArgs &a, int j, int k, long t) {
    double dzf = a.s.dz_face[t];
    double dz_old = dzf + divnt((a.s.dz_face_new[t] - dzf) * a.sub, a);
    double fl = a.g.face_length[j - 1];
    double Q = fl * dz_old * ((1.0 - a.p.theta) * a.s.un_face[t] + a.p.theta * a.s.un_face_new[t]);
    double D = fl * dz_old * a.s.kh[t] / a.g.delta_j[j - 1];
    double d = fmax(0.0, D - 0.5 * fabs(Q));
    double phi = Q == 0.0 ? 1.0 : fmin(1.0, 2.0 * D / fabs(Q));
    a.w.qj[t] = Q;
    a.w.dj[t] = d;
    a.w.phij[t] = phi;
}

__global__ void k_tr_face_coef(TArgs a) {
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
                a.w.qj[t] = 0.0;
                a.w.dj[t] = 0.0;
                a.w.phij[t] = 0.0;
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
__device__ __forceinline__ void cell_coef_at(const TArgs &a, int i, long t) {
    double ar = a.g.area[i - 1];
    double Q = ar * ((1.0 - a.p.theta) * a.s.wn_cell[t] + a.p.theta * a.s.wn_cell_new[t]);
    double dzh = a.s.dzhalf_cell[t];
    double dz_old = dzh + divnt((a.s.dzhalf_cell_new[t] - dzh) * a.sub, a);
    double D = ar * a.s.kv[t] / dz_old;
    a.w.qi[t] = Q;
    a.w.di[t] = fmax(0.0, D - 0.5 * fabs(Q));
    a.w.phii[t] = Q == 0.0 ? 1.0 : fmin(1.0, 2.0 * D / fabs(Q));
}

__global__ void k_tr_cell_coef(TArgs a) {
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
                a.w.qi[t] = 0.0;
                a.w.di[t] = 0.0;
                a.w.phii[t] = 0.0;
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
__device__ __forceinline__ double oqb_value(const TArgs &a, int i, int k, int tr) {
    const Geom &g = a.g;
    int ith_qb = g.qb_element_flag[i - 1];
    if (ith_qb > 0) return a.w.qbk[((long)tr * g.NQB + ith_qb - 1) * g.L + k - 1];
    int ith_ob = g.ob_element_flag[i - 1];
    if (ith_ob > 0) return a.w.obk[((long)tr * g.NOB + ith_ob - 1) * g.L + k - 1];
    return 0.0;
}

__device__ __forceinline__ double phi_limit(int code, double small_phi, double r) {
    switch (code) {
    case 1: return fmax(small_phi, fmin(1.0, r)) - small_phi;
    case 2: return fmax(small_phi, (r + fabs(r)) / (1.0 + fabs(r))) - small_phi;
    case 3: return fmax(fmax(small_phi, fmin(1.0, 2.0 * r)), fmin(2.0, r)) - small_phi;
    default: return 0.0;
    }
}

// :624-871 per cell column: upwind-weighted differences of every layer (sum1_all, sum2_all) for
// the face ratios r_jk, and the vertical ratios r_ik -> PSI_ik.
__global__ void k_tr_limiter_cells(TArgs a) {
    unsigned tid = flat_tid();
    const Geom &g = a.g;
    if (tid >= (unsigned)g.NC) return;
    int i = g.cell_order[tid];
    const int L = g.L, NC = g.NC;
    int tl = a.s.top_cell[i - 1], b = g.bottom_cell[i - 1];
    if (tl == 0) return;
    int nvl = tl - b + 1;
    int tq = g.tri_or_quad[i - 1];
    int fj[4], nb[4], sg[4];
    bool open[4];
    for (int l = 1; l <= tq; ++l) {
        fj[l - 1] = g.cell_face(l, i);
        nb[l - 1] = g.cell_adj(l, i);
        sg[l - 1] = g.cell_sign(l, i);
        open[l - 1] = face_open(g, fj[l - 1]);
    }
    double last1[2] = {0.0, 0.0}, last2[2] = {0.0, 0.0};
    for (int k = b; k <= tl; ++k) {
        double s1a[2] = {0.0, 0.0}, s2a[2] = {0.0, 0.0}, s1[2] = {0.0, 0.0}, s2[2] = {0.0, 0.0};
        for (int tr = 0; tr < a.ntr; ++tr) {
            double ck = a.con[ic(k, i, tr, L, NC)];
            if (nvl != 1) {
                if (k == b) {
                    double rt2 = pos_part(a.w.qi[ix0(k, i, L)]);
                    s1a[tr] = rt2 * (ck - a.con[ic(k + 1, i, tr, L, NC)]);
                    s2a[tr] = rt2;
                } else if (k == tl) {
                    double rt1 = pos_part(a.w.qi[ix0(k - 1, i, L)]);
                    s1a[tr] = rt1 * (ck - a.con[ic(k - 1, i, tr, L, NC)]);
                    s2a[tr] = rt1;
                } else {
                    double rt1 = pos_part(a.w.qi[ix0(k - 1, i, L)]);
                    double rt2 = pos_part(a.w.qi[ix0(k, i, L)]);
                    s1a[tr] = rt1 * (ck - a.con[ic(k - 1, i, tr, L, NC)]) + rt2 * (ck - a.con[ic(k + 1, i, tr, L, NC)]);
                    s2a[tr] = rt1 + rt2;
                }
            }
        }
        for (int l = 0; l < tq; ++l) {
            if (!open[l]) continue;
            double q2 = flip(a.w.qj[ix(k, fj[l], L)], sg[l]);
            if (is_neg(q2)) {
                for (int tr = 0; tr < a.ntr; ++tr) {
                    double cik = nb[l] > 0 ? a.con[ic(k, nb[l], tr, L, NC)] : oqb_value(a, i, k, tr);
                    s1[tr] = s1[tr] + fabs(q2) * (a.con[ic(k, i, tr, L, NC)] - cik);
                    s2[tr] = s2[tr] + fabs(q2);
                }
            }
        }
        for (int tr = 0; tr < a.ntr; ++tr) {
            s1a[tr] = s1a[tr] + s1[tr];
            s2a[tr] = s2a[tr] + s2[tr];
            a.w.sa1[((long)tr * NC + i - 1) * L + k - 1] = s1a[tr];
            a.w.sa2[((long)tr * NC + i - 1) * L + k - 1] = s2a[tr];
            last1[tr] = s1[tr];
            last2[tr] = s2[tr];
        }
    }
    // :806-840 (Q_ik_theta at the top interface is never assigned: 0 -> first branch)
    for (int tr = 0; tr < a.ntr; ++tr) {
        double *psi = a.w.psii + (long)tr * NC * (L + 1);
        for (int k = b; k <= tl - 1; ++k) {
            double qm = (k - 1 >= b) ? a.w.qi[ix0(k - 1, i, L)] : 0.0;
            double ck = a.con[ic(k, i, tr, L, NC)];
            double rt1 = last1[tr] + fabs(qm) * (ck - a.con[ic(k - 1, i, tr, L, NC)]);
            double rt2 = last2[tr] + fabs(qm);
            double rtemp = (a.con[ic(k + 1, i, tr, L, NC)] - ck) * rt2;
            double r = rtemp == 0.0 ? 1.0 : rt1 / rtemp;
            psi[ix0(k, i, L)] = phi_limit(a.p.h_flux_limiter, a.w.phii[ix0(k, i, L)], r);
        }
    }
}

// :769-799 + :876-900 face ratio r_jk from its upwind cell (the last writer in cell order), PSI_jk;
// one thread per face walks its wet layers
__global__ void k_tr_limiter_faces(TArgs a) {
    unsigned tid = flat_tid();
    const Geom &g = a.g;
    if (tid >= (unsigned)g.NF) return;
    int j = g.face_order[tid];
    const int L = g.L, NC = g.NC;
    int b = g.bottom_face[j - 1], tf = a.s.top_face[j - 1];
    if (tf == 0) return;
    bool open = face_open(g, j);
    int c1 = g.face_cell(1, j), c2 = g.face_cell(2, j);
    int t1 = a.s.top_cell[c1 - 1], b1 = g.bottom_cell[c1 - 1];
    int t2 = c2 != 0 ? a.s.top_cell[c2 - 1] : 0, b2 = c2 != 0 ? g.bottom_cell[c2 - 1] : 0;
    for (int k = b; k <= tf; ++k) {
        long t = ix(k, j, L);
        double Q = a.w.qj[t];
        int writer = 0;
        if (open) {
            // a cell writes when it is wet, holds layer k and sees Q*sign >= 0; cell 2 comes later
            if (c2 != 0 && t2 != 0 && k >= b2 && k <= t2 && !is_pos(Q)) writer = c2;   // -Q >= 0
            else if (t1 != 0 && k >= b1 && k <= t1 && !is_neg(Q)) writer = c1;        // Q >= 0
        }
        for (int tr = 0; tr < a.ntr; ++tr) {
            double r = 1.0;
            if (writer != 0) {
                int i = writer;
                int other = (writer == c1) ? c2 : c1;
                double cik = other > 0 ? a.con[ic(k, other, tr, L, NC)] : oqb_value(a, i, k, tr);
                double rtemp = a.w.sa2[((long)tr * NC + i - 1) * L + k - 1] * (cik - a.con[ic(k, i, tr, L, NC)]);
                r = rtemp == 0.0 ? 1.0 : a.w.sa1[((long)tr * NC + i - 1) * L + k - 1] / rtemp;
            }
            a.w.psij[(long)tr * g.NF * L + t] = phi_limit(a.p.h_flux_limiter, a.w.phij[t], r);
        }
    }
}

// :921-1346 per cell column: explicit horizontal fluxes + limiter, implicit vertical system,
// Thomas solve, clamp to [0, 50]; writes the full next column (zero outside the wet range).
__global__ void __launch_bounds__(128) k_tr_solve(TArgs a) {
    unsigned tid = flat_tid();
    const Geom &g = a.g;
    if (tid >= (unsigned)g.NC) return;
    int i = g.cell_order[tid];
    const int L = g.L, NC = g.NC;
    int tl = a.s.top_cell[i - 1], b = g.bottom_cell[i - 1];
    const double dt2 = a.dt2;
    const int Nt = a.Nt, sub = a.sub;
    const bool lim = a.p.h_flux_limiter > 0 || a.p.v_flux_limiter > 0;
    if (tl == 0) {
        for (int k = 0; k <= L + 1; ++k)
            for (int tr = 0; tr < a.ntr; ++tr) a.con_new[ic(k, i, tr, L, NC)] = 0.0;
        return;
    }
    int nvl = tl - b + 1;
    double ar = g.area[i - 1];
    double am[GOM_MAXL], bm[GOM_MAXL], cm[GOM_MAXL], gm[GOM_MAXL];
    double rhs[GOM_MAXL][2];
    for (int k = b + 1; k <= tl - 1; ++k) {
        int kk = tl + 1 - k;
        am[kk - 1] = -dt2 * a.w.di[ix0(k, i, L)];
        cm[kk - 1] = -dt2 * a.w.di[ix0(k - 1, i, L)];
        double dzc = a.s.dz_cell[ix(k, i, L)];
        double dz_new = dzc + divnt((a.s.dz_cell_new[ix(k, i, L)] - dzc) * (sub + 1), a);
        bm[kk - 1] = -am[kk - 1] + ar * dz_new - cm[kk - 1];
    }
    {
        double dzc = a.s.dz_cell[ix(tl, i, L)];
        double dz_new = dzc + divnt((a.s.dz_cell_new[ix(tl, i, L)] - dzc) * (sub + 1), a);
        if (tl == b) {
            bm[0] = ar * dz_new;
        } else {
            cm[0] = -dt2 * a.w.di[ix0(tl - 1, i, L)];
            bm[0] = ar * dz_new - cm[0];
            am[nvl - 1] = -dt2 * a.w.di[ix0(b, i, L)];
            double dzb = a.s.dz_cell[ix(b, i, L)];
            double dz_newb = dzb + divnt((a.s.dz_cell_new[ix(b, i, L)] - dzb) * (sub + 1), a);
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
        double sQi[2] = {0, 0}, sQii[2] = {0, 0}, shd[2] = {0, 0}, shl[2] = {0, 0};
        double ck[2];
        for (int tr = 0; tr < a.ntr; ++tr) ck[tr] = a.con[ic(k, i, tr, L, NC)];
        for (int l = 0; l < tq; ++l) {
            if (!open[l]) continue;
            bool in_face = k >= fb[l] && k <= ft[l];
            long fo = ix(k, fj[l], L);
            double q2 = flip(in_face ? a.w.qj[fo] : 0.0, sg[l]);
            double dface = in_face ? a.w.dj[fo] : 0.0;
            bool qpos = is_pos(q2), qneg = is_neg(q2);
            for (int tr = 0; tr < a.ntr; ++tr) {
                double cik = nb[l] > 0 ? a.con[ic(k, nb[l], tr, L, NC)] : oqb_value(a, i, k, tr);
                if (qpos) sQi[tr] = sQi[tr] + fabs(q2) * ck[tr];
                else if (qneg) sQii[tr] = sQii[tr] + fabs(q2) * cik;
                shd[tr] = shd[tr] + dface * (cik - ck[tr]);
                double psi = (lim && in_face) ? a.w.psij[(long)tr * g.NF * L + fo] : 0.0;
                shl[tr] = shl[tr] + psi * fabs(q2) * (ck[tr] - cik);
            }
        }
        double dzc = a.s.dz_cell[ix(k, i, L)];
        double dz_old = dzc + divnt((a.s.dz_cell_new[ix(k, i, L)] - dzc) * sub, a);
        for (int tr = 0; tr < a.ntr; ++tr) {
            double h_adv = dt2 * (sQii[tr] - sQi[tr]);
            double h_diff = dt2 * shd[tr];
            double h_flux = 0.5 * dt2 * shl[tr];
            double v = ar * dz_old * ck[tr] + h_adv + h_diff;
            if (a.p.h_flux_limiter > 0) v = v + h_flux;
            rhs[kk - 1][tr] = v;
        }
    }
    if (nvl != 1) {
        for (int k = b; k <= tl; ++k) {
            int kk = tl + 1 - k;
            for (int tr = 0; tr < a.ntr; ++tr) {
                const double *psi = a.w.psii + (long)tr * NC * (L + 1);
                double c0 = a.con[ic(k, i, tr, L, NC)];
                double v = rhs[kk - 1][tr];
                if (k == b) {
                    double q = a.w.qi[ix0(k, i, L)];
                    double qp = pos_part(q), qm = neg_part(q);
                    double cp1 = a.con[ic(k + 1, i, tr, L, NC)];
                    v = v + dt2 * (-qp * c0 + qm * cp1);
                    if (a.p.v_flux_limiter > 0) {
                        double ps = lim ? psi[ix0(k, i, L)] : 0.0;
                        v = v + 0.5 * dt2 * (-ps * qp * (cp1 - c0) + ps * qm * (c0 - cp1));
                    }
                } else if (k == tl) {
                    double q = a.w.qi[ix0(k - 1, i, L)];
                    double qp = pos_part(q), qm = neg_part(q);
                    double cm1 = a.con[ic(k - 1, i, tr, L, NC)];
                    v = v + dt2 * (qp * cm1 - qm * c0);
                    if (a.p.v_flux_limiter > 0) {
                        double ps = lim ? psi[ix0(k - 1, i, L)] : 0.0;
                        v = v + 0.5 * dt2 * (ps * qp * (c0 - cm1) - ps * qm * (cm1 - c0));
                    }
                } else {
                    double q1 = a.w.qi[ix0(k - 1, i, L)], q = a.w.qi[ix0(k, i, L)];
                    double qp1 = pos_part(q1), qm1 = neg_part(q1);
                    double qp = pos_part(q), qm = neg_part(q);
                    double cm1 = a.con[ic(k - 1, i, tr, L, NC)], cp1 = a.con[ic(k + 1, i, tr, L, NC)];
                    v = v + dt2 * (qp1 * cm1 - qp * c0 + qm * cp1 - qm1 * c0);
                    if (a.p.v_flux_limiter > 0) {
                        double p1 = lim ? psi[ix0(k - 1, i, L)] : 0.0, p0 = lim ? psi[ix0(k, i, L)] : 0.0;
                        v = v + 0.5 * dt2 *
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
        double r1[GOM_MAXL][1];
        for (int k = 0; k < nvl; ++k) r1[k][0] = rhs[k][0];
        okp = thomas<1>(nvl, am, bm, cm, r1, gm);
        for (int k = 0; k < nvl; ++k) rhs[k][0] = r1[k][0];
    }
    if (!okp) {
        record_error(a.st, GOM_E_ZERO_PIVOT, 1285, i, 0, 0.0);
        return;
    }
    for (int tr = 0; tr < a.ntr; ++tr) {
        for (int k = 0; k <= L + 1; ++k) {
            double v = 0.0;
            if (k >= b && k <= tl) {
                double sv = rhs[tl - k][tr];
                if (sv >= 0.0 && sv <= 50.0) v = sv;
                else if (sv < 0.0) v = 0.0;
                else if (sv > 50.0) v = 50.0;
                else v = a.con[ic(k, i, tr, L, NC)];   // NaN: the reference keeps the previous value
            }
            a.con_new[ic(k, i, tr, L, NC)] = v;
        }
    }
}

// :1403-1454 node averages (column, top-down) and :1457-1482 face averages + write-back
__global__ void k_tr_nodes(TArgs a) {
    unsigned tid = flat_tid();
    const Geom &g = a.g;
    if (tid >= (unsigned)g.NN) return;
    int i = g.node_order[tid];
    const int L = g.L, NC = g.NC;
    int tn = a.s.top_node[i - 1], bn = g.bottom_node[i - 1];
    int na = g.adj_cells_at_node[i - 1];
    for (int tr = 0; tr < a.ntr; ++tr) {
        double *dst = a.tid[tr] == 1 ? a.s.salt_node : a.s.temp_node;
        bool write = a.tid[tr] <= a.ntr;   // slot 1 -> salt, slot 2 -> temperature
        double above = 0.0;
        for (int k = L; k >= 1; --k) {
            double v = 0.0;
            if (tn != 0 && k <= tn && k >= bn) {
                double s11 = 0.0, s22 = 0.0;
                int count1 = 0;
                for (int l = 1; l <= na; ++l) {
                    int ii = g.node_cell(l, i);
                    if (k >= g.bottom_cell[ii - 1] && k <= a.s.top_cell[ii - 1]) {
                        double w = g.area[ii - 1] * a.s.dz_cell_new[ix(k, ii, L)];
                        s11 = s11 + w;
                        s22 = s22 + w * a.con[ic(k, ii, tr, L, NC)];
                    } else {
                        count1 = count1 + 1;
                    }
                }
                v = s11 == 0.0 ? 0.0 : s22 / s11;
                if (count1 == na && k != tn) v = above;
            }
            if (write) dst[ix(k, i, L)] = v;
            above = v;
        }
    }
}

__global__ void k_tr_faces_cells(TArgs a) {
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
            const double *src = a.tid[tr] == 1 ? a.s.salt_node : a.s.temp_node;
            double *dst = a.tid[tr] == 1 ? a.s.salt_face : a.s.temp_face;
            dst[t] = in ? (src[ix(k, n1, L)] + src[ix(k, n2, L)]) * 0.5 : 0.0;
        }
    } else if (t < nfl + ncl) {
        unsigned u = t - nfl;
        int i, k;
        split_index(u, L, i, k);
        i += 1;
        k += 1;
        for (int tr = 0; tr < a.ntr; ++tr) {
            if (a.tid[tr] > a.ntr) continue;
            double *dst = a.tid[tr] == 1 ? a.s.salt_cell_new : a.s.temp_cell_new;
            dst[u] = a.con[ic(k, i, tr, L, NC)];
        }
    }
}

cudaError_t launch_transport(const Launch &x) {
    const Params &p = x.p;
    if (!p.transport_flag) return cudaSuccess;
    TArgs a;
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
    a.dt2 = p.dt / a.Nt;
    a.pow2 = (a.Nt & (a.Nt - 1)) == 0;
    a.inv_nt = 1.0 / a.Nt;
    a.changed_only = false;
    const Geom &g = x.g;
    const int L = g.L;
    a.con = x.w.con;
    a.con_new = x.w.con2;
    k_tr_load<<<blocks_for((long)g.NC * (L + 2), 256), 256, 0, x.stream>>>(a);
    bool lim = p.h_flux_limiter > 0 || p.v_flux_limiter > 0;
    double *cur = x.w.con, *nxt = x.w.con2;
    for (int sub = 0; sub < a.Nt; ++sub) {
        a.sub = sub;
        a.con = cur;
        a.con_new = nxt;
        if (g.NOB + g.NQB > 0) k_tr_bc<<<blocks_for(g.NOB + g.NQB, 128), 128, 0, x.stream>>>(a);
        a.changed_only = sub > 0;
        k_tr_face_coef<<<blocks_for(g.NF, 128), 128, 0, x.stream>>>(a);
        k_tr_cell_coef<<<blocks_for(g.NC, 128), 128, 0, x.stream>>>(a);
        if (lim) {
            k_tr_limiter_cells<<<blocks_for(g.NC, 128), 128, 0, x.stream>>>(a);
            k_tr_limiter_faces<<<blocks_for(g.NF, 128), 128, 0, x.stream>>>(a);
        }
        k_tr_solve<<<blocks_for(g.NC, 128), 128, 0, x.stream>>>(a);
        double *t = cur;
        cur = nxt;
        nxt = t;
    }
    a.con = cur;
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
template <int KIND>
__global__ void k_density_col(Geom g, State s, Params p, gom_status *st) {
    unsigned tid = flat_tid();
    int n = KIND == 0 ? g.NN : g.NF;
    if (tid >= (unsigned)n) return;
    int e = KIND == 0 ? g.node_order[tid] : g.face_order[tid];
    const int L = g.L;
    int t = KIND == 0 ? s.top_node[e - 1] : s.top_face[e - 1];
    if (t == 0) return;
    int b = KIND == 0 ? g.bottom_node[e - 1] : g.bottom_face[e - 1];
    double *rho = KIND == 0 ? s.rho_node : s.rho_face;
    const double *tt = KIND == 0 ? s.temp_node : s.temp_face;
    const double *ss = KIND == 0 ? s.salt_node : s.salt_face;
    const double *dz = KIND == 0 ? s.dz_node : s.dz_face;
    const double c981 = F(9.81f), c1e5h = (double)(1.0e-5f * 0.5f), c1e5 = F(1.0e-5f);
    for (int k = b; k <= t; ++k) {
        double rtemp = tt[ix(k, e, L)], rsalt = ss[ix(k, e, L)];
        if (rtemp < -5.0 || rtemp > 100.0 || rsalt < -5.0 || rsalt > 100.0) {
            record_error(st, GOM_E_DENSITY, KIND == 0 ? 43 : 130, e, k, (rtemp < -5.0 || rtemp > 100.0) ? rtemp : rsalt);
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
                    double ptmp = c981 * rho[ix(kk, e, L)] * dz[ix(kk, e, L)];
                    pres = pres + (kk == k ? c1e5h : c1e5) * ptmp;
                }
                double sbm = eos_bulk(rtemp, rsalt, pres);
                r = r * (1.0 / (1.0 - pres / sbm));
            }
        }
        rho[ix(k, e, L)] = r;
        if (r < F(980.0f)) {
            record_error(st, GOM_E_DENSITY, KIND == 0 ? 103 : 188, e, k, r);
            return;
        }
    }
    double rb = rho[ix(b, e, L)], rt = rho[ix(t, e, L)];
    for (int k = 1; k <= b - 1; ++k) rho[ix(k, e, L)] = rb;
    for (int k = t + 1; k <= L; ++k) rho[ix(k, e, L)] = rt;
}

// :207-238 cell density = mean of its wet nodes
__global__ void k_density_cells(Geom g, State s, gom_status *st) {
    unsigned tid = flat_tid();
    if (tid >= (unsigned)g.NC) return;
    int i = g.cell_order[tid];
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
            record_error(st, GOM_E_DRY, 224, i, k, 0.0);
            return;
        }
        s.rho_cell[ix(k, i, L)] = r / icount;
    }
    double rb = s.rho_cell[ix(b, i, L)], rt = s.rho_cell[ix(t, i, L)];
    for (int k = 1; k <= b - 1; ++k) s.rho_cell[ix(k, i, L)] = rb;
    for (int k = t + 1; k <= L; ++k) s.rho_cell[ix(k, i, L)] = rt;
}

cudaError_t launch_density(const Launch &x) {
    if (x.p.baroclinic_flag != 1) return cudaSuccess;
    k_density_col<0><<<blocks_for(x.g.NN, 128), 128, 0, x.stream>>>(x.g, x.s, x.p, x.status);
    if (x.p.ana_density == 0) k_density_col<1><<<blocks_for(x.g.NF, 128), 128, 0, x.stream>>>(x.g, x.s, x.p, x.status);
    k_density_cells<<<blocks_for(x.g.NC, 128), 128, 0, x.stream>>>(x.g, x.s, x.status);
    return cudaGetLastError();
}

// ============================================================================================
// volume and salt mass in FP64: per-block sums, then one block adds the block sums in order
__global__ void k_conservation_partial(Geom g, State s, double *part) {
    __shared__ double sv[256], ss[256];
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int L = g.L;
    double v = 0.0, m = 0.0;
    if (i <= g.NC) {
        int t = s.top_cell[i - 1];
        for (int k = g.bottom_cell[i - 1]; k <= t; ++k) {
            double vv = g.area[i - 1] * s.dz_cell[ix(k, i, L)];
            v = v + vv;
            m = m + vv * s.salt_cell[ix(k, i, L)];
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

cudaError_t launch_conservation(const Launch &x) {
    int nb = blocks_for(x.g.NC, 256);
    k_conservation_partial<<<nb, 256, 0, x.stream>>>(x.g, x.s, x.w.cons);
    k_conservation_final<<<1, 32, 0, x.stream>>>(x.w.cons, nb);
    return cudaGetLastError();
}

}  // namespace gom
