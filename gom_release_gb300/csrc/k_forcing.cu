// k_forcing.cu -- per-step storm-surge forcing evaluated on the device, so that a step of a
// storm-surge context (one run or a packed ensemble) needs no host-to-device traffic.
//
// What the Fortran driver computes on the host every step (GOM_Rv1.1.0/source):
//   setup_spinup.f90:22-31            tanh spin-up ramp,
//   holland_storm_surge.f90:131-232   vortex winds, air pressure, inverse-barometer set-up,
//   calculate_wind_stress.f90:105-137 wind drag law (wind_formular 1, Cd <= 0.003),
//   compute_boundary_eta.f90:72-90    harmonic tide at the open boundary.
// The vortex follows holland_storm_surge.f90 (gradient wind from the cyclostrophic and
// geostrophic speeds with the translation asymmetry, 0.95 gradient-to-surface factor, 18 degree
// inflow, face wind = mean of its two node winds) with a Holland exponent b in the profile
// (Holland 1980: V_c^2 = b dp / rho_a (rmax/r)^b exp(-(rmax/r)^b)); the reference fixes b = 1.
#include "gom_launch.h"

namespace gom {

namespace {

constexpr double kAirDensity = 1.293;       // holland_storm_surge.f90:27
constexpr double kGradToSurface = 0.95;     // holland_storm_surge.f90:28
constexpr double kPFar = 101300.0;          // holland_storm_surge.f90:29, Pa
constexpr double kInflow = 18.0 * 3.141592653589793 / 180.0;
constexpr int kStormDoubles = 13;           // gom_storm

struct StormView {
    double x0, y0, heading, speed, rmax, dp, b, coriolis, amp, period, phase, spinup, t0;
};

__device__ __forceinline__ StormView storm_at(const double *s, int r) {
    const double *p = s + (long)r * kStormDoubles;
    return StormView{p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8], p[9], p[10], p[11], p[12]};
}

// run holding entity e (0-based) given the runs' first entities
__device__ __forceinline__ int run_of(const int *start, int nr, int e) {
    if (nr <= 1) return 0;
    int lo = 0, hi = nr;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (start[mid] <= e) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ double spin_at(const StormView &s, double t) {
    if (s.spinup <= 0.0 || t >= s.spinup) return 1.0;
    return tanh(2.0 * t / s.spinup);
}

// surface wind (u, v) and air pressure at (x, y), time t
__device__ void vortex(const StormView &s, double t, double x, double y, double &u, double &v, double &p) {
    double ct, st;
    sincos(s.heading, &st, &ct);
    double xe = s.x0 + s.speed * t * ct, ye = s.y0 + s.speed * t * st;
    double dx = x - xe, dy = y - ye;
    double r = fmax(sqrt(dx * dx + dy * dy), 1.0);
    double a = pow(s.rmax / r, s.b);
    double e = exp(-a);
    p = kPFar - s.dp * (1.0 - e);
    double vc2 = s.b * s.dp / kAirDensity * a * e;
    double vc = sqrt(vc2);
    double th = atan2(dy, dx) - s.heading;
    double w = 0.0;
    if (vc >= 1e-3) {
        double vg = vc2 / (r * s.coriolis);
        double gamma = 0.5 * (s.speed * sin(th) / vc + vc / vg);
        w = vc * (sqrt(gamma * gamma + 1.0) - gamma) * kGradToSurface;
    }
    double sa, ca;
    sincos(0.5 * 3.141592653589793 + th + s.heading + kInflow, &sa, &ca);
    u = w * ca;
    v = w * sa;
}

__global__ void k_forcing_clock(double *scal, double dt) {
    if (threadIdx.x == 0 && blockIdx.x == 0) scal[0] = scal[0] + dt;
}

__global__ void k_storm_nodes(Geom g, const double *scal, const double *storms, double *wu, double *wv, double *air_p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.NN) return;
    StormView s = storm_at(storms, run_of(g.run_node_start, g.NR, i));
    double u, v, p;
    vortex(s, scal[0] - s.t0, g.x_node[i], g.y_node[i], u, v, p);
    wu[i] = u;
    wv[i] = v;
    air_p[i] = p;
}

__global__ void k_storm_faces(Geom g, const double *scal, const double *storms, const double *wu, const double *wv,
                              double rho_ratio, double *wsn, double *wst, double *gamma_t) {
    int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (j > g.NF) return;
    StormView s = storm_at(storms, run_of(g.run_face_start, g.NR, j - 1));
    double spin = spin_at(s, scal[0] - s.t0);
    int n1 = g.face_node(1, j), n2 = g.face_node(2, j);
    double u = (wu[n1 - 1] + wu[n2 - 1]) / 2.0, v = (wv[n1 - 1] + wv[n2 - 1]) / 2.0;
    double speed = sqrt(u * u + v * v);
    double ct = g.cos_theta[j - 1], sn = g.sin_theta[j - 1];
    double normal = u * ct + v * sn, tangent = -u * sn + v * ct;
    double cda = fmin(0.001 * (0.75 + 0.067 * speed), (double)0.003f);   // MIN with a default-REAL 0.003
    double gt = cda * rho_ratio * speed;
    wsn[j - 1] = gt * normal * spin;
    wst[j - 1] = gt * tangent * spin;
    gamma_t[j - 1] = gt;
}

__device__ __forceinline__ double ob_elevation(const StormView &s, double t, double x, double y, double rho_g) {
    double u, v, p;
    vortex(s, t, x, y, u, v, p);
    double tide = s.amp * cos(2.0 * 3.141592653589793 * t / s.period + s.phase);
    return spin_at(s, t) * (tide + (kPFar - p) / rho_g);
}

__global__ void k_storm_ob(Geom g, const double *scal, const double *storms, double rho_g, double dt, double *eta_old,
                           double *eta_new) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.NOB) return;
    StormView s = storm_at(storms, run_of(g.run_ob_start, g.NR, i));
    int cell = g.ob_cell_id[i];
    double x = g.x_cell[cell - 1], y = g.y_cell[cell - 1], t = scal[0] - s.t0;
    eta_old[i] = ob_elevation(s, t - dt, x, y, rho_g);
    eta_new[i] = ob_elevation(s, t, x, y, rho_g);
}

// ---------------------------------------------------------------------------- boundary series
// The value of series id (1-based) of one kind at model time u2: the first interval of the
// reference's search (compute_boundary_eta.f90:100-111, calculate_Q.f90:30-41,
// solve_transport_equation_v19.f90:245-257) with u1 <= u2 <= u3 on times minus reference_diff_days,
// found by bisection (series times never decrease, checked when they are set), and
// v2 = (u2 - u1)(v3 - v1)/(u3 - u1) + v1.  False when no interval holds u2.
__device__ bool series_at(const SeriesDev &S, int kind, int id, double u2, double &v) {
    if (id < 1 || id > S.n[kind]) return false;
    const int s0 = S.start[kind][id - 1], n = S.start[kind][id] - s0;
    const double *t = S.time[kind] + s0, *val = S.value[kind] + s0;
    if (n < 2) return false;
    int lo = 0, hi = n;   // first index with t - rdd >= u2
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (t[mid] - S.rdd_s >= u2) hi = mid;
        else lo = mid + 1;
    }
    int k;
    if (lo == 0) {
        if (!(t[0] - S.rdd_s == u2)) return false;
        k = 1;
    } else if (lo >= n) {
        return false;
    } else {
        k = lo;
    }
    const double u1 = t[k - 1] - S.rdd_s, u3 = t[k] - S.rdd_s;
    v = (u2 - u1) * (val[k] - val[k - 1]) / (u3 - u1) + val[k - 1];
    return true;
}

// setup_spinup.f90:12-54 and main.f90:54-56 (elapsed_time = it dt, julian_day += dt / 86400)
__global__ void k_series_clock(double *scal, double dt, double tide_per, double bc_per, double wind_per) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double it = scal[5] + 1.0;
    const double elapsed = it * dt;
    scal[5] = it;
    scal[0] = elapsed;
    scal[4] = scal[4] + dt / 86400.0;
    scal[1] = (tide_per > 0.0 && elapsed < tide_per) ? tanh(2.0 * elapsed / tide_per) : 1.0;
    scal[2] = (bc_per > 0.0 && elapsed < bc_per) ? tanh(2.0 * elapsed / bc_per) : 1.0;
    scal[6] = (wind_per > 0.0 && elapsed < wind_per) ? tanh(2.0 * elapsed / wind_per) : 1.0;
}

// get_windp_at_face.f90:18-38 / IDW_windp_ser.f90:27-52: each station's wind at u2 =
// julian_day x 86400, v12 = (v13 - v11) / (u3 - u1) (u2 - u1) + v11 on the first interval that
// holds u2, 0 when none does
__global__ void k_series_wind_stations(Forcing f, SeriesDev S) {
    const int k = threadIdx.x;
    if (k >= S.n_wind) return;
    const double u2 = f.scal[4] * 86400.0;
    double vals[2] = {0.0, 0.0};
    for (int c = 0; c < 2; ++c) {
        const int kind = 4 + c;
        const int s0 = S.start[kind][k], n = S.start[kind][k + 1] - s0;
        const double *t = S.time[kind] + s0, *val = S.value[kind] + s0;
        for (int q = 1; q < n; ++q) {
            const double u1 = t[q - 1] - S.rdd_s, u3 = t[q] - S.rdd_s;
            if (u2 >= u1 && u2 <= u3) {
                vals[c] = (val[q] - val[q - 1]) / (u3 - u1) * (u2 - u1) + val[q - 1];
                break;
            }
        }
    }
    S.wind_at_station[2 * k] = vals[0];
    S.wind_at_station[2 * k + 1] = vals[1];
}

// IDW_windp_ser.f90:77-118 at one node (power 1): two stations weighted by the other's distance,
// three by the product of the other two
__device__ __forceinline__ void idw_node(const Geom &g, const SeriesDev &S, int node, double &u, double &v) {
    const double x = g.x_node[node - 1], y = g.y_node[node - 1];
    double dist[3];
    for (int k = 0; k < S.n_wind; ++k) {
        const int sn = S.wind_node[k];
        const double dx = x - g.x_node[sn - 1], dy = y - g.y_node[sn - 1];
        dist[k] = sqrt(dx * dx + dy * dy);
    }
    const double *w = S.wind_at_station;
    if (S.n_wind == 2) {
        const double r1 = dist[1], r2 = dist[0];
        u = (r1 * w[0] + r2 * w[2]) / (r1 + r2);
        v = (r1 * w[1] + r2 * w[3]) / (r1 + r2);
    } else {
        const double r1 = dist[1] * dist[2], r2 = dist[0] * dist[2], r3 = dist[0] * dist[1];
        u = (r1 * w[0] + r2 * w[2] + r3 * w[4]) / (r1 + r2 + r3);
        v = (r1 * w[1] + r2 * w[3] + r3 * w[5]) / (r1 + r2 + r3);
    }
}

// get_windp_at_face.f90:40-48 and calculate_wind_stress.f90:41-65 (heat_model_flag 0): one thread
// per face
__global__ void k_series_wind_faces(Geom g, Forcing f, SeriesDev S) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.NF) return;
    double u, v;
    if (S.n_wind == 1) {
        u = S.wind_at_station[0];
        v = S.wind_at_station[1];
    } else {
        double u1, v1, u2, v2;
        idw_node(g, S, g.nodenum_at_face[2 * j], u1, v1);
        idw_node(g, S, g.nodenum_at_face[2 * j + 1], u2, v2);
        u = (u1 + u2) * 0.5;
        v = (v1 + v2) * 0.5;
    }
    if (S.hur_flag == 1) {   // the hurricane drag law follows on these face winds
        S.face_u[j] = u;
        S.face_v[j] = v;
        return;
    }
    const double speed = sqrt(u * u + v * v);
    const double normal = u * g.cos_theta[j] + v * g.sin_theta[j];
    const double tangent = -u * g.sin_theta[j] + v * g.cos_theta[j];
    double cda;
    if (S.wind_formular == 1) cda = 0.001 * (0.75 + 0.067 * speed);
    else if (S.wind_formular == 2) cda = 0.001 * (0.61 + 0.063 * speed);
    else cda = 0.001 * (0.80 + 0.065 * speed);
    cda = fmin(fmax(cda, S.cda_min), S.cda_max);
    const double gamma_t = cda * S.rho_ratio * speed;
    const double spin = f.scal[6];
    const_cast<double *>(f.gamma_t)[j] = gamma_t;
    const_cast<double *>(f.wind_stress_normal)[j] = gamma_t * normal * spin;
    const_cast<double *>(f.wind_stress_tangnt)[j] = gamma_t * tangent * spin;
}

// main.f90:115-127: read_hurricane_ser_1 runs while julian_day (already advanced) lies in the window
__device__ __forceinline__ bool hurricane_window(const Forcing &f, const SeriesDev &S) {
    const double jd = f.scal[4];
    return jd >= S.hur_start && jd <= S.hur_end;
}

__device__ __forceinline__ bool hurricane_read_step(const Forcing &f, const SeriesDev &S) {
    return (long long)f.scal[5] % S.hur_interval == 0;
}

// read_hurricane_ser_2.f90:19-83: the storm centre of this step, by one thread before the nodes.
// A read step moves the first centre to the second and takes the pushed one; otherwise the time
// ratio and the centre shift of the step are kept for the nodes and the first centre and its
// time advance (the reference's order).
__global__ void k_hurricane_track(Forcing f, SeriesDev S, double dt, gom_status *st) {
    if (threadIdx.x != 0 || blockIdx.x != 0 || !hurricane_window(f, S)) return;
    double *t = S.hur_track;
    if (hurricane_read_step(f, S)) {
        t[0] = t[3];
        t[1] = t[4];
        if (*S.hur_track_ready == 0) {
            record_error(st, GOM_E_ARG, 38, 0, 0, f.scal[5], GOM_ENTITY_OTHER);
        } else {
            t[3] = t[6];
            t[4] = t[7];
            t[5] = t[8];
        }
        *S.hur_track_ready = 0;
        return;
    }
    const double tr = (f.scal[4] - t[2]) / (t[5] - t[2]);
    const double dx = t[3] - t[0], dy = t[4] - t[1];
    const double cx = t[0] + dx * tr, cy = t[1] + dy * tr;
    t[9] = tr;
    t[10] = dx;
    t[11] = dy;
    t[0] = cx;
    t[1] = cy;
    t[2] = t[2] + dt / 86400.0;
}

// IDW_5.f90:36-80 at (xn, yn) over node i's neighbour list (0-based i): the three nearest, the
// first of equal distances (the list is in node order, as minloc scans it), with the reference's
// taken-entry value 1.0e15 (default REAL) where the list is shorter than three
__device__ void idw5(const Geom &g, const SeriesDev &S, int i, double xn, double yn, const double *v, long nn,
                     double out[3]) {
    const double far = (double)1.0e15f;
    const long long s0 = S.search_start[i], cnt = S.search_start[i + 1] - s0;
    double md[3] = {far, far, far};
    int nsel[3] = {0, 0, 0};
    for (long long k = 0; k < cnt; ++k) {
        const int nd = S.search_nodes[s0 + k];
        const double dx = xn - g.x_node[nd - 1], dy = yn - g.y_node[nd - 1];
        const double d = sqrt(dx * dx + dy * dy);
        // distances are +0 or more (or NaN): the bit-pattern order is their order
        if (k < 3 || lt_of_nonneg(d, md[2])) {
            if (k == 0 || lt_of_nonneg(d, md[0])) {
                md[2] = md[1];
                nsel[2] = nsel[1];
                md[1] = md[0];
                nsel[1] = nsel[0];
                md[0] = d;
                nsel[0] = nd;
            } else if (k == 1 || lt_of_nonneg(d, md[1])) {
                md[2] = md[1];
                nsel[2] = nsel[1];
                md[1] = d;
                nsel[1] = nd;
            } else {
                md[2] = d;
                nsel[2] = nd;
            }
        }
    }
    for (int q = (int)(cnt < 3 ? cnt : 3); q < 3; ++q) {   // minloc over taken entries only
        md[q] = far;
        nsel[q] = S.search_nodes[s0];
    }
    const double r1 = md[1] * md[2], r2 = md[0] * md[2], r3 = md[0] * md[1];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const double *w = v + c * nn;
        out[c] = (r1 * w[nsel[0] - 1] + r2 * w[nsel[1] - 1] + r3 * w[nsel[2] - 1]) / (r1 + r2 + r3);
    }
}

// read_hurricane_ser_1.f90:20-75 at one node: on a read step frames 0 and 1 take frame 2 and
// frame 2 the pushed record; otherwise frame 1 steps by (frame 2 - frame 0) / real(interval)
// (the integer widened through default REAL), or with method 2 (read_hurricane_ser_2.f90:84-125)
// frames 1 and 2 are moved with the centre and blended into hur_w1n (k_hurricane_blend copies it
// into frame 1 once every node has read the old one).  air_p (air_p1) follows frame 1.
__global__ void k_hurricane_nodes(Geom g, Forcing f, SeriesDev S, gom_status *st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.NN || !hurricane_window(f, S)) return;
    const long nn = g.NN;
    double *w0 = S.hur_frames, *w1 = S.hur_frames + 3 * nn, *w2 = S.hur_frames + 6 * nn;
    if (S.hur_method == 2 && !hurricane_read_step(f, S)) {
        const double tr = S.hur_track[9], dx = S.hur_track[10], dy = S.hur_track[11];
        double o1[3], o2[3];
        idw5(g, S, i, g.x_node[i] - dx * tr, g.y_node[i] - dy * tr, w1, nn, o1);
        idw5(g, S, i, g.x_node[i] + dx * (1.0 - tr), g.y_node[i] + dy * (1.0 - tr), w2, nn, o2);
#pragma unroll
        for (int c = 0; c < 3; ++c) S.hur_w1n[c * nn + i] = (1.0 - tr) * o1[c] + tr * o2[c];
        return;
    }
    if (hurricane_read_step(f, S)) {
        const bool ready = *S.hur_ready != 0;
        if (!ready && i == 0) record_error(st, GOM_E_ARG, 34, 0, 0, f.scal[5], GOM_ENTITY_OTHER);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double v2 = w2[c * nn + i];
            w0[c * nn + i] = v2;
            w1[c * nn + i] = v2;
            if (ready) w2[c * nn + i] = S.hur_next[c * nn + i];
        }
    } else {
        const double den = (double)(float)S.hur_interval;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double inc = (w2[c * nn + i] - w0[c * nn + i]) / den;
            w1[c * nn + i] = w1[c * nn + i] + inc;
        }
    }
    const_cast<double *>(f.air_p)[i] = w1[2 * nn + i];
}

// find_neighbour_nodes.f90:19-45 for node i (0-based): its nearest neighbour's distance (with
// the default-REAL 1.0e15 standing in for itself), the search range (20 km when that neighbour is
// nearer than 5 km, else four times its distance) and the nodes within it, in node order; pass 0
// counts, pass 1 writes
template <int PASS>
__global__ void k_hur_neighbours(Geom g, int *count, const long long *start, int *nodes) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.NN) return;
    const double far = (double)1.0e15f;
    const double xi = g.x_node[i], yi = g.y_node[i];
    double min_dist = far;
    for (int ii = 0; ii < g.NN; ++ii) {
        if (ii == i) continue;
        const double dx = xi - g.x_node[ii], dy = yi - g.y_node[ii];
        const double d = sqrt(dx * dx + dy * dy);
        if (lt_of_nonneg(d, min_dist)) min_dist = d;
    }
    const double range = min_dist < 5000.0 ? (double)(20 * 1000.0f) : min_dist * 4;
    long long o = PASS == 1 ? start[i] : 0;
    int n = 0;
    for (int ii = 0; ii < g.NN; ++ii) {
        double d = far;
        if (ii != i) {
            const double dx = xi - g.x_node[ii], dy = yi - g.y_node[ii];
            d = sqrt(dx * dx + dy * dy);
        }
        if (d <= range) {
            if (PASS == 1) nodes[o++] = ii + 1;
            ++n;
        }
    }
    if (PASS == 0) count[i] = n;
}

// method 2, a step between reads: frame 1 takes the blend, air_p follows
__global__ void k_hurricane_blend(Geom g, Forcing f, SeriesDev S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.NN || !hurricane_window(f, S) || hurricane_read_step(f, S)) return;
    const long nn = g.NN;
    double *w1 = S.hur_frames + 3 * nn;
#pragma unroll
    for (int c = 0; c < 3; ++c) w1[c * nn + i] = S.hur_w1n[c * nn + i];
    const_cast<double *>(f.air_p)[i] = w1[2 * nn + i];
}

// read_hurricane_ser_1.f90:52-59 / :78-84 (face winds from frame 1 inside the window) and
// calculate_wind_stress.f90:105-137 on every face, every step
__global__ void k_hurricane_faces(Geom g, Forcing f, SeriesDev S) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.NF) return;
    const bool win = hurricane_window(f, S);
    if (j == 0 && win && hurricane_read_step(f, S)) *S.hur_ready = 0;   // the record is taken
    double u, v;
    if (win) {
        const double *w1 = S.hur_frames + 3 * (long)g.NN;
        const int n1 = g.nodenum_at_face[2 * j] - 1, n2 = g.nodenum_at_face[2 * j + 1] - 1;
        u = (w1[n1] + w1[n2]) * 0.5;
        v = (w1[g.NN + n1] + w1[g.NN + n2]) * 0.5;
        S.face_u[j] = u;
        S.face_v[j] = v;
    } else {
        u = S.face_u[j];
        v = S.face_v[j];
    }
    const double speed = sqrt(u * u + v * v);
    const double normal = u * g.cos_theta[j] + v * g.sin_theta[j];
    const double tangent = -u * g.sin_theta[j] + v * g.cos_theta[j];
    double cda;
    if (S.wind_formular == 1) cda = 0.001 * (0.75 + 0.067 * speed);
    else if (S.wind_formular == 3) cda = 0.001 * (0.80 + 0.065 * speed);
    else cda = 0.001 * (0.61 + 0.063 * speed);   // formula 2, and the reference's default
    cda = fmin(S.hur_cda_max, cda);
    const double gamma_t = cda * S.rho_ratio * speed;
    const double spin = f.scal[6];
    const_cast<double *>(f.gamma_t)[j] = gamma_t;
    const_cast<double *>(f.wind_stress_normal)[j] = gamma_t * normal * spin;
    const_cast<double *>(f.wind_stress_tangnt)[j] = gamma_t * tangent * spin;
}

// compute_boundary_eta.f90:45-124 (types 1 and 2) and the open-boundary concentrations of every
// subcycle (solve_transport_equation_v19.f90:229-282); one thread per open-boundary cell
__global__ void k_series_ob(Geom g, Forcing f, Params p, SeriesDev S, const double *eta_cell, gom_status *st,
                            int ntr_salt, int ntr_temp, int nt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.NOB) return;
    const double elapsed = f.scal[0], spin = f.scal[1], spin_bc = f.scal[2], jd_s = f.scal[4] * 86400.0;
    const double dt = p.dt;
    double *eta_old = const_cast<double *>(f.eta_at_ob_old), *eta_new = const_cast<double *>(f.eta_at_ob_new);
    const int type = S.ob_type[i];
    if (type == -1) {
        // compute_boundary_eta.f90:45-70: the mean elevation of the interior cells around the
        // open-boundary cell's nodes (each counted once per node it shares), old level only;
        // the elevations are those the step starts from (nothing before this phase changes them)
        const int cell = g.ob_cell_id[i];
        double sum0 = 0.0;
        int icount = 0;
        for (int l = 1; l <= g.tri_or_quad[cell - 1]; ++l) {
            const int nd = g.cell_node(l, cell);
            for (int i2 = 1; i2 <= g.adj_cells_at_node[nd - 1]; ++i2) {
                const int ie = g.node_cell(i2, nd);
                if (g.ob_element_flag[ie - 1] == 0) {
                    icount = icount + 1;
                    sum0 = sum0 + eta_cell[ie - 1];
                }
            }
        }
        if (icount == 0) record_error(st, GOM_E_ARG, 0, i + 1, 0, 0.0, GOM_ENTITY_OTHER);   // an isolated cell
        else eta_old[i] = sum0 / icount;
    } else if (type == 1) {
        const double deg2rad = 3.141592653589793 / 180.0;
        const int h = S.ob_h[i];
        double o = 0.0, nw = 0.0;
        if (h >= 1 && h <= S.n_harm) {
            for (int j = S.h_start[h - 1]; j < S.h_start[h]; ++j) {
                const double w = 2.0 * 3.141592653589793 / (S.per_h[j] * 3600.0);
                const double a = spin * S.amp[j] * S.nodal[j];
                o = o + a * cos(w * (elapsed - dt) + S.eq[j] * deg2rad - S.ph[j] * deg2rad - S.shift[h - 1] * deg2rad);
                nw = nw + a * cos(w * elapsed + S.eq[j] * deg2rad - S.ph[j] * deg2rad - S.shift[h - 1] * deg2rad);
            }
        }
        eta_old[i] = o;
        eta_new[i] = nw;
    } else if (type == 2) {
        double v;
        if (series_at(S, 0, S.ob_eta[i], jd_s - dt, v)) eta_old[i] = spin * v;
        if (series_at(S, 0, S.ob_eta[i], jd_s, v)) eta_new[i] = spin * v;
    }
    double *con = const_cast<double *>(f.con_at_ob);
    const double dt2 = dt / nt;
    for (int sub = 0; sub < nt; ++sub) {
        const double u2 = (jd_s - dt) + (sub + 1) * dt2;
        double v;
        if (ntr_salt) {
            double *c = con + ((long)sub * 2 + 0) * g.NOB + i;
            if (S.ob_salt[i] <= 0) *c = 0.0;
            else if (series_at(S, 2, S.ob_salt[i], u2, v)) *c = spin_bc * v;
        }
        if (ntr_temp) {
            double *c = con + ((long)sub * 2 + 1) * g.NOB + i;
            if (S.ob_temp[i] <= 0) *c = 0.0;
            else if (series_at(S, 3, S.ob_temp[i], u2, v)) *c = spin_bc * v;
        }
    }
}

// calculate_Q.f90:47-75, second-order Lagrange through three samples (raw series times)
__device__ double q_lagrange(const SeriesDev &S, int id, double u2) {
    const int s0 = S.start[1][id - 1], n = S.start[1][id] - s0;
    const double *t = S.time[1] + s0, *val = S.value[1] + s0;
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

// calculate_Q.f90:21-75 and the river concentrations (solve_transport_equation_v19.f90:326-382)
__global__ void k_series_qb(Geom g, Forcing f, Params p, SeriesDev S, int ntr_salt, int ntr_temp, int nt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.NQB) return;
    const double spin_bc = f.scal[2], jd_s = f.scal[4] * 86400.0, dt = p.dt;
    double *q = const_cast<double *>(f.q_add);
    const int qid = S.qb_q[i];
    if (qid >= 1 && qid <= S.n[1]) {
        double v;
        if (S.q_method == 2) q[i] = q_lagrange(S, qid, jd_s) * S.qb_portion[i];
        else if (series_at(S, 1, qid, jd_s, v)) q[i] = v * S.qb_portion[i];
    }
    double *con = const_cast<double *>(f.con_at_qb);
    const double dt2 = dt / nt;
    for (int sub = 0; sub < nt; ++sub) {
        const double u2 = (jd_s - dt) + (sub + 1) * dt2;
        double v;
        if (ntr_salt) {
            double *c = con + ((long)sub * 2 + 0) * g.NQB + i;
            if (S.qb_salt[i] <= 0) *c = 0.0;
            else if (series_at(S, 2, S.qb_salt[i], u2, v)) *c = spin_bc * v;
        }
        if (ntr_temp) {
            double *c = con + ((long)sub * 2 + 1) * g.NQB + i;
            if (S.qb_temp[i] <= 0) *c = 0.0;
            else if (series_at(S, 3, S.qb_temp[i], u2, v)) *c = spin_bc * v;
        }
    }
}

}  // namespace

cudaError_t launch_storm_forcing(const Geom &g, const Forcing &f, const Params &p, cudaStream_t stream,
                                 const double *storms, double *wu, double *wv) {
    double *scal = const_cast<double *>(f.scal);
    k_forcing_clock<<<1, 32, 0, stream>>>(scal, p.dt);
    k_storm_nodes<<<blocks_for(g.NN, 256), 256, 0, stream>>>(g, scal, storms, wu, wv, const_cast<double *>(f.air_p));
    k_storm_faces<<<blocks_for(g.NF, 256), 256, 0, stream>>>(
        g, scal, storms, wu, wv, kAirDensity / p.rho_o, const_cast<double *>(f.wind_stress_normal),
        const_cast<double *>(f.wind_stress_tangnt), const_cast<double *>(f.gamma_t));
    if (g.NOB > 0)
        k_storm_ob<<<blocks_for(g.NOB, 128), 128, 0, stream>>>(g, scal, storms, p.rho_o * p.gravity, p.dt,
                                                                const_cast<double *>(f.eta_at_ob_old),
                                                                const_cast<double *>(f.eta_at_ob_new));
    return cudaGetLastError();
}

// heat_term_by_term.f90:27-110 (sol_swr 2), one thread: the air series at u2 = julian_day x 86400
// on the first interval that holds it ((u2 - u1)(v3 - v1)/(u3 - u1) + v1; none: zeros), then the
// short-wave term, the atmospheric long-wave term, the wind function and the air vapour pressure.
// Default-REAL constants are widened from single precision, as the reference's mixed expressions
// widen them; integer powers are products (x^4 = (x^2)^2, x^6 = (x^2 x)^2).
// julian_to_localtime.f90:16-86 with its state: the hour of julian day jday.  The month table is
// saved between calls and set with the month; in a leap year (other than 1900) only while the
// month variable is 3 or more (so a run starting in January or February keeps a zero table)
__device__ int local_hour(int year, int *state, double jday) {
    const double leap[12] = {0, 32, 60, 91, 121, 152, 182, 213, 244, 274, 305, 335};
    const double normal[12] = {0, 31, 59, 90, 120, 151, 181, 212, 243, 273, 304, 334};
    const double leap_top[11] = {31, 60, 91, 121, 152, 182, 213, 244, 274, 305, 335};
    const double normal_top[11] = {31, 59, 90, 120, 151, 181, 212, 243, 273, 304, 334};
    int month = state[0];
    double m;
    if (year % 4 == 0) {
        if (year != 1900 && month >= 3) {
            int k = 0;
            while (k < 11 && jday > leap_top[k]) ++k;
            month = k + 1;
            state[1] = 1;
        }
        m = state[1] ? leap[month - 1] : 0.0;
    } else {
        int k = 0;
        while (k < 11 && jday > normal_top[k]) ++k;
        month = k + 1;
        m = normal[month - 1];
    }
    state[0] = month;
    const double day_temp = jday - m;
    const int day = (int)day_temp + 1;
    return (int)((day_temp + 1 - day) * 24.0);
}

__global__ void k_heat_scalars(Forcing f, SeriesDev S) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double u2 = f.scal[4] * 86400.0;
    double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};   // Ta, Tdew, w_speed, sol_rad, cloudness
    for (int t = 1; t < S.n_air; ++t) {
        const double u1 = S.air_time[t - 1] - S.rdd_s, u3 = S.air_time[t] - S.rdd_s;
        if (u2 >= u1 && u2 <= u3) {
            for (int c = 0; c < 5; ++c) {
                const double v1 = S.air_values[(long)c * S.n_air + t - 1], v3 = S.air_values[(long)c * S.n_air + t];
                v[c] = (u2 - u1) * (v3 - v1) / (u3 - u1) + v1;
            }
            break;
        }
    }
    const double Ta = v[0], Tdew = v[1], w_speed = v[2], sol_rad = v[3], cloud = v[4];
    const double c2 = cloud * cloud;
    double phi_sn = 0.0;   // sol_swr 1 with the sun below the horizon: the reference leaves it unset
    if (S.sol_swr == 1) {
        // :64-83: the sun's elevation A0 at the local hour, and the clear-sky short-wave from it
        const int hr = local_hour(S.year, S.heat_month, f.scal[4]);
        const double pi = 3.141592653589793, deg2rad = pi / 180.0, rad2deg = 180.0 / pi;
        const double j_day = f.scal[4] + 1;
        const double tau_d = 2.0 * pi * (double)((int)(j_day + 1) - 1) / 365.0;
        const double sdec = (double)0.006918f - (double)0.399912f * cos(tau_d) + (double)0.070257f * sin(tau_d) -
                            (double)0.006758f * cos(2.0 * tau_d) + (double)0.000907f * sin(2.0 * tau_d) -
                            (double)0.002697f * cos(3.0 * tau_d) + (double)0.001480f * sin(3.0 * tau_d);
        const double eqt = (double)0.170f * sin(4.0 * pi * (double)((int)j_day - 80) / 373.0) -
                           (double)0.129f * sin(2.0 * pi * (double)((int)j_day - 8) / 355.0);
        const double sm = 15.0 * (double)(int)(S.lon / 15.0);
        const double lha = (double)0.261799f * ((double)hr - (S.lon - sm) * (double)0.0666667f + eqt - 12.0);
        const double a0 =
            asin(sin(S.lat * deg2rad) * sin(sdec) + cos(S.lat * deg2rad) * cos(sdec) * cos(lha)) * rad2deg;
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
        phi_ac = (double)5.67e-8f * (x2 * x2) * (1.0 - (double)0.261f * exp(-((double)7.77e-4f * (Ta * Ta))));
    }
    const double phi_an = phi_ac * (1.0 + (double)0.17f * c2) * 0.97;
    const double z0 = w_speed <= (double)2.3f ? (double)0.001f : (double)0.005f;
    const double alpha = log(S.wind_height / z0) / log(2.0 / z0);
    const double bz = S.fwz_b / pow(alpha, S.fwz_c);
    const double fwz = S.fwz_a + bz * pow(w_speed, S.fwz_c);
    const double ea = exp(2.3026 * (7.5 * Tdew / (Tdew + 237.3) + (double)0.6609f));
    S.heat_scal[0] = Ta;
    S.heat_scal[1] = phi_sn;
    S.heat_scal[2] = phi_an;
    S.heat_scal[3] = fwz;
    S.heat_scal[4] = ea;
}

// heat_term_by_term.f90:112-156 for one cell column: a dry column's phi_sz is 0 (phi_sw kept); a
// wet one gets the net surface flux less the short-wave that passes the top layer, the short-wave
// absorbed in each lower layer, and in every wet layer the sediment share and the bottom exchange
// (layers above the top keep their values)
template <typename R> __global__ void k_heat_cells(Geom g, Forcing f, StateT<R> s, SeriesDev S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.NC) return;
    const int L = g.L;
    double *phi_sz = const_cast<double *>(f.phi_sz);
    const int tl = s.top_cell[i], b = g.bottom_cell[i];
    if (tl == 0) {
        for (int k = 1; k <= L; ++k) phi_sz[(long)i * L + k - 1] = 0.0;
        return;
    }
    const double Ta = S.heat_scal[0], phi_sn = S.heat_scal[1], phi_an = S.heat_scal[2], fwz = S.heat_scal[3],
                 ea = S.heat_scal[4];
    const double Tw = (double)s.temp_cell[ix(tl, i + 1, L)];
    const double xw = Tw + (double)273.15f, x2 = xw * xw;
    const double phi_br = (double)(0.97f * 5.67e-8f) * (x2 * x2);
    const double es = Tw < 0.0 ? exp(2.3026 * (9.5 * Tw / (Tw + 265.5) + (double)0.6609f))
                               : exp(2.3026 * (7.5 * Tw / (Tw + 237.3) + (double)0.6609f));
    const double phi_e = fwz * (es - ea);
    const double phi_c = 0.47 * fwz * (Tw - Ta);
    const double phi_n = phi_sn + phi_an - phi_br - phi_e - phi_c;
    const double Tb = (double)s.temp_cell[ix(b, i + 1, L)];
    const double phi_sw = S.sed_water_exchange * (S.t_sed - Tb);
    const_cast<double *>(f.phi_sw)[i] = phi_sw;
    double sol_out = (1.0 - S.sol_absorb) * phi_sn * exp(-(S.light_extinction * (double)s.dz_cell[ix(tl, i + 1, L)]));
    phi_sz[(long)i * L + tl - 1] = phi_n - sol_out;
    for (int k = tl - 1; k >= b; --k) {
        const double sol_in = sol_out;
        sol_out = sol_in * exp(-(S.light_extinction * (double)s.dz_cell[ix(k, i + 1, L)]));
        phi_sz[(long)i * L + k - 1] = sol_in - sol_out;
    }
    for (int k = b; k <= tl; ++k) {
        double v = phi_sz[(long)i * L + k - 1];
        v = v + sol_out * S.sed_temp_coeff;
        v = v + phi_sw;
        phi_sz[(long)i * L + k - 1] = v;
    }
}

cudaError_t hurricane_neighbour_counts(const Geom &g, int *count, cudaStream_t stream) {
    k_hur_neighbours<0><<<blocks_for(g.NN, 128), 128, 0, stream>>>(g, count, nullptr, nullptr);
    return cudaGetLastError();
}

cudaError_t hurricane_neighbour_fill(const Geom &g, const long long *start, int *nodes, cudaStream_t stream) {
    k_hur_neighbours<1><<<blocks_for(g.NN, 128), 128, 0, stream>>>(g, nullptr, start, nodes);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_heat_terms(const Geom &g, const Forcing &f, const StateT<R> &s, const SeriesDev &S,
                              cudaStream_t stream) {
    k_heat_scalars<<<1, 32, 0, stream>>>(f, S);
    k_heat_cells<R><<<blocks_for(g.NC, 128), 128, 0, stream>>>(g, f, s, S);
    return cudaGetLastError();
}
template cudaError_t launch_heat_terms<double>(const Geom &, const Forcing &, const StateT<double> &,
                                               const SeriesDev &, cudaStream_t);
template cudaError_t launch_heat_terms<float>(const Geom &, const Forcing &, const StateT<float> &,
                                              const SeriesDev &, cudaStream_t);

cudaError_t launch_series_forcing(const Geom &g, const Forcing &f, const Params &p, const SeriesDev &s,
                                  const double *eta_cell, gom_status *status, cudaStream_t stream) {
    k_series_clock<<<1, 32, 0, stream>>>(const_cast<double *>(f.scal), p.dt, s.tide_per_s, s.bc_per_s, s.wind_per_s);
    if (s.wind_flag == 1) {
        k_series_wind_stations<<<1, 32, 0, stream>>>(f, s);
        k_series_wind_faces<<<blocks_for(g.NF, 256), 256, 0, stream>>>(g, f, s);
    }
    if (s.hur_flag == 1) {
        if (s.hur_method == 2) k_hurricane_track<<<1, 32, 0, stream>>>(f, s, p.dt, status);
        k_hurricane_nodes<<<blocks_for(g.NN, 256), 256, 0, stream>>>(g, f, s, status);
        if (s.hur_method == 2) k_hurricane_blend<<<blocks_for(g.NN, 256), 256, 0, stream>>>(g, f, s);
        k_hurricane_faces<<<blocks_for(g.NF, 256), 256, 0, stream>>>(g, f, s);
    }
    const int nt = p.trans_sub_iter > 0 ? p.trans_sub_iter : 1;
    const int salt = p.transport_flag && p.is_salt, temp = p.transport_flag && p.is_temp;
    if (g.NOB > 0) k_series_ob<<<blocks_for(g.NOB, 128), 128, 0, stream>>>(g, f, p, s, eta_cell, status, salt, temp, nt);
    if (g.NQB > 0) k_series_qb<<<blocks_for(g.NQB, 128), 128, 0, stream>>>(g, f, p, s, salt, temp, nt);
    return cudaGetLastError();
}

}  // namespace gom
