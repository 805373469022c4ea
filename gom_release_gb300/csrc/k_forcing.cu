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
    double cda = fmin(0.001 * (0.75 + 0.067 * speed), 0.003);
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

}  // namespace gom
