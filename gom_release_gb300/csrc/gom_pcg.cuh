// gom_pcg.cuh -- the Jacobi-preconditioned conjugate gradient of pre_conj_grad.f90:9-230 as one
// cooperative kernel, shared by the translation units that launch it.  Definitions have internal
// linkage (anonymous namespace), so each including file gets its own copy.
#pragma once

#include "gom_device.cuh"

namespace gom {
namespace {

// -------------------------------------------------------------------- grid-wide barrier
__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Sense-counting barrier over all blocks of a cooperative launch.  Every wait is bounded: after
// about 1 s the block records GOM_E_TIMEOUT and the caller leaves the kernel.
__device__ bool grid_barrier(unsigned *bar, unsigned nblocks, gom_status *st) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = bar + 1;
        unsigned gen = *vgen;
        __threadfence();
        unsigned arrived = atomicAdd(bar, 1u);
        int good = 1;
        if (arrived == nblocks - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            unsigned long long t0 = globaltimer_ns();
            while (*vgen == gen) {
                __nanosleep(64);
                if (globaltimer_ns() - t0 > 1000000000ull) {
                    record_error(st, GOM_E_TIMEOUT, 1, (int)blockIdx.x, 0, 0.0, GOM_ENTITY_OTHER);
                    good = 0;
                    break;
                }
            }
        }
        __threadfence();
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// block reduction of one double; result valid in every thread
template <int THREADS>
__device__ __forceinline__ double block_sum(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    if (w == 0) {
        t = lane < THREADS / 32 ? sh[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) sh[32] = t;
    }
    __syncthreads();
    double r = sh[32];
    __syncthreads();
    return r;
}

// sum of all block partials in a fixed order (identical in every block)
__device__ __forceinline__ double sum_partials(const double *part, int n, double *sh) {
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (w == 0) {
        double t = 0.0;
        for (int i = lane; i < n; i += 32) t += ((volatile const double *)part)[i];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) sh[33] = t;
    }
    __syncthreads();
    double r = sh[33];
    __syncthreads();
    return r;
}

// block reduction of two doubles at once (one pair of __syncthreads); results valid in every thread
template <int THREADS>
__device__ __forceinline__ void block_sum2(double &a, double &b, double *sh) {
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sh[w] = a;
        sh[32 + w] = b;
    }
    __syncthreads();
    if (w == 0) {
        double ta = lane < THREADS / 32 ? sh[lane] : 0.0;
        double tb = lane < THREADS / 32 ? sh[32 + lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            ta += __shfl_down_sync(0xffffffffu, ta, o);
            tb += __shfl_down_sync(0xffffffffu, tb, o);
        }
        if (lane == 0) {
            sh[64] = ta;
            sh[65] = tb;
        }
    }
    __syncthreads();
    a = sh[64];
    b = sh[65];
    __syncthreads();
}

// -------------------------------------------------------------------- single-run FP64 solver
// Grid barrier on a counter that only grows within a launch (cleared before it): barrier number k
// waits until the counter reaches k x (blocks + phantom).  Arrival is a release reduction (the
// block's earlier writes become visible before the count), the wait an acquire load; each wait
// gives up after about 1 s with GOM_E_TIMEOUT.
struct GridSync {
    unsigned *bar;
    unsigned nblocks;   // blocks of the grid + phantom blocks (tests)
    unsigned k;
    gom_status *st;
    __device__ bool sync() {
        __shared__ int ok;
        __syncthreads();
        ++k;
        if (threadIdx.x == 0) {
            asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(bar), "r"(1u) : "memory");
            const unsigned target = k * nblocks;
            int good = 1;
            const unsigned long long t0 = globaltimer_ns();
            unsigned spins = 0, v;
            for (;;) {
                asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(bar) : "memory");
                if (v >= target) break;
                if ((++spins & 255u) == 0 && globaltimer_ns() - t0 > 1000000000ull) {
                    record_error(st, GOM_E_TIMEOUT, 1, (int)blockIdx.x, 0, 0.0, GOM_ENTITY_OTHER);
                    good = 0;
                    break;
                }
            }
            __threadfence();
            ok = good;
        }
        __syncthreads();
        return ok != 0;
    }
};

// pre_conj_grad.f90:9-230 -- the Jacobi-preconditioned CG of the reference, restated for GB300:
//  * the Jacobi preconditioner is folded into the matrix: CG on A' = D^-1/2 A D^-1/2 with
//    x' = D^1/2 x and r' = D^-1/2 r produces the iterates of Jacobi-PCG on A (M = D), with the
//    reference's stop quantity r^T M^-1 r = r'^T r' -- and no M^-1 products per iteration
//    (GB300 issues about 1 TFLOP/s of FP64, so FP64 operations per row set the cost);
//  * the single-reduction form of Chronopoulos and Gear (J. Comput. Appl. Math. 25, 1989): both
//    inner products of an iteration, gamma = r'^T r' and delta = w^T r' (w = A' r'), are reduced
//    together, so an iteration needs ONE grid barrier.  Recurrences (s = A' p):
//        p = r' + beta p,  s = w + beta s,  x' = x' + alpha p,  r' = r' - alpha s,  w = A' r',
//        beta = gamma_new / gamma,  alpha = gamma_new / (delta_new - beta gamma_new / alpha).
//    The product w = A' r' of a row needs the neighbours' new r', which the neighbours form in the
//    same pass; each row recomputes them from the neighbours' previous r', s and w (the very
//    operations the neighbour performs, so the values are identical), and r', s, w alternate
//    between two buffers so that the previous values stay readable until the next barrier;
//  * the stop test is the reference's, sqrt(gamma^2 / gamma_0^2) < tol after every iteration; one
//    thread of each block forms the scalars from the block partials summed in a fixed order (so
//    every block takes the same decisions); a zero initial residual leaves x untouched (the
//    reference would divide 0 by 0).
// The sums run in parallel, so the solution differs from a serial run in the last bits.
struct PcgArgs {
    Geom g;                     // NC, tri_or_quad, adj_cellnum_at_cell
    const double *sp, *b;       // (0:4, NC) rows, diagonal first; right-hand side
    double *x;                  // initial guess in, solution out
    double *dr;                 // D^-1/2 (work)
    double *xs, *p;             // x' and p (work of the form without register rows)
    double *r[2], *s[2], *w[2]; // r', A' p, A' r' (two buffers each)
    double *pg, *pd;            // block partials of gamma and delta, two halves of gridDim.x each
    unsigned *bar;
    int *iters;
    int maxit;
    double tol;
    gom_status *st;
    unsigned phantom;           // blocks the barriers wait for in addition to the grid (tests only)
    int check_diag;             // 1: a non-positive diagonal is GOM_E_NOT_SPD (systems the caller built)
};

constexpr int PCG_CG_THREADS = 256;
constexpr int PCG_CG_ROWS = 4;   // rows per thread of the register form

// warp 0 sums the block partials (fixed order, reads from L2); with first, gamma_0 and alpha_0,
// else one thread forms the iteration's scalars and the stop decision
__device__ __forceinline__ void cg_scalars(const double *pg, const double *pd, int n, bool first, double &gamma,
                                           double &alpha, double &beta, double gamma_0, double tol, int &stop,
                                           double *sh) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (w == 0) {
        double ta = 0.0, tb = 0.0;
        for (int i = lane; i < n; i += 32) {
            ta += __ldcg(pg + i);
            tb += __ldcg(pd + i);
        }
        for (int o = 16; o > 0; o >>= 1) {
            ta += __shfl_down_sync(0xffffffffu, ta, o);
            tb += __shfl_down_sync(0xffffffffu, tb, o);
        }
        if (lane == 0) {
            const double gn = ta, dn = tb;
            sh[66] = gn;
            if (first) {
                sh[67] = 0.0;
                sh[68] = gn / dn;
                sh[69] = 0.0;
            } else {
                sh[69] = sqrt(gn * gn / (gamma_0 * gamma_0)) < tol ? 1.0 : 0.0;
                const double bt = gn / gamma;
                sh[67] = bt;
                sh[68] = gn / (dn - bt * gn / alpha);
            }
        }
    }
    __syncthreads();
    gamma = sh[66];
    beta = sh[67];
    alpha = sh[68];
    stop = sh[69] != 0.0;
    __syncthreads();
}

// ROWS > 0: each thread keeps its ROWS rows (scaled coefficients, neighbour ids, x', p, r', s, w)
// in registers for the whole solve (grid x PCG_CG_THREADS x ROWS >= NC); ROWS == 0: rows
// grid-strided, vectors in memory (any NC).  Both forms evaluate the same expressions in the same
// order, so they give the same solution bit for bit.
template <int ROWS> __global__ void __launch_bounds__(PCG_CG_THREADS, 1) k_pcg_cg1(PcgArgs a) {
    constexpr int T = PCG_CG_THREADS;
    constexpr int RR = ROWS > 0 ? ROWS : 1;
    __shared__ double sh[72];
    const Geom &g = a.g;
    const int n = g.NC;
    const int P = gridDim.x;
    const int stride = gridDim.x * T;
    const int t0 = blockIdx.x * T + threadIdx.x;
    GridSync B{a.bar, gridDim.x + a.phantom, 0u, a.st};
    // D^-1/2
    for (int i = t0; i < n; i += stride) {
        const double d = a.sp[(long)i * 5];
        if (a.check_diag && !(d > 0.0)) record_error(a.st, GOM_E_NOT_SPD, 100, i + 1, 0, d, GOM_ENTITY_CELL);
        a.dr[i] = 1.0 / sqrt(d);
    }
    if (!B.sync() || failed(a.st)) return;
    // scaled rows a'_il = dr_i a_il dr_m; r' = dr (b - A x); x' = x / dr
    double spr[RR][4], xr[RR], pr[RR], rr[RR], sr[RR], wr[RR];
    int nbr[RR][4];
    if constexpr (ROWS > 0) {
#pragma unroll
        for (int q = 0; q < ROWS; ++q) {
            const int i = t0 + q * stride;
            const int ii = i < n ? i : 0;
            const double *row = a.sp + (long)ii * 5;
            const double di = a.dr[ii];
            const int tq = g.tri_or_quad[ii];
            double sum = row[0] * a.x[ii];
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                nbr[q][l] = l < tq ? g.adj_cellnum_at_cell[(long)ii * 4 + l] : 0;
                spr[q][l] = 0.0;
                if (nbr[q][l] != 0) {
                    const int m = nbr[q][l] - 1;
                    sum = fma(row[l + 1], a.x[m], sum);
                    spr[q][l] = di * row[l + 1] * __ldcg(a.dr + m);
                }
            }
            rr[q] = (a.b[ii] - sum) * di;
            xr[q] = a.x[ii] / di;
            pr[q] = 0.0;
            sr[q] = 0.0;
            if (i < n) {
                a.r[0][i] = rr[q];
                a.s[0][i] = 0.0;
            }
        }
    } else {
        for (int i = t0; i < n; i += stride) {
            const double *row = a.sp + (long)i * 5;
            const double di = a.dr[i];
            const int tq = g.tri_or_quad[i];
            double sum = row[0] * a.x[i];
            for (int l = 0; l < tq; ++l) {
                const int nb = g.adj_cellnum_at_cell[(long)i * 4 + l];
                if (nb != 0) sum = fma(row[l + 1], a.x[nb - 1], sum);
            }
            a.r[0][i] = (a.b[i] - sum) * di;
            a.xs[i] = a.x[i] / di;
            a.p[i] = 0.0;
            a.s[0][i] = 0.0;
        }
    }
    if (!B.sync()) return;
    // w = A' r', gamma_0, delta_0
    double gl = 0.0, dl = 0.0;
    if constexpr (ROWS > 0) {
#pragma unroll
        for (int q = 0; q < ROWS; ++q) {
            const int i = t0 + q * stride;
            double wsum = rr[q];
#pragma unroll
            for (int l = 0; l < 4; ++l)
                if (nbr[q][l] != 0) wsum = fma(spr[q][l], __ldcg(a.r[0] + nbr[q][l] - 1), wsum);
            wr[q] = wsum;
            if (i < n) {
                a.w[0][i] = wsum;
                gl = fma(rr[q], rr[q], gl);
                dl = fma(wsum, rr[q], dl);
            }
        }
    } else {
        for (int i = t0; i < n; i += stride) {
            const double *row = a.sp + (long)i * 5;
            const double di = a.dr[i];
            const double ri = a.r[0][i];
            const int tq = g.tri_or_quad[i];
            double wsum = ri;
            for (int l = 0; l < tq; ++l) {
                const int nb = g.adj_cellnum_at_cell[(long)i * 4 + l];
                if (nb != 0) wsum = fma(di * row[l + 1] * __ldcg(a.dr + nb - 1), __ldcg(a.r[0] + nb - 1), wsum);
            }
            a.w[0][i] = wsum;
            gl = fma(ri, ri, gl);
            dl = fma(wsum, ri, dl);
        }
    }
    block_sum2<T>(gl, dl, sh);
    if (threadIdx.x == 0) {
        a.pg[blockIdx.x] = gl;
        a.pd[blockIdx.x] = dl;
    }
    if (!B.sync()) return;
    double gamma = 0.0, alpha = 0.0, beta = 0.0;
    int stop = 0;
    cg_scalars(a.pg, a.pd, P, true, gamma, alpha, beta, 0.0, 0.0, stop, sh);
    const double gamma_0 = gamma;
    int iters = 0;
    if (gamma_0 != 0.0) {
        int cur = 0, par = 1;
        for (int it = 1; it <= a.maxit; ++it) {
            if (failed(a.st)) return;
            const double *rc = a.r[cur], *sc = a.s[cur], *wc = a.w[cur];
            double *rn = a.r[cur ^ 1], *sn = a.s[cur ^ 1], *wn = a.w[cur ^ 1];
            gl = 0.0;
            dl = 0.0;
            if constexpr (ROWS > 0) {
                double nr[ROWS][4], ns[ROWS][4], nw[ROWS][4];
#pragma unroll
                for (int q = 0; q < ROWS; ++q)
#pragma unroll
                    for (int l = 0; l < 4; ++l) {
                        const int m = nbr[q][l] != 0 ? nbr[q][l] - 1 : 0;
                        nr[q][l] = __ldcg(rc + m);
                        ns[q][l] = __ldcg(sc + m);
                        nw[q][l] = __ldcg(wc + m);
                    }
#pragma unroll
                for (int q = 0; q < ROWS; ++q) {
                    const int i = t0 + q * stride;
                    const double pi = fma(beta, pr[q], rr[q]);
                    const double si = fma(beta, sr[q], wr[q]);
                    pr[q] = pi;
                    xr[q] = fma(alpha, pi, xr[q]);
                    const double rni = fma(-alpha, si, rr[q]);
                    double wsum = rni;
#pragma unroll
                    for (int l = 0; l < 4; ++l)
                        if (nbr[q][l] != 0)
                            wsum = fma(spr[q][l], fma(-alpha, fma(beta, ns[q][l], nw[q][l]), nr[q][l]), wsum);
                    rr[q] = rni;
                    sr[q] = si;
                    wr[q] = wsum;
                    if (i < n) {
                        rn[i] = rni;
                        sn[i] = si;
                        wn[i] = wsum;
                        gl = fma(rni, rni, gl);
                        dl = fma(wsum, rni, dl);
                    }
                }
            } else {
                for (int i = t0; i < n; i += stride) {
                    const double *row = a.sp + (long)i * 5;
                    const double di = a.dr[i];
                    const double pi = fma(beta, a.p[i], rc[i]);
                    const double si = fma(beta, sc[i], wc[i]);
                    a.p[i] = pi;
                    a.xs[i] = fma(alpha, pi, a.xs[i]);
                    const double rni = fma(-alpha, si, rc[i]);
                    double wsum = rni;
                    const int tq = g.tri_or_quad[i];
                    for (int l = 0; l < tq; ++l) {
                        const int nb = g.adj_cellnum_at_cell[(long)i * 4 + l];
                        if (nb != 0) {
                            const int m = nb - 1;
                            const double al = di * row[l + 1] * __ldcg(a.dr + m);
                            wsum = fma(al, fma(-alpha, fma(beta, __ldcg(sc + m), __ldcg(wc + m)), __ldcg(rc + m)), wsum);
                        }
                    }
                    rn[i] = rni;
                    sn[i] = si;
                    wn[i] = wsum;
                    gl = fma(rni, rni, gl);
                    dl = fma(wsum, rni, dl);
                }
            }
            block_sum2<T>(gl, dl, sh);
            if (threadIdx.x == 0) {
                a.pg[par * P + blockIdx.x] = gl;
                a.pd[par * P + blockIdx.x] = dl;
            }
            if (!B.sync()) return;
            cg_scalars(a.pg + par * P, a.pd + par * P, P, false, gamma, alpha, beta, gamma_0, a.tol, stop, sh);
            par ^= 1;
            cur ^= 1;
            iters = it;
            if (stop) break;
        }
    }
    // x = D^-1/2 x' (a solve without iterations leaves x as it came)
    if (iters > 0) {
        if constexpr (ROWS > 0) {
#pragma unroll
            for (int q = 0; q < ROWS; ++q) {
                const int i = t0 + q * stride;
                if (i < n) a.x[i] = xr[q] * a.dr[i];
            }
        } else {
            for (int i = t0; i < n; i += stride) a.x[i] = a.xs[i] * a.dr[i];
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.iters = iters;
}

// Launch of the single-run solver (cooperative, on cfg's stream): the register form when the rows
// fit num_sms x PCG_CG_THREADS x PCG_CG_ROWS, else the strided form on one block per SM.
inline cudaError_t launch_pcg_cg1(cudaLaunchConfig_t cfg, const PcgArgs &a, int num_sms) {
    const long n = a.g.NC;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.blockDim = dim3(PCG_CG_THREADS);
    cfg.dynamicSmemBytes = 0;
    const long per_block = (long)PCG_CG_THREADS * PCG_CG_ROWS;
    if (n <= per_block * num_sms) {
        long b = (n + per_block - 1) / per_block;
        cfg.gridDim = dim3((unsigned)(b < 1 ? 1 : b));
        return cudaLaunchKernelEx(&cfg, k_pcg_cg1<PCG_CG_ROWS>, a);
    }
    cfg.gridDim = dim3((unsigned)num_sms);
    return cudaLaunchKernelEx(&cfg, k_pcg_cg1<0>, a);
}

// threads per block of the mixed-precision and packed-run solvers below
constexpr int PCG_THREADS = 256;

// -------------------------------------------------------------------- mixed precision
// FP32 inner PCG iterations inside FP64 iterative refinement.  Each refinement step forms the
// true residual r = b - A x of the FP64 system in FP64 and its Jacobi norm delta = r^T M^-1 r;
// the stop test is the reference's, sqrt(delta^2 / delta_0^2) < tol, on that FP64 residual
// (delta_0 of the initial guess).  The correction equation A e = r is then solved by PCG in FP32
// (FP32 copy of the system, FP32 vectors) from e = 0 until its own ratio falls below what the
// outer test still needs, bounded below by what FP32 vectors can reach; every inner step adds its
// FP32 increment alpha*d to the FP64 solution x.  iters counts inner iterations; maxit bounds them.
struct PcgMixedArgs {
    Geom g;
    const double *sp, *b;
    double *x;
    float *sp32;                          // (5, NC) FP32 copy of the system
    float *minv, *r, *s, *q, *dA, *dB;
    double *pdq, *pdelta;
    unsigned *bar;
    int *iters;
    int maxit;
    double tol;
    gom_status *st;
    unsigned phantom;
};

// block reduction of one float (accumulated in FP32 within the block)
template <int THREADS>
__device__ __forceinline__ float block_sumf(float v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *shf = reinterpret_cast<float *>(sh);
    if (lane == 0) shf[w] = v;
    __syncthreads();
    if (w == 0) {
        float t = lane < THREADS / 32 ? shf[lane] : 0.0f;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) shf[68] = t;
    }
    __syncthreads();
    float r = shf[68];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(PCG_THREADS) k_pcg_mixed(PcgMixedArgs a) {
    __shared__ double sh[40];
    const Geom &g = a.g;
    const int n = g.NC;
    const unsigned nblocks = gridDim.x + a.phantom;
    const long stride = (long)gridDim.x * blockDim.x;
    const long t0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const float FP32_FLOOR = 1e-10f;   // inner ratio below which FP32 recurrences stop paying
    for (long i = t0; i < n; i += stride) {
        const double *row = a.sp + i * 5;
        float *row32 = a.sp32 + i * 5;
        for (int l = 0; l < 5; ++l) row32[l] = (float)row[l];
        a.minv[i] = (float)(1.0 / row[0]);
    }
    double delta_0 = 0.0;
    int iters = 0;
    // The partial sums alternate between two halves of pdq / pdelta with every grid barrier: a
    // block that has read the sums behind one barrier may write the next ones while a slower
    // block still reads, and the half it writes is the other one (the barrier after that write
    // orders the next reuse).
    int par = 0;
    const unsigned P = gridDim.x;
    for (int outer = 0;; ++outer) {
        // true residual r = b - A x and its Jacobi norm in FP64; the FP32 residual, d = M^-1 r and
        // the inner r^T d in the same pass (the previous inner step's barrier ordered the x update)
        double loc = 0.0;
        float floc = 0.0f;
        for (long i = t0; i < n; i += stride) {
            const double *row = a.sp + i * 5;
            int cell = (int)i + 1;
            double sum = row[0] * a.x[i];
            int tq = g.tri_or_quad[i];
            for (int l = 1; l <= tq; ++l) {
                int nb = g.cell_adj(l, cell);
                if (nb != 0) sum = fma(row[l], a.x[nb - 1], sum);
            }
            double ri = a.b[i] - sum;
            loc = fma(ri, ri / row[0], loc);
            float rf = (float)ri;
            float df = a.minv[i] * rf;
            a.r[i] = rf;
            a.dA[i] = df;
            floc = fmaf(rf, df, floc);
        }
        double bs = block_sum<PCG_THREADS>(loc, sh);
        float fbs = block_sumf<PCG_THREADS>(floc, sh);
        if (threadIdx.x == 0) {
            a.pdelta[par * P + blockIdx.x] = bs;
            a.pdq[par * P + blockIdx.x] = (double)fbs;
        }
        if (!grid_barrier(a.bar, nblocks, a.st)) return;
        double delta_true = sum_partials(a.pdelta + par * P, gridDim.x, sh);
        float delta_new = (float)sum_partials(a.pdq + par * P, gridDim.x, sh);
        par ^= 1;
        if (outer == 0) {
            delta_0 = delta_true;
            if (delta_0 == 0.0) break;
        } else if (sqrt(delta_true * delta_true / (delta_0 * delta_0)) < a.tol) {
            break;
        }
        if (iters >= a.maxit || !(delta_new > 0.0f)) break;
        const float inner_tol = fmaxf((float)(0.25 * a.tol * delta_0 / delta_true), FP32_FLOOR);
        const float din0 = delta_new;
        float beta = 0.0f;
        float *dcur = a.dA, *dnext = a.dB;
        bool first = true;
        while (iters < a.maxit) {
            if (failed(a.st)) return;
            floc = 0.0f;
            for (long i = t0; i < n; i += stride) {
                const float *row = a.sp32 + i * 5;
                int cell = (int)i + 1;
                float di = first ? dcur[i] : fmaf(beta, dcur[i], a.s[i]);
                float sum = row[0] * di;
                int tq = g.tri_or_quad[i];
                for (int l = 1; l <= tq; ++l) {
                    int nb = g.cell_adj(l, cell);
                    if (nb != 0) {
                        float dn = first ? dcur[nb - 1] : fmaf(beta, dcur[nb - 1], a.s[nb - 1]);
                        sum = fmaf(row[l], dn, sum);
                    }
                }
                if (!first) dnext[i] = di;
                a.q[i] = sum;
                floc = fmaf(di, sum, floc);
            }
            fbs = block_sumf<PCG_THREADS>(floc, sh);
            if (threadIdx.x == 0) a.pdq[par * P + blockIdx.x] = (double)fbs;
            if (!grid_barrier(a.bar, nblocks, a.st)) return;
            float dq = (float)sum_partials(a.pdq + par * P, gridDim.x, sh);
            par ^= 1;
            float alpha = delta_new / dq;
            float *dv = first ? dcur : dnext;
            floc = 0.0f;
            for (long i = t0; i < n; i += stride) {
                float di = dv[i];
                a.x[i] = a.x[i] + (double)(alpha * di);
                float ri = fmaf(-alpha, a.q[i], a.r[i]);
                a.r[i] = ri;
                float si = a.minv[i] * ri;
                a.s[i] = si;
                floc = fmaf(ri, si, floc);
            }
            fbs = block_sumf<PCG_THREADS>(floc, sh);
            if (threadIdx.x == 0) a.pdelta[par * P + blockIdx.x] = (double)fbs;
            if (!grid_barrier(a.bar, nblocks, a.st)) return;
            float delta_old = delta_new;
            delta_new = (float)sum_partials(a.pdelta + par * P, gridDim.x, sh);
            par ^= 1;
            beta = delta_new / delta_old;
            if (!first) {
                float *t = dcur;
                dcur = dnext;
                dnext = t;
            }
            first = false;
            ++iters;
            if (delta_new < inner_tol * din0 || !(delta_new > 0.0f)) break;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.iters = iters;
}

// -------------------------------------------------------------------- packed runs
// A packed context holds several independent runs; its free-surface matrix is block diagonal.
// Each run keeps its own PCG: the grid's blocks are split among the runs (run_block_start), a
// block works only on its run's rows, and after every grid barrier each block recomputes every
// run's scalars from the per-block partial sums in a fixed order, so all blocks agree on every
// run's alpha, beta and stop test, and on when all runs have stopped.  A converged run freezes
// while the others continue; the kernel ends when every run has stopped.

struct RunRows {
    int run, c0, c1;     // run index, rows [c0, c1)
    long start, stride;  // first row of this thread, row stride within the run
};

__device__ __forceinline__ RunRows run_rows(const Geom &g, const int *run_block_start) {
    int lo = 0, hi = g.NR;   // find r with run_block_start[r] <= blockIdx.x < run_block_start[r+1]
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (run_block_start[mid] <= (int)blockIdx.x) lo = mid;
        else hi = mid;
    }
    RunRows rr;
    rr.run = lo;
    rr.c0 = g.run_cell_start[lo];
    rr.c1 = g.run_cell_start[lo + 1];
    int nb = run_block_start[lo + 1] - run_block_start[lo];
    rr.start = rr.c0 + (long)(blockIdx.x - run_block_start[lo]) * blockDim.x + threadIdx.x;
    rr.stride = (long)nb * blockDim.x;
    return rr;
}

// sum of run r's block partials in block order
__device__ __forceinline__ double run_sum(const double *part, const int *run_block_start, int r) {
    double t = 0.0;
    for (int b = run_block_start[r]; b < run_block_start[r + 1]; ++b) t += ((volatile const double *)part)[b];
    return t;
}

struct PcgSegArgs {
    Geom g;
    const double *sp, *b;
    double *x, *minv, *r, *s, *q, *dA, *dB, *pdq, *pdelta;
    const int *run_block_start;
    int *run_iters;
    unsigned *bar;
    int *iters;
    int maxit;
    double tol;
    gom_status *st;
    unsigned phantom;
};

__global__ void __launch_bounds__(PCG_THREADS) k_pcg_seg(PcgSegArgs a) {
    __shared__ double sh[40];
    __shared__ double s_d0[PCG_MAX_RUNS], s_dn[PCG_MAX_RUNS], s_alpha[PCG_MAX_RUNS], s_beta[PCG_MAX_RUNS];
    __shared__ int s_done[PCG_MAX_RUNS], s_it[PCG_MAX_RUNS];
    const Geom &g = a.g;
    const int NR = g.NR;
    const unsigned nblocks = gridDim.x + a.phantom;
    const RunRows me = run_rows(g, a.run_block_start);
    double loc = 0.0;
    for (long i = me.start; i < me.c1; i += me.stride) {
        const double *row = a.sp + i * 5;
        int cell = (int)i + 1;
        double sum = row[0] * a.x[i];
        int tq = g.tri_or_quad[i];
        for (int l = 1; l <= tq; ++l) {
            int nb = g.cell_adj(l, cell);
            if (nb != 0) sum = fma(row[l], a.x[nb - 1], sum);
        }
        double mi = 1.0 / row[0];
        double ri = a.b[i] - sum;
        double di = mi * ri;
        a.minv[i] = mi;
        a.r[i] = ri;
        a.dA[i] = di;
        loc = fma(ri, di, loc);
    }
    double bs = block_sum<PCG_THREADS>(loc, sh);
    if (threadIdx.x == 0) a.pdelta[blockIdx.x] = bs;
    if (!grid_barrier(a.bar, nblocks, a.st)) return;
    for (int r = threadIdx.x; r < NR; r += blockDim.x) {
        double d0 = run_sum(a.pdelta, a.run_block_start, r);
        s_d0[r] = d0;
        s_dn[r] = d0;
        s_done[r] = d0 == 0.0;
        s_it[r] = 0;
    }
    __syncthreads();
    double *dcur = a.dA, *dnext = a.dB;
    bool first = true;
    // no early exit on a failure recorded elsewhere: a failure belongs to one run, and the other
    // runs' solves must complete (a barrier that times out ends the solve by itself)
    for (int it = 1; it <= a.maxit; ++it) {
        int active = 0;
        for (int r = 0; r < NR; ++r) active |= !s_done[r];
        if (!active) break;
        const bool mine = !s_done[me.run];
        loc = 0.0;
        if (mine) {
            const double beta = s_beta[me.run];
            for (long i = me.start; i < me.c1; i += me.stride) {
                const double *row = a.sp + i * 5;
                int cell = (int)i + 1;
                double di = first ? dcur[i] : fma(beta, dcur[i], a.s[i]);
                double sum = row[0] * di;
                int tq = g.tri_or_quad[i];
                for (int l = 1; l <= tq; ++l) {
                    int nb = g.cell_adj(l, cell);
                    if (nb != 0) {
                        double dn = first ? dcur[nb - 1] : fma(beta, dcur[nb - 1], a.s[nb - 1]);
                        sum = fma(row[l], dn, sum);
                    }
                }
                if (!first) dnext[i] = di;
                a.q[i] = sum;
                loc = fma(di, sum, loc);
            }
        }
        bs = block_sum<PCG_THREADS>(loc, sh);
        if (threadIdx.x == 0) a.pdq[blockIdx.x] = bs;
        if (!grid_barrier(a.bar, nblocks, a.st)) return;
        for (int r = threadIdx.x; r < NR; r += blockDim.x)
            if (!s_done[r]) s_alpha[r] = s_dn[r] / run_sum(a.pdq, a.run_block_start, r);
        __syncthreads();
        loc = 0.0;
        if (mine) {
            const double alpha = s_alpha[me.run];
            double *dv = first ? dcur : dnext;
            for (long i = me.start; i < me.c1; i += me.stride) {
                double di = dv[i];
                a.x[i] = fma(alpha, di, a.x[i]);
                double ri = fma(-alpha, a.q[i], a.r[i]);
                a.r[i] = ri;
                double si = a.minv[i] * ri;
                a.s[i] = si;
                loc = fma(ri, si, loc);
            }
        }
        bs = block_sum<PCG_THREADS>(loc, sh);
        if (threadIdx.x == 0) a.pdelta[blockIdx.x] = bs;
        if (!grid_barrier(a.bar, nblocks, a.st)) return;
        for (int r = threadIdx.x; r < NR; r += blockDim.x) {
            if (s_done[r]) continue;
            double dold = s_dn[r];
            double dn = run_sum(a.pdelta, a.run_block_start, r);
            s_dn[r] = dn;
            s_beta[r] = dn / dold;
            s_it[r] = it;
            if (sqrt(dn * dn / (s_d0[r] * s_d0[r])) < a.tol) s_done[r] = 1;
        }
        __syncthreads();
        if (!first) {
            double *t = dcur;
            dcur = dnext;
            dnext = t;
        }
        first = false;
    }
    if (blockIdx.x == 0) {
        for (int r = threadIdx.x; r < NR; r += blockDim.x) a.run_iters[r] = s_it[r];
        if (threadIdx.x == 0) {
            int mx = 0;
            for (int r = 0; r < NR; ++r) mx = max(mx, s_it[r]);
            *a.iters = mx;
        }
    }
}

// mixed precision, packed runs: each run runs the refinement / inner-iteration scheme of
// k_pcg_mixed as a state machine (true-residual pass, then inner iterations until its inner
// stop, then a residual pass again ...).  The runs are independent, so each run's blocks meet
// only at the run's own barrier (bar + 2 r): a run's step costs a barrier over its few blocks
// instead of the whole grid, a run that has converged leaves, and the others do not wait for
// it.  All blocks of a run recompute its scalars from its block partials in block order, so they
// agree on every decision.  Partial sums alternate between two halves of pdq / pdelta with every
// barrier (as in k_pcg_mixed).
struct PcgMixedSegArgs {
    Geom g;
    const double *sp, *b;
    double *x;
    float *sp32, *minv, *r, *s, *q, *dA, *dB;
    double *pdq, *pdelta;
    const int *run_block_start;
    int *run_iters;
    unsigned *bar;
    int *iters;   // zero at launch; the largest per-run inner count on return
    int maxit;
    double tol;
    gom_status *st;
    unsigned phantom;
};

enum { RUN_RESID = 0, RUN_INNER = 1, RUN_DONE = 2 };

__global__ void __launch_bounds__(PCG_THREADS) k_pcg_mixed_seg(PcgMixedSegArgs a) {
    __shared__ double sh[40];
    const Geom &g = a.g;
    const RunRows me = run_rows(g, a.run_block_start);
    const int run = me.run;
    const int b0 = a.run_block_start[run];
    const unsigned nbar = (unsigned)(a.run_block_start[run + 1] - b0) + a.phantom;
    unsigned *bar = a.bar + 2 * run;
    const unsigned P = gridDim.x;
    const float FP32_FLOOR = 1e-10f;
    for (long i = me.start; i < me.c1; i += me.stride) {
        const double *row = a.sp + i * 5;
        float *row32 = a.sp32 + i * 5;
        for (int l = 0; l < 5; ++l) row32[l] = (float)row[l];
        a.minv[i] = (float)(1.0 / row[0]);
    }
    // the run's state (identical in all of its blocks)
    int mode = RUN_RESID, outer = 0, its = 0, dpar = 0, par = 0;
    bool first = true;
    double d0 = 0.0;
    float dn = 0.0f, din0 = 0.0f, itol = 0.0f, beta = 0.0f;
    // no early exit on a failure recorded elsewhere: it belongs to one run, and the others' solves
    // must complete (a barrier of this run that times out ends this run's solve by itself)
    for (;;) {
        if (mode == RUN_DONE) break;
        float *dcur = dpar ? a.dB : a.dA, *dnext = dpar ? a.dA : a.dB;
        // pass A: true residual (RESID) or inner matrix-vector product (INNER)
        double loc = 0.0;
        float floc = 0.0f;
        if (mode == RUN_RESID) {
            for (long i = me.start; i < me.c1; i += me.stride) {
                const double *row = a.sp + i * 5;
                int cell = (int)i + 1;
                double sum = row[0] * a.x[i];
                int tq = g.tri_or_quad[i];
                for (int l = 1; l <= tq; ++l) {
                    int nb = g.cell_adj(l, cell);
                    if (nb != 0) sum = fma(row[l], a.x[nb - 1], sum);
                }
                double ri = a.b[i] - sum;
                loc = fma(ri, ri / row[0], loc);
                float rf = (float)ri;
                float df = a.minv[i] * rf;
                a.r[i] = rf;
                a.dA[i] = df;
                floc = fmaf(rf, df, floc);
            }
        } else {
            for (long i = me.start; i < me.c1; i += me.stride) {
                const float *row = a.sp32 + i * 5;
                int cell = (int)i + 1;
                float di = first ? dcur[i] : fmaf(beta, dcur[i], a.s[i]);
                float sum = row[0] * di;
                int tq = g.tri_or_quad[i];
                for (int l = 1; l <= tq; ++l) {
                    int nb = g.cell_adj(l, cell);
                    if (nb != 0) {
                        float dnb = first ? dcur[nb - 1] : fmaf(beta, dcur[nb - 1], a.s[nb - 1]);
                        sum = fmaf(row[l], dnb, sum);
                    }
                }
                if (!first) dnext[i] = di;
                a.q[i] = sum;
                floc = fmaf(di, sum, floc);
            }
        }
        double bs = block_sum<PCG_THREADS>(loc, sh);
        float fbs = block_sumf<PCG_THREADS>(floc, sh);
        if (threadIdx.x == 0) {
            a.pdelta[par * P + blockIdx.x] = bs;
            a.pdq[par * P + blockIdx.x] = (double)fbs;
        }
        if (!grid_barrier(bar, nbar, a.st)) return;
        if (mode == RUN_RESID) {
            const double dt = run_sum(a.pdelta + par * P, a.run_block_start, run);
            const float di = (float)run_sum(a.pdq + par * P, a.run_block_start, run);
            par ^= 1;
            bool stop;
            if (outer == 0) {
                d0 = dt;
                stop = dt == 0.0;
            } else {
                stop = sqrt(dt * dt / (d0 * d0)) < a.tol;
            }
            if (stop || its >= a.maxit || !(di > 0.0f)) {
                mode = RUN_DONE;
            } else {
                mode = RUN_INNER;
                outer += 1;
                din0 = di;
                dn = di;
                itol = fmaxf((float)(0.25 * a.tol * d0 / dt), FP32_FLOOR);
                first = true;
                dpar = 0;
            }
            if (outer == 0) outer = 1;
            continue;
        }
        // pass B: the inner update
        const float alpha = dn / (float)run_sum(a.pdq + par * P, a.run_block_start, run);
        par ^= 1;
        floc = 0.0f;
        {
            float *dv = first ? dcur : dnext;
            for (long i = me.start; i < me.c1; i += me.stride) {
                float di = dv[i];
                a.x[i] = a.x[i] + (double)(alpha * di);
                float ri = fmaf(-alpha, a.q[i], a.r[i]);
                a.r[i] = ri;
                float si = a.minv[i] * ri;
                a.s[i] = si;
                floc = fmaf(ri, si, floc);
            }
        }
        fbs = block_sumf<PCG_THREADS>(floc, sh);
        if (threadIdx.x == 0) a.pdelta[par * P + blockIdx.x] = (double)fbs;
        if (!grid_barrier(bar, nbar, a.st)) return;
        const float dold = dn;
        dn = (float)run_sum(a.pdelta + par * P, a.run_block_start, run);
        par ^= 1;
        beta = dn / dold;
        if (!first) dpar ^= 1;
        first = false;
        its += 1;
        if (dn < itol * din0 || !(dn > 0.0f) || its >= a.maxit) mode = RUN_RESID;
    }
    if ((int)blockIdx.x == b0 && threadIdx.x == 0) {
        a.run_iters[run] = its;
        atomicMax(a.iters, its);
    }
}

// grid of the cooperative launch: enough blocks for one row per thread, at most two resident
// blocks per SM (and never more than the occupancy allows)
inline int pcg_blocks_for(long n_rows, int per_sm, int num_sms) {
    if (per_sm < 1) per_sm = 1;
    long need = (n_rows + PCG_THREADS - 1) / PCG_THREADS;
    long maxb = (long)per_sm * num_sms;
    long cap = (long)num_sms * (per_sm < 2 ? per_sm : 2);
    if (cap > maxb) cap = maxb;
    long b = need < cap ? need : cap;
    return b < 1 ? 1 : (int)b;
}

}  // namespace
}  // namespace gom
