// k_surface.cu -- theta-scheme free surface (assembly + Jacobi-PCG), node elevations, velocity
// recovery, layer/wet-dry update and node velocities, for sm_103a.
//
// References (GOM_Rv1.1.0/source):
//   solve_free_surface_equation.f90:17-396, pre_conj_grad.f90:9-230, solve_velocities.f90:8-260,
//   update_vertical_layers_1.f90:18-333, calculate_velocity_at_node.f90:10-140.
#include "gom_launch.h"
#include "gom_pcg.cuh"
#include "gom_scan.cuh"

#include <algorithm>
#include <vector>

namespace gom {

// ============================================================================================
// solve_free_surface_equation.f90:65-214: one thread per cell builds its 5-point row and RHS.
// The system and its right-hand side are formed in FP64 whatever the storage type R.
// Per-face column sums of the assembly (:66-130, :134-151, :185-212), formed once per face
// instead of once per adjacent cell (same expressions in the same order, hence the same values):
// fs = [gravity dt^2 theta^2 fl/dj * sum dz AinvDZ1, sum dz un, sum dz AinvG1] per face.
template <typename R> __global__ void k_fs_face_sums(Geom g, StateT<R> s, Params p, double *fs) {
    unsigned tid = flat_tid();
    if (tid >= (unsigned)g.NF) return;
    const int j = column_entity<R>(g.face_order, tid);
    const int L = g.L;
    const int tj = s.top_face[j - 1];
    double *o = fs + (long)(j - 1) * 3;
    if (tj == 0) return;   // not read
    const double dt = p.dt, gravity = p.gravity, theta = p.theta;
    const double gdt2th2 = gravity * (dt * dt) * (theta * theta);
    const int nvl = tj - g.bottom_face[j - 1] + 1;
    double sdz = 0.0, c1 = 0.0, c2 = 0.0;
    for (int k = 1; k <= nvl; ++k) {
        const int kk = tj + 1 - k;
        const double dz = s.dz_face[ix(kk, j, L)];
        sdz = sdz + dz * (double)s.ainvdz1[ix(k, j, L)];
        c1 = c1 + dz * (double)s.un_face[ix(kk, j, L)];
        c2 = c2 + dz * (double)s.ainvg1[ix(k, j, L)];
    }
    o[0] = gdt2th2 * g.face_length[j - 1] / g.delta_j[j - 1] * sdz;
    o[1] = c1;
    o[2] = c2;
}

// solve_free_surface_equation.f90:65-212: matrix row and right-hand side of each cell
template <typename R>
__global__ void k_fs_assemble(Geom g, StateT<R> s, Forcing f, Params p, const double *fs, double *sparsem, double *rhs,
                              gom_status *st) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i > g.NC) return;
    const double dt = p.dt, theta = p.theta;
    int tq = g.tri_or_quad[i - 1];
    double ar = g.area[i - 1];
    double diag = ar;
    double off[4] = {0.0, 0.0, 0.0, 0.0};
    double r = ar * s.eta_cell[i - 1];
    int obf = g.ob_element_flag[i - 1];
    for (int l = 1; l <= tq; ++l) {
        int j = g.cell_face(l, i);
        if (s.top_face[j - 1] == 0) continue;
        double coef = fs[(long)(j - 1) * 3] * g.cos_theta2[j - 1];
        if (coef < 0.0) {
            record_error(st, GOM_E_NOT_SPD, 100, i, 0, coef, GOM_ENTITY_CELL);
            return;
        }
        diag = diag + coef;
        if (g.cell_adj(l, i) != 0) off[l - 1] = -coef;
    }
    // RHS (:134-151), computed in a second pass like the reference
    for (int l = 1; l <= tq; ++l) {
        int j = g.cell_face(l, i);
        if (s.top_face[j - 1] == 0) continue;
        const double c1 = fs[(long)(j - 1) * 3 + 1], c2 = fs[(long)(j - 1) * 3 + 2];
        double sgn = (double)g.cell_sign(l, i);
        double fl = g.face_length[j - 1];
        r = r - (1.0 - theta) * dt * sgn * fl * c1 - theta * dt * sgn * fl * c2;
    }
    // open-boundary Dirichlet term (:185-212)
    if (obf > 0) {
        for (int l = 1; l <= tq; ++l) {
            int j = g.cell_face(l, i);
            if (g.boundary_type_of_face[j - 1] > 0 && s.top_face[j - 1] != 0)
                r = r + fs[(long)(j - 1) * 3] * f.eta_at_ob_new[obf - 1];
        }
    }
    double *row = sparsem + (long)(i - 1) * 5;
    row[0] = diag;
    row[1] = off[0];
    row[2] = off[1];
    row[3] = off[2];
    row[4] = off[3];
    rhs[i - 1] = r;
}

// :353-375 node elevation from wet cells; wetdry_node
template <typename R> __global__ void k_node_eta(Geom g, StateT<R> s) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i > g.NN) return;
    int wd = 0;
    double sum1 = 0.0, sum0 = 0.0;
    int na = g.adj_cells_at_node[i - 1];
    for (int j = 1; j <= na; ++j) {
        int ie = g.node_cell(j, i);
        if (s.top_cell[ie - 1] == 0) wd = 1;
        else {
            double ar = g.area[ie - 1];
            sum1 = sum1 + ar * s.eta_cell_new[ie - 1];
            sum0 = sum0 + ar;
        }
    }
    s.wetdry_node[i - 1] = wd;
    if (wd == 0) s.eta_node[i - 1] = sum1 / sum0;
}

// :378-394 dry nodes take the mean of their wet neighbours
template <typename R> __global__ void k_node_eta_dry(Geom g, StateT<R> s) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i > g.NN) return;
    if (s.wetdry_node[i - 1] != 1) return;
    double sum0 = 0.0;
    int icount = 0;
    int nn = g.adj_nodes_at_node[i - 1];
    for (int j = 1; j <= nn; ++j) {
        int nd = g.node_nb(j, i);
        if (s.wetdry_node[nd - 1] == 0) {
            icount = icount + 1;
            sum0 = sum0 + s.eta_node[nd - 1];
        }
    }
    if (icount != 0) s.eta_node[i - 1] = sum0 / icount;
}

template <typename R> cudaError_t pcg_configure(LaunchT<R> &x, int device) {
    // every block of the cooperative grid must be resident, whichever solver the context uses
    int per_sm = 1 << 30;
    const void *kernels[] = {(const void *)k_pcg_mixed, (const void *)k_pcg_seg, (const void *)k_pcg_mixed_seg};
    for (const void *k : kernels) {
        int n = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, PCG_THREADS, 0);
        if (e != cudaSuccess) return e;
        per_sm = std::min(per_sm, n);
    }
    if (per_sm < 1) per_sm = 1;
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
    if (!coop) return cudaErrorNotSupported;
    x.w.pcg_threads = PCG_THREADS;
    if (x.g.NR <= 1) {
        x.w.pcg_blocks = pcg_blocks_for(x.g.NC, per_sm, x.num_sms);
        // the single-run FP64 solver: one block of PCG_CG_THREADS per SM
        for (const void *k : {(const void *)k_pcg_cg1<PCG_CG_ROWS>, (const void *)k_pcg_cg1<0>}) {
            int cg_per_sm = 0;
            cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cg_per_sm, k, PCG_CG_THREADS, 0);
            if (e != cudaSuccess) return e;
            if (cg_per_sm < 1) return cudaErrorNotSupported;
        }
        return cudaSuccess;
    }
    // packed runs: one block at least per run, the rest of the grid split in proportion to the
    // rows (largest remainders), never more blocks than rows / threads
    const int NR = x.g.NR;
    std::vector<int> cs(NR + 1);
    cudaError_t e = cudaMemcpy(cs.data(), x.g.run_cell_start, (NR + 1) * sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return e;
    const long cap = (long)x.num_sms * std::min(per_sm, 2);
    if (NR > PCG_MAX_RUNS || NR > cap) return cudaErrorInvalidValue;
    std::vector<long> want(NR), got(NR, 1);
    long spare = cap - NR;
    const double total = (double)cs[NR];
    std::vector<std::pair<double, int>> rem;
    for (int r = 0; r < NR; ++r) {
        long rows = cs[r + 1] - cs[r];
        want[r] = std::max(1L, (rows + PCG_THREADS - 1) / PCG_THREADS);
        double share = spare * (rows / total);
        long extra = std::min((long)share, want[r] - 1);
        got[r] += extra;
        rem.push_back({share - (double)(long)share, r});
    }
    long used = 0;
    for (long v : got) used += v;
    std::sort(rem.begin(), rem.end(), [](auto &p, auto &q) { return p.first > q.first || (p.first == q.first && p.second < q.second); });
    for (auto &pr : rem) {
        if (used >= cap) break;
        if (got[pr.second] < want[pr.second]) {
            got[pr.second] += 1;
            used += 1;
        }
    }
    std::vector<int> rbs(NR + 1, 0);
    for (int r = 0; r < NR; ++r) rbs[r + 1] = rbs[r] + (int)got[r];
    x.w.pcg_blocks = rbs[NR];
    return cudaMemcpy(x.w.run_block_start, rbs.data(), (NR + 1) * sizeof(int), cudaMemcpyHostToDevice);
}

template <typename R> cudaError_t launch_free_surface(const LaunchT<R> &x) {
    const Geom &g = x.g;
    k_fs_face_sums<<<blocks_for(g.NF, 128), 128, 0, x.stream>>>(x.g, x.s, x.p, x.w.fs_sums);
    k_fs_assemble<<<blocks_for(g.NC, 128), 128, 0, x.stream>>>(x.g, x.s, x.f, x.p, x.w.fs_sums, x.w.sparsem, x.w.rhs,
                                                               x.status);
    cudaError_t e = cudaMemsetAsync(x.w.barrier, 0, 2 * sizeof(unsigned) * (size_t)std::max(1, g.NR), x.stream);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(x.w.pcg_blocks);
    cfg.blockDim = dim3(x.w.pcg_threads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = x.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const unsigned phantom = (unsigned)(x.p.test_barrier_phantom_blocks > 0 ? x.p.test_barrier_phantom_blocks : 0);
    if (g.NR > 1 && x.w.sp32) {
        PcgMixedSegArgs m;
        m.g = g;
        m.sp = x.w.sparsem;
        m.b = x.w.rhs;
        m.x = x.s.eta_cell_new;
        m.sp32 = x.w.sp32;
        m.minv = reinterpret_cast<float *>(x.w.minv);
        m.r = reinterpret_cast<float *>(x.w.r);
        m.s = reinterpret_cast<float *>(x.w.s);
        m.q = reinterpret_cast<float *>(x.w.q);
        m.dA = reinterpret_cast<float *>(x.w.d0);
        m.dB = reinterpret_cast<float *>(x.w.d1);
        m.pdq = x.w.partial_dq;
        m.pdelta = x.w.partial_delta;
        m.run_block_start = x.w.run_block_start;
        m.run_iters = x.w.run_iters;
        m.bar = x.w.barrier;
        m.iters = x.w.pcg_iters;
        m.maxit = x.p.max_iteration_pcg;
        m.tol = x.p.error_tolerance;
        m.st = x.status;
        m.phantom = phantom;
        e = cudaMemsetAsync(x.w.pcg_iters, 0, sizeof(int), x.stream);
        if (e == cudaSuccess) e = cudaLaunchKernelEx(&cfg, k_pcg_mixed_seg, m);
    } else if (g.NR > 1) {
        PcgSegArgs m;
        m.g = g;
        m.sp = x.w.sparsem;
        m.b = x.w.rhs;
        m.x = x.s.eta_cell_new;
        m.minv = x.w.minv;
        m.r = x.w.r;
        m.s = x.w.s;
        m.q = x.w.q;
        m.dA = x.w.d0;
        m.dB = x.w.d1;
        m.pdq = x.w.partial_dq;
        m.pdelta = x.w.partial_delta;
        m.run_block_start = x.w.run_block_start;
        m.run_iters = x.w.run_iters;
        m.bar = x.w.barrier;
        m.iters = x.w.pcg_iters;
        m.maxit = x.p.max_iteration_pcg;
        m.tol = x.p.error_tolerance;
        m.st = x.status;
        m.phantom = phantom;
        e = cudaLaunchKernelEx(&cfg, k_pcg_seg, m);
    }
    if (g.NR > 1) {
        if (e != cudaSuccess) return e;
        k_node_eta<<<blocks_for(g.NN, 256), 256, 0, x.stream>>>(x.g, x.s);
        k_node_eta_dry<<<blocks_for(g.NN, 256), 256, 0, x.stream>>>(x.g, x.s);
        return cudaGetLastError();
    }
    if (x.w.sp32) {
        // mixed precision: the FP64 work vectors hold the FP32 inner vectors
        PcgMixedArgs m;
        m.g = g;
        m.sp = x.w.sparsem;
        m.b = x.w.rhs;
        m.x = x.s.eta_cell_new;
        m.sp32 = x.w.sp32;
        m.minv = reinterpret_cast<float *>(x.w.minv);
        m.r = reinterpret_cast<float *>(x.w.r);
        m.s = reinterpret_cast<float *>(x.w.s);
        m.q = reinterpret_cast<float *>(x.w.q);
        m.dA = reinterpret_cast<float *>(x.w.d0);
        m.dB = reinterpret_cast<float *>(x.w.d1);
        m.pdq = x.w.partial_dq;
        m.pdelta = x.w.partial_delta;
        m.bar = x.w.barrier;
        m.iters = x.w.pcg_iters;
        m.maxit = x.p.max_iteration_pcg;
        m.tol = x.p.error_tolerance;
        m.st = x.status;
        m.phantom = phantom;
        e = cudaLaunchKernelEx(&cfg, k_pcg_mixed, m);
        if (e != cudaSuccess) return e;
        k_node_eta<<<blocks_for(g.NN, 256), 256, 0, x.stream>>>(x.g, x.s);
        k_node_eta_dry<<<blocks_for(g.NN, 256), 256, 0, x.stream>>>(x.g, x.s);
        return cudaGetLastError();
    }
    PcgArgs a;
    a.g = g;
    a.sp = x.w.sparsem;
    a.b = x.w.rhs;
    a.x = x.s.eta_cell_new;
    a.dr = x.w.minv;
    a.xs = x.w.cg_xs;
    a.p = x.w.d0;
    a.r[0] = x.w.r;
    a.r[1] = x.w.d1;
    a.s[0] = x.w.s;
    a.s[1] = x.w.cg_s1;
    a.w[0] = x.w.q;
    a.w[1] = x.w.cg_w1;
    a.pg = x.w.partial_dq;
    a.pd = x.w.partial_delta;
    a.bar = x.w.barrier;
    a.iters = x.w.pcg_iters;
    a.maxit = x.p.max_iteration_pcg;
    a.tol = x.p.error_tolerance;
    a.st = x.status;
    a.phantom = phantom;
    a.check_diag = 0;   // k_fs_assemble has checked every row
    e = launch_pcg_cg1(cfg, a, x.num_sms);
    if (e != cudaSuccess) return e;
    k_node_eta<<<blocks_for(g.NN, 256), 256, 0, x.stream>>>(x.g, x.s);
    k_node_eta_dry<<<blocks_for(g.NN, 256), 256, 0, x.stream>>>(x.g, x.s);
    return cudaGetLastError();
}

// ============================================================================================
// solve_velocities.f90:23-184: one thread per face column.  The elevation gradients are formed
// in FP64 per face; the per-layer products run in R.
template <typename R> __global__ void k_face_velocity(Geom g, StateT<R> s, Forcing f, Params p) {
    unsigned tid = flat_tid();
    if (tid >= (unsigned)g.NF) return;
    int j = column_entity<R>(g.face_order, tid);
    const int L = g.L;
    int tj = s.top_face[j - 1];
    if (tj == 0) {
        for (int k = 1; k <= L; ++k) {
            s.un_face_new[ix(k, j, L)] = R(0);
            s.vn_face_new[ix(k, j, L)] = R(0);
        }
        return;
    }
    const double dt = p.dt, gravity = p.gravity, theta = p.theta;
    int bj = g.bottom_face[j - 1];
    int n1 = g.face_node(1, j), n2 = g.face_node(2, j);
    int btype = g.boundary_type_of_face[j - 1];
    int a1 = g.face_cell(1, j), a2 = g.face_cell(2, j);
    bool wet = s.wetdry_node[n1 - 1] == 0 && s.wetdry_node[n2 - 1] == 0;
    bool init_dry = g.initial_wetdry_node[n1 - 1] == 1 || g.initial_wetdry_node[n2 - 1] == 1;
    double dj = g.delta_j[j - 1], fl = g.face_length[j - 1];
    double dEta = 0.0;
    if (btype == 0) dEta = s.eta_cell_new[a2 - 1] - s.eta_cell_new[a1 - 1];
    else if (btype > 0) dEta = f.eta_at_ob_new[g.ob_element_flag[a1 - 1] - 1] - s.eta_cell_new[a1 - 1];
    double dEtaN = s.eta_node[n2 - 1] - s.eta_node[n1 - 1];
    // theta*g*dt/dj*dEta and theta*g*dt/fl*dEtaN: the layer-independent left factors
    const R cj = (R)(theta * gravity * dt / dj * dEta), cn = (R)(theta * gravity * dt / fl * dEtaN);
    const R ct2 = (R)g.cos_theta2[j - 1], sn2 = (R)g.sin_theta2[j - 1];
    for (int k = 1; k <= tj - bj + 1; ++k) {
        int kk = tj + 1 - k;
        long o = ix(kk, j, L), ok = ix(k, j, L);
        R rtemp2 = R(0);
        if (btype == -1) {
            s.un_face_new[o] = R(0);
        } else if (btype == 0) {
            R rtemp0 = cj * s.ainvdz1[ok];
            R rtemp1 = rtemp0 * ct2;
            rtemp2 = rtemp0 * sn2;
            s.un_face_new[o] = s.ainvg1[ok] - rtemp1;
        } else {
            R rtemp0 = cj * s.ainvdz1[ok];
            s.un_face_new[o] = s.ainvg1[ok] - rtemp0;
        }
        if (wet) {
            R rtemp1 = cn * s.ainvdz2[ok];
            if (btype == 0) s.vn_face_new[o] = s.ainvg2[ok] - (rtemp1 + rtemp2);
            else s.vn_face_new[o] = s.ainvg2[ok] - rtemp1;
        }
        if (init_dry) s.vn_face_new[o] = fmax(R(-5), fmin(s.vn_face_new[o], R(5)));
    }
    int ibnd = g.isflowside3[j - 1];
    if (ibnd > 0) {
        R qu = (R)s.qu_boundary[ibnd - 1];
        for (int k = bj; k <= tj; ++k) s.un_face_new[ix(k, j, L)] = qu;
    }
    for (int k = 1; k <= bj - 1; ++k) {
        s.un_face_new[ix(k, j, L)] = R(0);
        s.vn_face_new[ix(k, j, L)] = R(0);
    }
    R ut = s.un_face_new[ix(tj, j, L)], vt = s.vn_face_new[ix(tj, j, L)];
    for (int k = tj + 1; k <= L; ++k) {
        s.un_face_new[ix(k, j, L)] = ut;
        s.vn_face_new[ix(k, j, L)] = vt;
    }
}

// FP32 path, the same per face: a block takes VT_TILE consecutive faces, forms each face's
// FP64 elevation factors once into shared memory, then sweeps the block's (layer, face) tile --
// contiguous in the (L, NF) arrays -- one thread per slot, so loads and stores are coalesced.
// Values and operation order are those of k_face_velocity<float>.  A face with a dry node keeps
// vn_face_new of its wet layers as it is (clamped at initially dry nodes), as the column kernel
// does; the layers above the top copy the top layer's values.
constexpr int VT_TILE = 64;

__global__ void __launch_bounds__(256) k_face_velocity_tile(Geom g, StateT<float> s, Forcing f, Params p) {
    __shared__ float cj_s[VT_TILE], cn_s[VT_TILE], ct2_s[VT_TILE], sn2_s[VT_TILE], qu_s[VT_TILE];
    __shared__ int tj_s[VT_TILE], bj_s[VT_TILE], bt_s[VT_TILE], fl_s[VT_TILE];
    const int j0 = blockIdx.x * VT_TILE;   // 0-based first face of the tile
    const int nf = min(VT_TILE, g.NF - j0);
    const int L = g.L;
    for (int t = threadIdx.x; t < nf; t += blockDim.x) {
        const int j = j0 + t + 1;
        const int tj = s.top_face[j - 1];
        tj_s[t] = tj;
        bj_s[t] = g.bottom_face[j - 1];
        if (tj == 0) continue;
        const int n1 = g.face_node(1, j), n2 = g.face_node(2, j);
        const int btype = g.boundary_type_of_face[j - 1];
        const int a1 = g.face_cell(1, j), a2 = g.face_cell(2, j);
        const bool wet = s.wetdry_node[n1 - 1] == 0 && s.wetdry_node[n2 - 1] == 0;
        const bool init_dry = g.initial_wetdry_node[n1 - 1] == 1 || g.initial_wetdry_node[n2 - 1] == 1;
        double dEta = 0.0;
        if (btype == 0) dEta = s.eta_cell_new[a2 - 1] - s.eta_cell_new[a1 - 1];
        else if (btype > 0) dEta = f.eta_at_ob_new[g.ob_element_flag[a1 - 1] - 1] - s.eta_cell_new[a1 - 1];
        const double dEtaN = s.eta_node[n2 - 1] - s.eta_node[n1 - 1];
        cj_s[t] = (float)(p.theta * p.gravity * p.dt / g.delta_j[j - 1] * dEta);
        cn_s[t] = (float)(p.theta * p.gravity * p.dt / g.face_length[j - 1] * dEtaN);
        ct2_s[t] = (float)g.cos_theta2[j - 1];
        sn2_s[t] = (float)g.sin_theta2[j - 1];
        bt_s[t] = btype;
        const int ibnd = g.isflowside3[j - 1];
        qu_s[t] = ibnd > 0 ? (float)s.qu_boundary[ibnd - 1] : 0.0f;
        fl_s[t] = (wet ? 1 : 0) | (init_dry ? 2 : 0) | (ibnd > 0 ? 4 : 0);
    }
    __syncthreads();
    const long base = (long)j0 * L;
    for (int t = threadIdx.x; t < nf * L; t += blockDim.x) {
        const int fi = t / L, kk = t - fi * L + 1;
        const long o = base + t;
        const int tj = tj_s[fi], bj = bj_s[fi];
        if (tj == 0 || kk < bj) {
            s.un_face_new[o] = 0.0f;
            s.vn_face_new[o] = 0.0f;
            continue;
        }
        const int kq = kk > tj ? tj : kk;       // layers above the top take the top layer's values
        const long oq = base + (long)fi * L + (kq - 1);
        const long orow = base + (long)fi * L + (tj - kq);   // top-down row tj + 1 - kq
        const int btype = bt_s[fi], fl = fl_s[fi];
        const float cj = cj_s[fi];
        float un, rtemp2 = 0.0f;
        if (btype == -1) {
            un = 0.0f;
        } else if (btype == 0) {
            const float rtemp0 = cj * s.ainvdz1[orow];
            const float rtemp1 = rtemp0 * ct2_s[fi];
            rtemp2 = rtemp0 * sn2_s[fi];
            un = s.ainvg1[orow] - rtemp1;
        } else {
            const float rtemp0 = cj * s.ainvdz1[orow];
            un = s.ainvg1[orow] - rtemp0;
        }
        if (fl & 4) un = qu_s[fi];
        s.un_face_new[o] = un;
        float vn;
        bool write_v = true;
        if (fl & 1) {
            const float rtemp1 = cn_s[fi] * s.ainvdz2[orow];
            if (btype == 0) vn = s.ainvg2[orow] - (rtemp1 + rtemp2);
            else vn = s.ainvg2[orow] - rtemp1;
        } else {
            vn = s.vn_face_new[oq];   // kept from before
            write_v = kk != kq || (fl & 2);
        }
        if (fl & 2) vn = fmaxf(-5.0f, fminf(vn, 5.0f));
        if (write_v) s.vn_face_new[o] = vn;
    }
}

// solve_velocities.f90:191-258: one thread per cell column
template <typename R> __global__ void k_cell_w(Geom g, StateT<R> s) {
    unsigned tid = flat_tid();
    if (tid >= (unsigned)g.NC) return;
    int i = column_entity<R>(g.cell_order, tid);
    const int L = g.L;
    int t = s.top_cell[i - 1], b = g.bottom_cell[i - 1];
    if (t == 0) {
        for (int k = 0; k <= L; ++k) s.wn_cell_new[ix0(k, i, L)] = R(0);
        return;
    }
    int tq = g.tri_or_quad[i - 1];
    int fj[4], fb[4], ft[4];
    R fsl[4];
    for (int l = 1; l <= tq; ++l) {
        int jt = g.cell_face(l, i);
        fj[l - 1] = jt;
        fb[l - 1] = g.bottom_face[jt - 1];
        ft[l - 1] = s.top_face[jt - 1];
        fsl[l - 1] = (R)((double)g.cell_sign(l, i) * g.face_length[jt - 1]);
    }
    const R ar = (R)g.area[i - 1];
    R w = R(0);
    s.wn_cell_new[ix0(b - 1, i, L)] = R(0);
    for (int k = b; k <= t; ++k) {
        R sum1 = R(0);
        for (int l = 0; l < tq; ++l) {
            if (k >= fb[l] && k <= ft[l])
                sum1 = sum1 + fsl[l] * s.dz_face[ix(k, fj[l], L)] * s.un_face_new[ix(k, fj[l], L)];
        }
        w = w - sum1 / ar;
        s.wn_cell_new[ix0(k, i, L)] = w;
    }
    for (int k = 0; k <= b - 2; ++k) s.wn_cell_new[ix0(k, i, L)] = R(0);
    for (int k = t + 1; k <= L; ++k) s.wn_cell_new[ix0(k, i, L)] = w;
}

// FP32 path, the same per cell: a block takes VT_TILE consecutive cells; each (cell, layer) slot
// forms its face-flux sum divided by the area in one thread, each cell integrates its column
// upwards in shared memory in the column kernel's order, and the block writes its (0:L, cell)
// tile with coalesced stores.
__global__ void __launch_bounds__(256) k_cell_w_tile(Geom g, StateT<float> s) {
    __shared__ float inc[VT_TILE][GOM_MAXL + 1];
    __shared__ float fsl_s[VT_TILE][4];
    __shared__ int fj_s[VT_TILE][4], fb_s[VT_TILE][4], ft_s[VT_TILE][4];
    __shared__ int t_s[VT_TILE], b_s[VT_TILE], tq_s[VT_TILE];
    __shared__ float ar_s[VT_TILE];
    const int i0 = blockIdx.x * VT_TILE;
    const int nc = min(VT_TILE, g.NC - i0);
    const int L = g.L;
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        const int i = i0 + c + 1;
        const int t = s.top_cell[i - 1];
        t_s[c] = t;
        b_s[c] = g.bottom_cell[i - 1];
        const int tq = g.tri_or_quad[i - 1];
        tq_s[c] = tq;
        ar_s[c] = g.area_f[i - 1];
        for (int l = 1; l <= tq; ++l) {
            const int jt = g.cell_face(l, i);
            fj_s[c][l - 1] = jt;
            fb_s[c][l - 1] = g.bottom_face[jt - 1];
            ft_s[c][l - 1] = s.top_face[jt - 1];
            fsl_s[c][l - 1] = (float)((double)g.cell_sign(l, i) * g.face_length[jt - 1]);
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nc * L; t += blockDim.x) {
        const int c = t / L, k = t - c * L + 1;
        if (t_s[c] == 0 || k < b_s[c] || k > t_s[c]) continue;
        float sum1 = 0.0f;
        for (int l = 0; l < tq_s[c]; ++l) {
            if (k >= fb_s[c][l] && k <= ft_s[c][l]) {
                const long of = (long)(fj_s[c][l] - 1) * L + (k - 1);
                sum1 = sum1 + fsl_s[c][l] * s.dz_face[of] * s.un_face_new[of];
            }
        }
        inc[c][k] = sum1 / ar_s[c];
    }
    __syncthreads();
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        if (t_s[c] == 0) continue;
        float w = 0.0f;
        for (int k = b_s[c]; k <= t_s[c]; ++k) {
            w = w - inc[c][k];
            inc[c][k] = w;
        }
    }
    __syncthreads();
    const long base = (long)i0 * (L + 1);
    for (int t = threadIdx.x; t < nc * (L + 1); t += blockDim.x) {
        const int c = t / (L + 1), k = t - c * (L + 1);
        const int tt = t_s[c], bb = b_s[c];
        float v = 0.0f;
        if (tt != 0 && k >= bb) v = inc[c][k > tt ? tt : k];
        s.wn_cell_new[base + t] = v;
    }
}

template <typename R> cudaError_t launch_velocities(const LaunchT<R> &x) {
    if constexpr (sizeof(R) == sizeof(float)) {
        k_face_velocity_tile<<<blocks_for(x.g.NF, VT_TILE), 256, 0, x.stream>>>(x.g, x.s, x.f, x.p);
        k_cell_w_tile<<<blocks_for(x.g.NC, VT_TILE), 256, 0, x.stream>>>(x.g, x.s);
    } else {
        k_face_velocity<<<blocks_for(x.g.NF, 128), 128, 0, x.stream>>>(x.g, x.s, x.f, x.p);
        k_cell_w<<<blocks_for(x.g.NC, 128), 128, 0, x.stream>>>(x.g, x.s);
    }
    return cudaGetLastError();
}

// ============================================================================================
// update_vertical_layers_1.f90: new top layers and thicknesses for an entity column.
// kind 0 = cell (:42-133), 1 = face (:139-198), 2 = node (:204-254)
// FP64 thickness of layer k of a column with bottom layer b and top layer t > b
__device__ __forceinline__ double column_dz(const Geom &g, double msl, double h, double eta, int b, int t, int k) {
    if (k == t) return (msl + eta) - g.z_level[t - 1];
    if (k == b) return g.z_level[b] - (msl - h);
    return g.delta_z[k - 1];
}

// Thicknesses are formed in FP64 and rounded once to the storage type (with R = double this is
// the reference's arithmetic, half-thicknesses included).
template <int KIND, typename R>
__device__ __forceinline__ int new_column(const Geom &g, const Params &p, double h, double eta, int b, R *dz, R *dzh,
                                          long base_dz, long base_dzh, bool &bad) {
    const int L = g.L;
    const double MSL = p.msl;
    int tnew = 0;
    bad = false;
    double total = h + eta;
    if (total <= p.dry_depth) return 0;
    double tmp = MSL + eta;
    for (int k = L - 1; k >= 0; --k) {
        if (tmp > g.z_level[k] && tmp <= g.z_level[k + 1]) {
            tnew = k + 1;
            dz[base_dz + tnew - 1] = (R)(tmp - g.z_level[k]);
            break;
        }
    }
    if (tnew < b) {
        bad = true;
        return tnew;
    }
    if (tnew == b) {
        dz[base_dz + tnew - 1] = (R)total;
        if (KIND == 1) dzh[base_dzh + tnew - 1] = (R)total;
        dzh[base_dzh + tnew] = (R)total;
    } else {
        for (int k = b; k <= tnew - 1; ++k) dz[base_dz + k - 1] = (R)column_dz(g, MSL, h, eta, b, tnew, k);
        for (int k = b; k <= tnew - 1; ++k)
            dzh[base_dzh + k] =
                (R)((column_dz(g, MSL, h, eta, b, tnew, k + 1) + column_dz(g, MSL, h, eta, b, tnew, k)) * 0.5);
        if (KIND != 2) {
            dzh[base_dzh + tnew] = (R)column_dz(g, MSL, h, eta, b, tnew, tnew);
            dzh[base_dzh + b - 1] = (R)column_dz(g, MSL, h, eta, b, tnew, b);
        }
    }
    return tnew;
}

template <typename R> __global__ void k_layers_cells(Geom g, StateT<R> s, Params p, gom_status *st) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i > g.NC) return;
    const int L = g.L;
    bool bad;
    int b = g.bottom_cell[i - 1];
    int tnew = new_column<0>(g, p, g.h_cell[i - 1], s.eta_cell_new[i - 1], b, s.dz_cell_new, s.dzhalf_cell_new,
                             (long)(i - 1) * L, (long)(i - 1) * (L + 1), bad);
    if (bad) {
        record_error(st, GOM_E_LAYER, 66, i, tnew, s.eta_cell_new[i - 1], GOM_ENTITY_CELL);
        return;
    }
    if (s.top_cell[i - 1] == 0 && tnew != 0)
        for (int k = 0; k <= L; ++k) s.wn_cell_new[ix0(k, i, L)] = R(0);
    s.top_cell[i - 1] = tnew;
}

template <typename R> __global__ void k_layers_faces(Geom g, StateT<R> s, Params p, gom_status *st) {
    int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (j > g.NF) return;
    const int L = g.L;
    int a1 = g.face_cell(1, j), a2 = g.face_cell(2, j);
    double eta_max = a2 != 0 ? fmax(s.eta_cell_new[a1 - 1], s.eta_cell_new[a2 - 1]) : s.eta_cell_new[a1 - 1];
    bool bad;
    int b = g.bottom_face[j - 1];
    int tnew = new_column<1>(g, p, g.h_face[j - 1], eta_max, b, s.dz_face_new, s.dzhalf_face_new, (long)(j - 1) * L,
                             (long)(j - 1) * (L + 1), bad);
    if (bad) {
        record_error(st, GOM_E_LAYER, 166, j, tnew, eta_max, GOM_ENTITY_FACE);
        return;
    }
    s.top_face[j - 1] = tnew;
    for (int k = b; k <= tnew - 1; ++k) {
        double v = s.dzhalf_face_new[ix0(k, j, L)];
        if (v < p.denominator_min_for_matrix) {
            record_error(st, GOM_E_LAYER, 301, j, k, v, GOM_ENTITY_FACE);
            return;
        }
    }
}

template <typename R> __global__ void k_layers_nodes(Geom g, StateT<R> s, Params p, gom_status *st) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i > g.NN) return;
    const int L = g.L;
    bool bad;
    int b = g.bottom_node[i - 1];
    int tnew = new_column<2>(g, p, g.h_node[i - 1], s.eta_node[i - 1], b, s.dz_node_new, s.dzhalf_node_new,
                             (long)(i - 1) * L, (long)(i - 1) * (L + 1), bad);
    if (bad) {
        record_error(st, GOM_E_LAYER, 224, i, tnew, s.eta_node[i - 1], GOM_ENTITY_NODE);
        return;
    }
    s.top_node[i - 1] = tnew;
    for (int k = b; k <= tnew - 1; ++k) {
        double v = s.dzhalf_node_new[ix0(k, i, L)];
        if (v < p.denominator_min_for_matrix) {
            record_error(st, GOM_E_LAYER, 318, i, k, v, GOM_ENTITY_NODE);
            return;
        }
    }
}

// :260-296 an element is dry when all its nodes are dry; consistency checks
template <typename R> __global__ void k_layers_check(Geom g, StateT<R> s, Params p, gom_status *st) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i > g.NC) return;
    const int L = g.L;
    int nsum1 = 0, nsum2 = 0;
    int tq = g.tri_or_quad[i - 1];
    for (int l = 1; l <= tq; ++l) {
        nsum1 += s.top_node[g.cell_node(l, i) - 1];
        nsum2 += s.top_face[g.cell_face(l, i) - 1];
    }
    int t = s.top_cell[i - 1];
    if (nsum1 == 0) {
        t = 0;
        s.top_cell[i - 1] = 0;
    }
    if (nsum2 == 0 && t != 0) {
        record_error(st, GOM_E_DRY, 273, i, 0, 0.0, GOM_ENTITY_CELL);
        return;
    }
    for (int k = g.bottom_cell[i - 1]; k <= t - 1; ++k) {
        double v = s.dzhalf_cell_new[ix0(k, i, L)];
        if (v < p.denominator_min_for_matrix) {
            record_error(st, GOM_E_LAYER, 284, i, k, v, GOM_ENTITY_CELL);
            return;
        }
    }
}

template <typename R> cudaError_t launch_layers(const LaunchT<R> &x) {
    k_layers_cells<<<blocks_for(x.g.NC, 256), 256, 0, x.stream>>>(x.g, x.s, x.p, x.status);
    k_layers_faces<<<blocks_for(x.g.NF, 256), 256, 0, x.stream>>>(x.g, x.s, x.p, x.status);
    k_layers_nodes<<<blocks_for(x.g.NN, 256), 256, 0, x.stream>>>(x.g, x.s, x.p, x.status);
    k_layers_check<<<blocks_for(x.g.NC, 256), 256, 0, x.stream>>>(x.g, x.s, x.p, x.status);
    return cudaGetLastError();
}

// ============================================================================================
// Cold start on the device (setup_cold_start.f90: eta = 0, no motion; update_vertical_layers_0.f90:
// the first layers and thicknesses; uniform tracers), for contexts whose initial 3-D state is
// too large to build on the host.  update_vertical_layers_0.f90 gives the edge half-thicknesses
// to faces and nodes (:146-263), not to cells.
template <int KIND, typename R>
__global__ void k_cold_layers(Geom g, Params p, int n, const double *h, const int *bottom, int *top, R *dz, R *dzh,
                              gom_status *st) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const int L = g.L;
    const double msl = p.msl, eta = 0.0;
    const double he = h[e], total = he + eta;
    R *z = dz + (long)e * L;
    R *zh = dzh + (long)e * (L + 1);
    int t = 0;
    if (total > p.dry_depth) {
        const double tmp = msl + eta;
        for (int k = L - 1; k >= 0; --k) {
            if (tmp > g.z_level[k] && tmp <= g.z_level[k + 1]) {
                t = k + 1;
                z[t - 1] = (R)(tmp - g.z_level[k]);
                break;
            }
        }
        const int b = bottom[e];
        if (t < b) {
            record_error(st, GOM_E_LAYER, 66, e + 1, t, eta, GOM_ENTITY_CELL);
            return;
        }
        if (t == b) {
            z[t - 1] = (R)total;
            if (KIND == 1) zh[t - 1] = (R)total;
            zh[t] = (R)total;
        } else {
            for (int k = b; k <= t - 1; ++k) z[k - 1] = (R)column_dz(g, msl, he, eta, b, t, k);
            for (int k = b; k <= t - 1; ++k)
                zh[k] = (R)((column_dz(g, msl, he, eta, b, t, k + 1) + column_dz(g, msl, he, eta, b, t, k)) * 0.5);
            if (KIND != 0) {
                zh[t] = (R)column_dz(g, msl, he, eta, b, t, t);
                zh[b - 1] = (R)column_dz(g, msl, he, eta, b, t, b);
            }
        }
    }
    top[e] = t;
}

// :270-286 an element all of whose nodes are dry is dry; tracers, Av, Kv and ELM substeps
template <typename R>
__global__ void k_cold_cells(Geom g, StateT<R> s, Params p, R salt, R temp, R av0, R kv0, gom_status *st) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int L = g.L;
    if (i <= g.NC) {
        int n1 = 0, n2 = 0, tq = g.tri_or_quad[i - 1];
        for (int l = 1; l <= tq; ++l) {
            n1 += s.top_node[g.cell_node(l, i) - 1];
            n2 += s.top_face[g.cell_face(l, i) - 1];
        }
        if (n1 == 0) s.top_cell[i - 1] = 0;
        if (n2 == 0 && s.top_cell[i - 1] != 0) record_error(st, GOM_E_DRY, 273, i, 0, 0.0, GOM_ENTITY_CELL);
        for (int k = 1; k <= L; ++k) {
            long o = ix(k, i, L);
            s.salt_cell[o] = salt;
            s.salt_cell_new[o] = salt;
            s.temp_cell[o] = temp;
            s.temp_cell_new[o] = temp;
            s.kv[ix0(k, i, L)] = kv0;
        }
    }
    if (i <= g.NF) {
        for (int k = 1; k <= L; ++k) {
            long o = ix(k, i, L);
            s.salt_face[o] = salt;
            s.temp_face[o] = temp;
            s.av[ix0(k, i, L)] = av0;
        }
    }
    if (i <= g.NN) {
        int nsub = p.elm_backtrace_flag == 0 ? p.elm_sub_iter : p.elm_backtrace_flag == 1 ? 1 : 0;
        for (int k = 1; k <= L; ++k) {
            long o = ix(k, i, L);
            s.salt_node[o] = salt;
            s.temp_node[o] = temp;
            s.num_sub_elm[o] = nsub;
        }
    }
}

template <typename R>
cudaError_t launch_cold_start(const LaunchT<R> &x, double salt, double temp, double av0, double kv0) {
    const Geom &g = x.g;
    k_cold_layers<0, R><<<blocks_for(g.NC, 256), 256, 0, x.stream>>>(g, x.p, g.NC, g.h_cell, g.bottom_cell,
                                                                       x.s.top_cell, x.s.dz_cell, x.s.dzhalf_cell, x.status);
    k_cold_layers<1, R><<<blocks_for(g.NF, 256), 256, 0, x.stream>>>(g, x.p, g.NF, g.h_face, g.bottom_face,
                                                                       x.s.top_face, x.s.dz_face, x.s.dzhalf_face, x.status);
    k_cold_layers<2, R><<<blocks_for(g.NN, 256), 256, 0, x.stream>>>(g, x.p, g.NN, g.h_node, g.bottom_node,
                                                                       x.s.top_node, x.s.dz_node, x.s.dzhalf_node, x.status);
    int n = std::max(g.NC, std::max(g.NF, g.NN));
    k_cold_cells<R><<<blocks_for(n, 256), 256, 0, x.stream>>>(g, x.s, x.p, (R)salt, (R)temp, (R)av0, (R)kv0,
                                                                 x.status);
    return cudaGetLastError();
}

template cudaError_t launch_cold_start<double>(const LaunchT<double> &, double, double, double, double);
template cudaError_t launch_cold_start<float>(const LaunchT<float> &, double, double, double, double);

// ============================================================================================
// calculate_velocity_at_node.f90:31-60: face-level velocities, one thread per face column.  The
// node loop divides each face level by the face length; that quotient is formed once here.
template <typename R> __global__ void k_face_level(Geom g, StateT<R> s, WorkT<R> w) {
    unsigned tid = flat_tid();
    if (tid >= (unsigned)g.NF) return;
    int j = g.face_order[tid];
    const int L = g.L;
    int t = s.top_face[j - 1];
    if (t == 0) return;
    int b = g.bottom_face[j - 1];
    const R ct = (R)g.cos_theta[j - 1], sn = (R)g.sin_theta[j - 1], fl = (R)g.face_length[j - 1];
    R uk, vk;
    {
        R un = s.un_face_new[ix(b, j, L)], vn = s.vn_face_new[ix(b, j, L)];
        uk = un * ct - vn * sn;
        vk = un * sn + vn * ct;
    }
    long o = ix0(b - 1, j, L);
    s.u_face_level[o] = uk;
    s.v_face_level[o] = vk;
    w.uflf[o] = uk / fl;
    w.vflf[o] = vk / fl;
    for (int k = b; k <= t - 1; ++k) {
        R un = s.un_face_new[ix(k + 1, j, L)], vn = s.vn_face_new[ix(k + 1, j, L)];
        R u1 = un * ct - vn * sn;
        R v1 = un * sn + vn * ct;
        R fac = s.dz_face[ix(k, j, L)] * R(0.5) / s.dzhalf_face[ix0(k, j, L)];
        R ul = uk + fac * (u1 - uk), vl = vk + fac * (v1 - vk);
        o = ix0(k, j, L);
        s.u_face_level[o] = ul;
        s.v_face_level[o] = vl;
        w.uflf[o] = ul / fl;
        w.vflf[o] = vl / fl;
        uk = u1;
        vk = v1;
    }
    o = ix0(t, j, L);
    s.u_face_level[o] = uk;
    s.v_face_level[o] = vk;
    w.uflf[o] = uk / fl;
    w.vflf[o] = vk / fl;
}

// FP32 path: one thread per (face, level)
__global__ void k_face_level_flat(Geom g, StateT<float> s, WorkT<float> w) {
    unsigned tt = flat_tid();
    const int L = g.L;
    if (tt >= (unsigned)g.NF * (L + 1)) return;
    int j, k;
    split_index(tt, L + 1, j, k);   // k = level 0..L
    j += 1;
    const int t = s.top_face[j - 1], b = g.bottom_face[j - 1];
    if (t == 0 || k < b - 1 || k > t) return;
    const float ct = g.cos_theta_f[j - 1], sn = g.sin_theta_f[j - 1], fl = g.face_length_f[j - 1];
    // the face velocity of layer m rotated to x/y
    auto rot = [&](int m, float &u, float &v) {
        float un = s.un_face_new[ix(m, j, L)], vn = s.vn_face_new[ix(m, j, L)];
        u = un * ct - vn * sn;
        v = un * sn + vn * ct;
    };
    float ul, vl;
    if (k == b - 1) {
        rot(b, ul, vl);
    } else if (k == t) {
        rot(t, ul, vl);
    } else {
        float uk, vk, u1, v1;
        rot(k, uk, vk);
        rot(k + 1, u1, v1);
        float fac = s.dz_face[ix(k, j, L)] * 0.5f / s.dzhalf_face[ix0(k, j, L)];
        ul = uk + fac * (u1 - uk);
        vl = vk + fac * (v1 - vk);
    }
    const long o = ix0(k, j, L);
    s.u_face_level[o] = ul;
    s.v_face_level[o] = vl;
    w.uflf[o] = ul / fl;
    w.vflf[o] = vl / fl;
}

// :103 the weight sums factor_weight/face_length over the node's faces whatever their wetness:
// a static per-node value, accumulated once in the reference's order
__global__ void k_node_weight(Geom g, double *node_weight) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i > g.NN) return;
    double weight = 0.0;
    int na = g.adj_cells_at_node[i - 1];
    for (int j = 1; j <= na; ++j) {
        int isn = g.node_cell(j, i), nc = g.node_count(j, i);
        int tq = g.tri_or_quad[isn - 1];
        for (int l = tq - 2; l <= tq - 1; ++l) {
            int ifn = g.cell_face(start_end_node(tq, nc, l), isn);
            double fw = g.face_cell(2, ifn) == 0 ? 2.0 : 1.0;
            weight = weight + fw / g.face_length[ifn - 1];
        }
    }
    node_weight[i - 1] = weight;
}

// the levels of node i (0-based) that a face or a cell of the node reaches, as list layers
// (level + 1): from min(bottom - 1) over the faces and cells k_node_uvw visits, to L
struct NodeLevelRange {
    Geom g;
    __device__ int2 operator()(int i0) const {
        const int i = i0 + 1;
        int lo = g.L + 1;
        const int na = g.adj_cells_at_node[i - 1];
        for (int j = 1; j <= na; ++j) {
            const int isn = g.node_cell(j, i), nc = g.node_count(j, i);
            const int tq = g.tri_or_quad[isn - 1];
            for (int l = tq - 2; l <= tq - 1; ++l)
                lo = min(lo, g.bottom_face[g.cell_face(start_end_node(tq, nc, l), isn) - 1] - 1);
            lo = min(lo, g.bottom_cell[isn - 1] - 1);
        }
        return make_int2(max(lo, 0) + 1, g.L + 1);
    }
};

template <typename R> cudaError_t launch_node_weights(const LaunchT<R> &x) {
    k_node_weight<<<blocks_for(x.g.NN, 256), 256, 0, x.stream>>>(x.g, x.w.node_weight);
    if (x.w.nl_list)
        return build_layer_list(x.g.NN, NodeLevelRange{x.g}, x.w.nl_off, x.w.nl_bsum, x.w.nl_list, x.w.nl_count,
                                x.stream);
    return cudaGetLastError();
}

// :67-138 node u, v (face-length weighted face levels) and w (area-weighted cell w) at one
// (node, level)
template <typename R> __device__ __forceinline__ void node_uvw_at(const Geom &g, const StateT<R> &s,
                                                                  const WorkT<R> &wk, int i, int k) {
    const int L = g.L;
    R u = R(0), v = R(0);
    int icount = 0;
    int na = g.adj_cells_at_node[i - 1];
    for (int j = 1; j <= na; ++j) {
        int isn = g.node_cell(j, i), nc = g.node_count(j, i);
        int tq = g.tri_or_quad[isn - 1];
        for (int l = tq - 2; l <= tq - 1; ++l) {
            int ifn = g.cell_face(start_end_node(tq, nc, l), isn);
            int tf = s.top_face[ifn - 1];
            if (tf != 0 && k >= g.bottom_face[ifn - 1] - 1) {
                R fw = g.face_cell(2, ifn) == 0 ? R(2) : R(1);
                long o = ix0(min(k, tf), ifn, L);
                u = u + wk.uflf[o] * fw;
                v = v + wk.vflf[o] * fw;
                icount = icount + 1;
            }
        }
    }
    if (icount != 0) {
        R weight = geo<R>(wk.node_weight, g.node_weight_f, i - 1);
        u = u / weight;
        v = v / weight;
    }
    R w = R(0), tw = R(0);
    for (int j = 1; j <= na; ++j) {
        int ite = g.node_cell(j, i);
        int te = s.top_cell[ite - 1];
        if (te != 0 && k >= g.bottom_cell[ite - 1] - 1) {
            int kvt = min(k, te);
            R ar = geo<R>(g.area, g.area_f, ite - 1);
            tw = tw + ar;
            w = w + s.wn_cell[ix0(kvt, ite, L)] * ar;
        }
    }
    if (tw != R(0)) w = w / tw;
    long o = ix0(k, i, L);
    s.u_node[o] = u;
    s.v_node[o] = v;
    s.w_node[o] = w;
}

// one thread per (node, level)
template <typename R> __global__ void k_node_uvw(Geom g, StateT<R> s, WorkT<R> wk) {
    unsigned tt = flat_tid();
    if (tt >= (unsigned)g.NN * (g.L + 1)) return;
    int i, k;
    split_index(tt, g.L + 1, i, k);
    node_uvw_at(g, s, wk, i + 1, k);
}

// FP64: one thread per listed (node, level); the levels below every face and cell of a node are
// 0 (no face or cell contributes there), written by a fill first.  GB300 issues an FP64 warp
// instruction at the same cost however few lanes are active, and a node's low levels would leave
// most lanes of its warps idle.
template <typename R> __global__ void __launch_bounds__(256) k_node_uvw_list(Geom g, StateT<R> s, WorkT<R> wk) {
    const int n = *wk.nl_count;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int code = wk.nl_list[t];
        node_uvw_at(g, s, wk, list_entity(code), list_layer(code) - 1);
    }
}

// FP32 path, the same per node by tiles: a block takes NV_TILE consecutive nodes and lists each
// node's faces (with weight and level range) and cells once in shared memory, in the order the
// per-(node, level) kernel visits them; every (node, level) slot then sums from the lists.  Same
// values as k_node_uvw<float>.
constexpr int NV_TILE = 32;

__global__ void __launch_bounds__(256) k_node_uvw_tile(Geom g, StateT<float> s, WorkT<float> wk) {
    __shared__ int fid[NV_TILE][2 * GOM_MAXNB], flo[NV_TILE][2 * GOM_MAXNB], fhi[NV_TILE][2 * GOM_MAXNB];
    __shared__ float fwt[NV_TILE][2 * GOM_MAXNB];
    __shared__ int cid[NV_TILE][GOM_MAXNB], clo[NV_TILE][GOM_MAXNB], chi[NV_TILE][GOM_MAXNB];
    __shared__ float car[NV_TILE][GOM_MAXNB];
    __shared__ int nf_s[NV_TILE], nc_s[NV_TILE];
    __shared__ float wgt_s[NV_TILE];
    const int L = g.L;
    const int i0 = blockIdx.x * NV_TILE;
    const int nn = min(NV_TILE, g.NN - i0);
    for (int c = threadIdx.x; c < nn; c += blockDim.x) {
        const int i = i0 + c + 1;
        const int na = g.adj_cells_at_node[i - 1];
        int nf = 0, nc = 0;
        for (int j = 1; j <= na; ++j) {
            const int isn = g.node_cell(j, i), ncnt = g.node_count(j, i);
            const int tq = g.tri_or_quad[isn - 1];
            for (int l = tq - 2; l <= tq - 1; ++l) {
                const int ifn = g.cell_face(start_end_node(tq, ncnt, l), isn);
                const int tf = s.top_face[ifn - 1];
                if (tf == 0) continue;   // contributes nothing at any level
                fid[c][nf] = ifn;
                flo[c][nf] = g.bottom_face[ifn - 1] - 1;
                fhi[c][nf] = tf;
                fwt[c][nf] = g.face_cell(2, ifn) == 0 ? 2.0f : 1.0f;
                ++nf;
            }
            const int te = s.top_cell[isn - 1];
            if (te != 0) {
                cid[c][nc] = isn;
                clo[c][nc] = g.bottom_cell[isn - 1] - 1;
                chi[c][nc] = te;
                car[c][nc] = g.area_f[isn - 1];
                ++nc;
            }
        }
        nf_s[c] = nf;
        nc_s[c] = nc;
        wgt_s[c] = g.node_weight_f[i - 1];
    }
    __syncthreads();
    const long base = (long)i0 * (L + 1);
    for (int t = threadIdx.x; t < nn * (L + 1); t += blockDim.x) {
        const int c = t / (L + 1), k = t - c * (L + 1);
        float u = 0.0f, v = 0.0f;
        int icount = 0;
        for (int q = 0; q < nf_s[c]; ++q) {
            if (k >= flo[c][q]) {
                const long o = ix0(min(k, fhi[c][q]), fid[c][q], L);
                u = u + wk.uflf[o] * fwt[c][q];
                v = v + wk.vflf[o] * fwt[c][q];
                icount = icount + 1;
            }
        }
        if (icount != 0) {
            u = u / wgt_s[c];
            v = v / wgt_s[c];
        }
        float w = 0.0f, tw = 0.0f;
        for (int q = 0; q < nc_s[c]; ++q) {
            if (k >= clo[c][q]) {
                const float ar = car[c][q];
                tw = tw + ar;
                w = w + s.wn_cell[ix0(min(k, chi[c][q]), cid[c][q], L)] * ar;
            }
        }
        if (tw != 0.0f) w = w / tw;
        s.u_node[base + t] = u;
        s.v_node[base + t] = v;
        s.w_node[base + t] = w;
    }
}

template <typename R> cudaError_t launch_node_velocity(const LaunchT<R> &x) {
    if constexpr (sizeof(R) == sizeof(float))
        k_face_level_flat<<<blocks_for((long)x.g.NF * (x.g.L + 1), 256), 256, 0, x.stream>>>(x.g, x.s, x.w);
    else
        k_face_level<<<blocks_for(x.g.NF, 128), 128, 0, x.stream>>>(x.g, x.s, x.w);
    if constexpr (sizeof(R) == sizeof(float)) {
        k_node_uvw_tile<<<blocks_for(x.g.NN, NV_TILE), 256, 0, x.stream>>>(x.g, x.s, x.w);
    } else if (x.w.nl_list) {
        const size_t bytes = (size_t)x.g.NN * (x.g.L + 1) * sizeof(R);
        cudaError_t e = cudaMemsetAsync(x.s.u_node, 0, bytes, x.stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(x.s.v_node, 0, bytes, x.stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(x.s.w_node, 0, bytes, x.stream);
        if (e != cudaSuccess) return e;
        k_node_uvw_list<<<x.num_sms * 8, 256, 0, x.stream>>>(x.g, x.s, x.w);
    } else {
        long n = (long)x.g.NN * (x.g.L + 1);
        k_node_uvw<<<blocks_for(n, 256), 256, 0, x.stream>>>(x.g, x.s, x.w);
    }
    return cudaGetLastError();
}

template cudaError_t pcg_configure<double>(LaunchT<double> &x, int device);
template cudaError_t pcg_configure<float>(LaunchT<float> &x, int device);
GOM_INSTANTIATE_LAUNCH(launch_free_surface)
GOM_INSTANTIATE_LAUNCH(launch_velocities)
GOM_INSTANTIATE_LAUNCH(launch_layers)
GOM_INSTANTIATE_LAUNCH(launch_node_velocity)
GOM_INSTANTIATE_LAUNCH(launch_node_weights)

}  // namespace gom
