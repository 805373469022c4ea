// k_geometry.cu -- GOM's start-up mesh geometry built on the GPU (gom_geometry_build).
//
// The reference builds it serially at start-up: cell areas in read_cell_inp.f90:54-87,
// set_geometry_1.f90 (node-cell and node-node adjacency, cell-cell adjacency, face numbering,
// face and cell centres, sign_in_outflow, delta_j, face angles), calculate_voronoi_center.f90 and
// set_geometry_2.f90 (boundary cells and faces, bottom layers).  Its results are fixed by the
// order of its loops; here every output is a function of the mesh alone, computed by one thread
// per cell, node, face or boundary pair, so the order-dependent pieces are reproduced as:
//   * node-cell lists: slots claimed with atomics, then each node's list sorted by (cell, local
//     node) -- the reference's traversal order;
//   * node-node lists: one thread per node walks its sorted cell list exactly as the reference;
//   * face numbers: an exclusive scan over the per-cell count of faces the cell owns (a boundary
//     edge or a neighbour with a larger index), cells ascending and local edges ascending;
//   * boundary flags: the largest boundary index wins where two boundaries share a cell or face,
//     as the reference's sequential loop leaves it.
// Doubles use the reference's expressions and order of operations (built with -fmad=false), so
// they equal a serial run bit for bit, except the face angles (CUDA's atan2 / cos / sin).
//
// Failures: the reference stops at its first failing check.  Each check here records a 64-bit
// key (stage, position in the reference's traversal, site) with atomicMin, so the smallest key is
// the check the reference would stop at.  The host reads it after each stage whose failure would
// leave later stages without valid indices, and stops there.
#include <cstdint>
#include <cstring>
#include <vector>

#include "gom_device.cuh"

namespace {

using u64 = unsigned long long;
constexpr u64 kNoFailure = ~0ull;
constexpr int kThreads = 256;

// failure key: stage (8 bits) | position (40 bits) | site (8 bits)
__device__ __forceinline__ void fail(u64 *key, int stage, u64 pos, int site) {
    atomicMin(key, ((u64)stage << 56) | (pos << 8) | (u64)site);
}

inline int blocks(long n) { return (int)((n + kThreads - 1) / kThreads); }

struct Mesh {
    int NN, NC, NB, L, NOB, NQB, voronoi;
    double msl;
    const double *x, *y, *h, *z_level;
    const int *tq, *cells;        // cells: (NC, 4) 1-based
    const int *ob_nodes, *qb_nodes;
};

__device__ __forceinline__ int cnode(const Mesh &m, int l, int i) { return m.cells[(i - 1) * 4 + l - 1]; }

// start_end_node(k, l, which) of set_geometry_1.f90:78-93: side l of a k-gon runs from local
// node l + 1 to l + 2 (which = 1, 2), wrapping past k
__device__ __forceinline__ int edge_end(int k, int l, int which) {
    int v = l + which;
    return v > k ? v - k : v;
}

__device__ __forceinline__ double cell_area(double x1, double x2, double x3, double y1, double y2, double y3) {
    return fabs((x1 - x3) * (y2 - y3) - (x2 - x3) * (y1 - y3)) * 0.5;   // mod_function_library.f90:49-60
}

// read_cell_inp.f90:54-87
__global__ void k_area(Mesh m, double *area, u64 *fk) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i > m.NC) return;
    const int n1 = cnode(m, 1, i), n2 = cnode(m, 2, i), n3 = cnode(m, 3, i);
    const double *x = m.x - 1, *y = m.y - 1;
    double a;
    if (m.tq[i - 1] == 3) {
        a = cell_area(x[n1], x[n2], x[n3], y[n1], y[n2], y[n3]);
    } else {
        const int n4 = cnode(m, 4, i);
        const double t1 = cell_area(x[n1], x[n2], x[n3], y[n1], y[n2], y[n3]);
        const double t2 = cell_area(x[n1], x[n3], x[n4], y[n1], y[n3], y[n4]);
        const double t3 = cell_area(x[n1], x[n2], x[n4], y[n1], y[n2], y[n4]);
        const double t4 = cell_area(x[n2], x[n3], x[n4], y[n2], y[n3], y[n4]);
        if (t1 <= 0.0 || t2 <= 0.0 || t3 <= 0.0 || t4 <= 0.0) {
            fail(fk, 1, (u64)i, GOM_GEO_CONCAVE);
            area[i - 1] = 0.0;
            return;
        }
        a = t1 + t2;
    }
    area[i - 1] = a;
    if (a <= 0.0) fail(fk, 1, (u64)i, GOM_GEO_AREA);
}

// set_geometry_1.f90:109-128: claim a slot of each node's list; keys (cell, local node) sorted later
__global__ void k_node_claim(Mesh m, int *count, int *slots, u64 *fk) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 4L * m.NC) return;
    const int i = (int)(t >> 2) + 1, l = (int)(t & 3) + 1;
    if (l > m.tq[i - 1]) return;
    const int nd = cnode(m, l, i);
    const int s = atomicAdd(&count[nd - 1], 1);
    if (s < m.NB) slots[(long)(nd - 1) * m.NB + s] = ((i - 1) << 2) | (l - 1);
    else fail(fk, 2, (u64)nd, GOM_GEO_MAX_NB);
}

// set_geometry_1.f90:109-135: each node's list in (cell, local node) order; hanging nodes
__global__ void k_node_sort(Mesh m, const int *count, const int *slots, int *acn, int *ncee, u64 *fk) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= m.NN) return;
    const int c = count[n];
    if (c == 0) {
        fail(fk, 3, (u64)(n + 1), GOM_GEO_HANGING);
        return;
    }
    if (c > m.NB) return;
    int key[GOM_MAXNB];
    for (int q = 0; q < c; ++q) {
        const int v = slots[(long)n * m.NB + q];
        int p = q;
        while (p > 0 && key[p - 1] > v) {
            key[p] = key[p - 1];
            --p;
        }
        key[p] = v;
    }
    for (int q = 0; q < m.NB; ++q) {
        acn[(long)n * m.NB + q] = q < c ? (key[q] >> 2) + 1 : 0;
        ncee[(long)n * m.NB + q] = q < c ? (key[q] & 3) + 1 : 0;
    }
}

// set_geometry_1.f90:160-184, one thread per node, in the reference's discovery order
__global__ void k_node_nodes(Mesh m, const int *count, const int *acn, int *an, int *ann, u64 *fk) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i > m.NN) return;
    int *row = ann + (long)(i - 1) * (m.NB + 1);   // index 0 unused (0:max_nb)
    for (int q = 0; q <= m.NB; ++q) row[q] = 0;
    int k_count = 0;
    for (int j = 1; j <= count[i - 1]; ++j) {
        const int ie = acn[(long)(i - 1) * m.NB + j - 1];
        for (int k = 1; k <= m.tq[ie - 1]; ++k) {
            const int nd = cnode(m, k, ie);
            // the test of nd == i sits inside the loop over the list, so while the list is
            // empty the node itself is taken (the first node of its first cell): kept as it is
            bool skip = false;
            for (int l = 1; l <= k_count && !skip; ++l) skip = nd == i || nd == row[l];
            if (skip) continue;
            k_count = k_count + 1;
            if (k_count > m.NB) {
                fail(fk, 4, (u64)i, GOM_GEO_SURROUNDING);
                an[i - 1] = m.NB;
                return;
            }
            row[k_count] = nd;
        }
    }
    an[i - 1] = k_count;
}

// set_geometry_1.f90:206-225 (the last cell around nd1 other than i that holds nd2) and the
// number of faces each cell owns (set_geometry_1.f90:241-252)
__global__ void k_cell_adj(Mesh m, const int *count, const int *acn, int *acc, int *owned) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i > m.NC) return;
    const int k = m.tq[i - 1];
    int own = 0;
    for (int l = 1; l <= 4; ++l) {
        int nb = 0;
        if (l <= k) {
            const int nd1 = cnode(m, edge_end(k, l, 1), i), nd2 = cnode(m, edge_end(k, l, 2), i);
            for (int q = 1; q <= count[nd1 - 1]; ++q) {
                const int c = acn[(long)(nd1 - 1) * m.NB + q - 1];
                if (c != i && (cnode(m, 1, c) == nd2 || cnode(m, 2, c) == nd2 || cnode(m, 3, c) == nd2 ||
                               (m.tq[c - 1] == 4 && cnode(m, 4, c) == nd2)))
                    nb = c;
            }
            if (nb == 0 || i < nb) ++own;
        }
        acc[(i - 1) * 4 + l - 1] = nb;
    }
    owned[i - 1] = own;
}

// ---------------------------------------------------------------- exclusive scan of owned faces
constexpr int kScanThreads = 1024, kScanItems = 4, kScanTile = kScanThreads * kScanItems;

__device__ int block_exclusive_scan(int v, int *warp_sums, int &total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_sums[lane] = w;   // inclusive over warps
    }
    __syncthreads();
    total = warp_sums[(blockDim.x >> 5) - 1];
    const int before = warp > 0 ? warp_sums[warp - 1] : 0;
    __syncthreads();
    return before + x - v;
}

// per tile: exclusive offsets within the tile, and the tile's sum
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const int *in, int n, int *out, int *tile_sum) {
    __shared__ int ws[32];
    const long base = (long)blockIdx.x * kScanTile + (long)threadIdx.x * kScanItems;
    int v[kScanItems], s = 0;
    for (int q = 0; q < kScanItems; ++q) {
        v[q] = base + q < n ? in[base + q] : 0;
        s += v[q];
    }
    int total;
    int run = block_exclusive_scan(s, ws, total);
    for (int q = 0; q < kScanItems; ++q) {
        if (base + q < n) out[base + q] = run;
        run += v[q];
    }
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

// one block: exclusive offsets of the tile sums (serial chunks per thread), and the grand total
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(int *tile_sum, int tiles, int *grand) {
    __shared__ int ws[32];
    const int per = (tiles + kScanThreads - 1) / kScanThreads;
    const int lo = threadIdx.x * per, hi = min(tiles, lo + per);
    int s = 0;
    for (int q = lo; q < hi; ++q) s += tile_sum[q];
    int total;
    int run = block_exclusive_scan(s, ws, total);
    for (int q = lo; q < hi; ++q) {
        const int v = tile_sum[q];
        tile_sum[q] = run;
        run += v;
    }
    if (threadIdx.x == 0) *grand = total;
}

__global__ void k_scan_add(int *out, int n, const int *tile_off) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] += tile_off[t / kScanTile];
}

// set_geometry_1.f90:296-345: the faces a cell owns, numbered after the faces of lower cells
__global__ void k_faces(Mesh m, const int *acc, const int *first, int *fac, int *acf, int *nof, double *x_face,
                        double *y_face, double *h_face, double *face_length, u64 *fk) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i > m.NC) return;
    const int k = m.tq[i - 1];
    int j = first[i - 1];
    for (int l = 1; l <= k; ++l) {
        const int nb = acc[(i - 1) * 4 + l - 1];
        if (!(nb == 0 || i < nb)) continue;
        j = j + 1;
        const int nd1 = cnode(m, edge_end(k, l, 1), i), nd2 = cnode(m, edge_end(k, l, 2), i);
        fac[(i - 1) * 4 + l - 1] = j;
        acf[(j - 1) * 2] = i;
        acf[(j - 1) * 2 + 1] = nb;
        nof[(j - 1) * 2] = nd1;
        nof[(j - 1) * 2 + 1] = nd2;
        const double xn1 = m.x[nd1 - 1], yn1 = m.y[nd1 - 1], xn2 = m.x[nd2 - 1], yn2 = m.y[nd2 - 1];
        x_face[j - 1] = (xn1 + xn2) * 0.5;
        y_face[j - 1] = (yn1 + yn2) * 0.5;
        h_face[j - 1] = (m.h[nd1 - 1] + m.h[nd2 - 1]) * 0.5;
        const double fl = sqrt((xn2 - xn1) * (xn2 - xn1) + (yn2 - yn1) * (yn2 - yn1));
        face_length[j - 1] = fl;
        if (fl == 0) fail(fk, 5, (u64)j << 1, GOM_GEO_FACE_LENGTH);
        if (nb != 0) {
            int index1 = 0;
            for (int l2 = 1; l2 <= m.tq[nb - 1]; ++l2)
                if (acc[(nb - 1) * 4 + l2 - 1] == i) {
                    index1 = l2;
                    break;
                }
            if (index1 == 0) fail(fk, 5, ((u64)j << 1) | 1, GOM_GEO_BALL);
            else fac[(nb - 1) * 4 + index1 - 1] = j;
        }
    }
}

// every side of every cell has a face number (a cell that shares two sides with one neighbour
// leaves the second without one; the reference would read outside its arrays there)
__global__ void k_check_fac(Mesh m, const int *fac, long fmax, u64 *fk) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i > m.NC) return;
    for (int l = 1; l <= m.tq[i - 1]; ++l)
        if (fac[(i - 1) * 4 + l - 1] <= 0) fail(fk, 5, ((u64)(fmax + i) << 1) | 1, GOM_GEO_BALL);
}

// set_geometry_1.f90:375-411 and calculate_voronoi_center.f90:36-98
__global__ void k_cells(Mesh m, const int *fac, const int *acf, const double *h_face, int *sign_io, double *x_cell,
                        double *y_cell, double *h_cell, u64 *fk) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i > m.NC) return;
    const int k = m.tq[i - 1];
    double x_sum = 0.0, y_sum = 0.0, hc = 0.0;
    for (int l = 1; l <= 4; ++l) {
        int s = 0;
        if (l <= k) {
            const int jsj = fac[(i - 1) * 4 + l - 1];
            const int a1 = acf[(jsj - 1) * 2], a2 = acf[(jsj - 1) * 2 + 1];
            s = (a2 - 2 * i + a1) / (a2 - a1);   // truncation toward zero, as Fortran
            x_sum = x_sum + m.x[cnode(m, l, i) - 1];
            y_sum = y_sum + m.y[cnode(m, l, i) - 1];
            if (h_face[jsj - 1] > hc) hc = h_face[jsj - 1];
        }
        sign_io[(i - 1) * 4 + l - 1] = s;
    }
    h_cell[i - 1] = hc;
    double xc = x_sum / k, yc = y_sum / k;
    if (m.voronoi == 1) {
        if (k == 3) {
            const double xi = m.x[cnode(m, 1, i) - 1], yi = m.y[cnode(m, 1, i) - 1];
            const double xj = m.x[cnode(m, 2, i) - 1], yj = m.y[cnode(m, 2, i) - 1];
            const double xk = m.x[cnode(m, 3, i) - 1], yk = m.y[cnode(m, 3, i) - 1];
            const double xij = 0.5 * (xi + xj), yij = 0.5 * (yi + yj);
            const double xjk = 0.5 * (xj + xk), yjk = 0.5 * (yj + yk);
            const double numerator = (xij - xjk) * (xj - xi) + (yij - yjk) * (yj - yi);
            const double denominator = (xj - xi) * (yk - yj) - (xk - xj) * (yj - yi);
            if (denominator != 0.0) {
                xc = xjk + numerator / denominator * (yk - yj);
                yc = yjk - numerator / denominator * (xk - xj);
            } else {
                fail(fk, 6, (u64)i, GOM_GEO_VORONOI);
            }
        } else {
            double tx = 0.0, ty = 0.0;
            for (int l = 1; l <= 4; ++l) {
                tx = tx + m.x[cnode(m, l, i) - 1];
                ty = ty + m.y[cnode(m, l, i) - 1];
            }
            xc = tx / 4.0;
            yc = ty / 4.0;
        }
    }
    x_cell[i - 1] = xc;
    y_cell[i - 1] = yc;
}

// set_geometry_1.f90:446-515, calculate_voronoi_center.f90:113-208
__global__ void k_faces2(Mesh m, int NF, const int *acf, const int *nof, const double *x_cell, const double *y_cell,
                         const double *x_face, const double *y_face, double *delta_j, double *cos_t, double *sin_t,
                         double *cos_t2, double *sin_t2, u64 *fk) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (j > NF) return;
    const int a1 = acf[(j - 1) * 2], a2 = acf[(j - 1) * 2 + 1];
    double d;
    if (a2 != 0) {
        const double dx = x_cell[a2 - 1] - x_cell[a1 - 1], dy = y_cell[a2 - 1] - y_cell[a1 - 1];
        d = sqrt(dx * dx + dy * dy);
        if (d == 0.0) fail(fk, 7, (u64)j, GOM_GEO_CENTRES);
    } else {
        const double dx = x_cell[a1 - 1] - x_face[j - 1], dy = y_cell[a1 - 1] - y_face[j - 1];
        d = sqrt(dx * dx + dy * dy) * 2.0;
    }
    delta_j[j - 1] = d;
    const int nd1 = nof[(j - 1) * 2], nd2 = nof[(j - 1) * 2 + 1];
    const double t0 = atan2(m.x[nd1 - 1] - m.x[nd2 - 1], m.y[nd2 - 1] - m.y[nd1 - 1]);
    cos_t[j - 1] = cos(t0);
    sin_t[j - 1] = sin(t0);
    double t1 = t0;
    if (a2 != 0) t1 = atan2(y_cell[a2 - 1] - y_cell[a1 - 1], x_cell[a2 - 1] - x_cell[a1 - 1]);
    const double t2 = (t1 - t0);
    cos_t2[j - 1] = cos(t2);
    sin_t2[j - 1] = sin(t2);
}

// find_element_and_face.f90:9-67 for the boundary pairs: the lowest cell holding n1 then n2 as
// consecutive CCW nodes (it holds n1, so it is in n1's sorted list), and the lowest face stored
// as (n1, n2) (a face holding n1 belongs to a cell around n1)
__global__ void k_boundary_find(Mesh m, const int *count, const int *acn, const int *fac, const int *nof,
                                int *ob_cell, int *ob_face, int *q_cell, int *q_face, u64 *fk) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m.NOB + m.NQB) return;
    const bool ob = t < m.NOB;
    const int *pair = ob ? m.ob_nodes + 2 * t : m.qb_nodes + 2 * (t - m.NOB);
    const int n1 = pair[0], n2 = pair[1];
    int element_id = 0, face_id = 0;
    for (int q = 1; q <= count[n1 - 1]; ++q) {
        const int c = acn[(long)(n1 - 1) * m.NB + q - 1];
        for (int l = 1; l <= 4; ++l) {
            const int f = l <= m.tq[c - 1] ? fac[(c - 1) * 4 + l - 1] : 0;
            if (f > 0 && nof[(f - 1) * 2] == n1 && nof[(f - 1) * 2 + 1] == n2 && (face_id == 0 || f < face_id))
                face_id = f;
        }
        if (element_id != 0) continue;
        for (int j1 = 1; j1 <= 4; ++j1) {
            const int nod1 = cnode(m, j1, c);
            int nod2 = cnode(m, j1 < 4 ? j1 + 1 : 1, c);
            if (nod2 == 0) nod2 = cnode(m, 1, c);
            if (nod1 == n1 && nod2 == n2) {
                element_id = c;
                break;
            }
        }
    }
    if (ob) {
        ob_cell[t] = element_id;
        ob_face[t] = face_id;
    } else {
        q_cell[t - m.NOB] = element_id;
        q_face[t - m.NOB] = face_id;
    }
    if (element_id == 0 || face_id == 0) fail(fk, 8, (u64)(t + 1), GOM_GEO_BOUNDARY);
}

// set_geometry_2.f90:48-53 and read_main_inp.f90:827-828: the later boundary wins a shared cell
// or face
__global__ void k_boundary_flags(Mesh m, const int *ob_cell, const int *ob_face, const int *q_cell,
                                 const int *q_face, int *ob_flag, int *btype, int *q_flag, int *isflow) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < m.NOB) {
        atomicMax(&ob_flag[ob_cell[t] - 1], t + 1);
        atomicMax(&btype[ob_face[t] - 1], t + 1);
    } else if (t < m.NOB + m.NQB) {
        const int i = t - m.NOB;
        atomicMax(&isflow[q_face[i] - 1], i + 1);
        atomicMax(&q_flag[q_cell[i] - 1], i + 1);
    }
}

// set_geometry_2.f90:54-58 and :101-189
__device__ __forceinline__ int bottom_layer(const Mesh &m, double h) {
    for (int k = 0; k <= m.L - 1; ++k)
        if ((m.msl - h) >= m.z_level[k] && (m.msl - h) < m.z_level[k + 1]) return k + 1;
    return 0;
}

__global__ void k_layers(Mesh m, int NF, const int *acf, const double *h_cell, const double *h_face, int *btype,
                         int *b_cell, int *b_face, int *b_node, int *wetdry, u64 *fk) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < m.NC) {
        if ((b_cell[t] = bottom_layer(m, h_cell[t])) == 0) fail(fk, 9, (u64)(t + 1), GOM_GEO_VERTICAL);
    }
    if (t < NF) {
        if (acf[t * 2 + 1] == 0 && btype[t] == 0) btype[t] = -1;
        if ((b_face[t] = bottom_layer(m, h_face[t])) == 0) fail(fk, 9, (1ull << 32) | (u64)(t + 1), GOM_GEO_VERTICAL);
    }
    if (t < m.NN) {
        if ((b_node[t] = bottom_layer(m, m.h[t])) == 0) fail(fk, 9, (2ull << 32) | (u64)(t + 1), GOM_GEO_VERTICAL);
        wetdry[t] = m.h[t] <= 0.0 ? 1 : 0;   // read_node_inp.f90:79-81
    }
}

// ---------------------------------------------------------------- host side
struct Arena {
    std::vector<void *> ptrs;
    bool ok = true;
    ~Arena() {
        for (void *p : ptrs) cudaFree(p);
    }
    template <typename T> T *get(size_t n) {
        void *p = nullptr;
        if (cudaMalloc(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) {
            ok = false;
            return nullptr;
        }
        ptrs.push_back(p);
        return (T *)p;
    }
};

struct Stream {
    cudaStream_t s = nullptr;
    ~Stream() {
        if (s) cudaStreamDestroy(s);
    }
};

}  // namespace

extern "C" int gom_geometry_build(const gom_mesh *mesh, gom_mesh_geometry *out, gom_status *failure) {
    if (failure) std::memset(failure, 0, sizeof(*failure));
    if (!mesh || !out || mesh->n_nodes <= 0 || mesh->n_cells <= 0 || mesh->max_nb <= 0 || mesh->max_nb > GOM_MAXNB ||
        mesh->n_layers <= 0 || mesh->n_ob < 0 || mesh->n_qb < 0 || !mesh->x_node || !mesh->y_node || !mesh->h_node ||
        !mesh->tri_or_quad || !mesh->nodenum_at_cell || !mesh->z_level || (mesh->n_ob > 0 && !mesh->ob_nodes) ||
        (mesh->n_qb > 0 && !mesh->qb_nodes) || out->face_capacity <= 0 || mesh->n_cells >= (1 << 29) ||
        mesh->n_nodes >= (1 << 30))
        return GOM_E_ARG;
    const gom_mesh &mh = *mesh;
    const int NN = mh.n_nodes, NC = mh.n_cells, NB = mh.max_nb, L = mh.n_layers, NOB = mh.n_ob, NQB = mh.n_qb;
    // every index the kernels follow is checked here first
    long sum_k = 0;
    for (int i = 0; i < NC; ++i) {
        const int k = mh.tri_or_quad[i];
        if (k != 3 && k != 4) return GOM_E_ARG;
        sum_k += k;
        for (int l = 0; l < 4; ++l) {
            const int nd = mh.nodenum_at_cell[(size_t)i * 4 + l];
            if (l < k ? (nd < 1 || nd > NN) : nd != 0) return GOM_E_ARG;
        }
    }
    for (int i = 0; i < 2 * (NOB + NQB); ++i) {
        const int nd = i < 2 * NOB ? mh.ob_nodes[i] : mh.qb_nodes[i - 2 * NOB];
        if (nd < 1 || nd > NN) return GOM_E_ARG;
    }
    Stream st;
    if (cudaStreamCreateWithFlags(&st.s, cudaStreamNonBlocking) != cudaSuccess) return GOM_E_CUDA;
    cudaStream_t s = st.s;
    Arena A;
    const size_t FMAX = (size_t)sum_k;
    Mesh m{NN, NC, NB, L, NOB, NQB, mh.voronoi, mh.msl};
    double *x = A.get<double>(NN), *y = A.get<double>(NN), *h = A.get<double>(NN), *zl = A.get<double>(L + 1);
    int *tq = A.get<int>(NC), *cells = A.get<int>(4 * (size_t)NC), *obn = A.get<int>(2 * (size_t)NOB),
        *qbn = A.get<int>(2 * (size_t)NQB);
    double *area = A.get<double>(NC), *x_cell = A.get<double>(NC), *y_cell = A.get<double>(NC),
           *h_cell = A.get<double>(NC);
    int *count = A.get<int>(NN), *slots = A.get<int>((size_t)NN * NB), *acn = A.get<int>((size_t)NN * NB),
        *ncee = A.get<int>((size_t)NN * NB), *an = A.get<int>(NN), *ann = A.get<int>((size_t)NN * (NB + 1));
    int *acc = A.get<int>(4 * (size_t)NC), *owned = A.get<int>(NC), *first = A.get<int>(NC),
        *fac = A.get<int>(4 * (size_t)NC), *sign_io = A.get<int>(4 * (size_t)NC);
    const int tiles = (int)((NC + kScanTile - 1) / kScanTile);
    int *tile_sum = A.get<int>(tiles), *grand = A.get<int>(1);
    int *acf = A.get<int>(2 * FMAX), *nof = A.get<int>(2 * FMAX);
    double *x_face = A.get<double>(FMAX), *y_face = A.get<double>(FMAX), *h_face = A.get<double>(FMAX),
           *flen = A.get<double>(FMAX), *dj = A.get<double>(FMAX), *ct = A.get<double>(FMAX),
           *stt = A.get<double>(FMAX), *ct2 = A.get<double>(FMAX), *st2 = A.get<double>(FMAX);
    int *ob_cell = A.get<int>(NOB), *ob_face = A.get<int>(NOB), *q_cell = A.get<int>(NQB), *q_face = A.get<int>(NQB);
    int *ob_flag = A.get<int>(NC), *q_flag = A.get<int>(NC), *btype = A.get<int>(FMAX), *isflow = A.get<int>(FMAX);
    int *b_cell = A.get<int>(NC), *b_face = A.get<int>(FMAX), *b_node = A.get<int>(NN), *wetdry = A.get<int>(NN);
    u64 *fk = A.get<u64>(1);
    if (!A.ok) return GOM_E_NOMEM;
    m.x = x, m.y = y, m.h = h, m.z_level = zl, m.tq = tq, m.cells = cells, m.ob_nodes = obn, m.qb_nodes = qbn;
    cudaError_t e = cudaSuccess;
    auto up = [&](void *dst, const void *src, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
    };
    auto zero = [&](void *dst, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemsetAsync(dst, 0, bytes, s);
    };
    up(x, mh.x_node, 8 * (size_t)NN);
    up(y, mh.y_node, 8 * (size_t)NN);
    up(h, mh.h_node, 8 * (size_t)NN);
    up(zl, mh.z_level, 8 * (size_t)(L + 1));
    up(tq, mh.tri_or_quad, 4 * (size_t)NC);
    up(cells, mh.nodenum_at_cell, 16 * (size_t)NC);
    up(obn, mh.ob_nodes, 8 * (size_t)NOB);
    up(qbn, mh.qb_nodes, 8 * (size_t)NQB);
    zero(count, 4 * (size_t)NN);
    zero(ob_flag, 4 * (size_t)NC);
    zero(q_flag, 4 * (size_t)NC);
    zero(btype, 4 * FMAX);
    zero(isflow, 4 * FMAX);
    zero(fac, 16 * (size_t)NC);
    if (e == cudaSuccess) e = cudaMemsetAsync(fk, 0xff, sizeof(u64), s);
    if (e != cudaSuccess) return GOM_E_CUDA;

    // the failure key after a stage; true when the build must stop there
    u64 key = kNoFailure;
    auto stopped = [&]() {
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(&key, fk, sizeof(u64), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        return e != cudaSuccess || key != kNoFailure;
    };
    auto report = [&]() -> int {
        if (e != cudaSuccess) return GOM_E_CUDA;
        const int site = (int)(key & 0xff);
        const u64 pos = (key >> 8) & ((1ull << 48) - 1);
        int entity = (int)pos, kind = GOM_ENTITY_OTHER;
        switch (site) {
        case GOM_GEO_CONCAVE: case GOM_GEO_AREA: case GOM_GEO_VORONOI: kind = GOM_ENTITY_CELL; break;
        case GOM_GEO_MAX_NB: case GOM_GEO_HANGING: case GOM_GEO_SURROUNDING: kind = GOM_ENTITY_NODE; break;
        case GOM_GEO_FACE_LENGTH: entity = (int)(pos >> 1), kind = GOM_ENTITY_FACE; break;
        case GOM_GEO_CENTRES: kind = GOM_ENTITY_FACE; break;
        case GOM_GEO_BALL: {   // the cell that owns face pos >> 1, or the cell fmax + i of k_check_fac
            int owner = 0;
            const u64 j = pos >> 1;
            if (j > FMAX) owner = (int)(j - FMAX);
            else cudaMemcpy(&owner, acf + 2 * (j - 1), sizeof(int), cudaMemcpyDeviceToHost);
            entity = owner, kind = GOM_ENTITY_CELL;
            break;
        }
        case GOM_GEO_VERTICAL: {
            const int which = (int)(pos >> 32);
            entity = (int)(pos & 0xffffffffu);
            kind = which == 0 ? GOM_ENTITY_CELL : which == 1 ? GOM_ENTITY_FACE : GOM_ENTITY_NODE;
            break;
        }
        default: break;
        }
        if (failure) {
            failure->code = GOM_E_ARG;
            failure->site = site;
            failure->entity = entity;
            failure->entity_kind = kind;
        }
        return GOM_E_ARG;
    };

    k_area<<<blocks(NC), kThreads, 0, s>>>(m, area, fk);
    k_node_claim<<<blocks(4L * NC), kThreads, 0, s>>>(m, count, slots, fk);
    k_node_sort<<<blocks(NN), kThreads, 0, s>>>(m, count, slots, acn, ncee, fk);
    if (stopped()) return report();
    k_node_nodes<<<blocks(NN), kThreads, 0, s>>>(m, count, acn, an, ann, fk);
    k_cell_adj<<<blocks(NC), kThreads, 0, s>>>(m, count, acn, acc, owned);
    k_scan_tiles<<<tiles, kScanThreads, 0, s>>>(owned, NC, first, tile_sum);
    k_scan_sums<<<1, kScanThreads, 0, s>>>(tile_sum, tiles, grand);
    k_scan_add<<<blocks(NC), kThreads, 0, s>>>(first, NC, tile_sum);
    if (stopped()) return report();
    int NF = 0;
    if (cudaMemcpy(&NF, grand, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return GOM_E_CUDA;
    if (NF < NC || NF < NN || NF > out->face_capacity || (size_t)NF > FMAX) {
        key = ((u64)5 << 56) | GOM_GEO_FACE_COUNT;   // set_geometry_1.f90:254-257, or no room in out
        report();
        if (failure) failure->entity = NF;
        return GOM_E_ARG;
    }
    k_faces<<<blocks(NC), kThreads, 0, s>>>(m, acc, first, fac, acf, nof, x_face, y_face, h_face, flen, fk);
    k_check_fac<<<blocks(NC), kThreads, 0, s>>>(m, fac, (long)FMAX, fk);
    if (stopped()) return report();
    k_cells<<<blocks(NC), kThreads, 0, s>>>(m, fac, acf, h_face, sign_io, x_cell, y_cell, h_cell, fk);
    k_faces2<<<blocks(NF), kThreads, 0, s>>>(m, NF, acf, nof, x_cell, y_cell, x_face, y_face, dj, ct, stt, ct2, st2, fk);
    if (NOB + NQB > 0)
        k_boundary_find<<<blocks(NOB + NQB), kThreads, 0, s>>>(m, count, acn, fac, nof, ob_cell, ob_face, q_cell,
                                                                q_face, fk);
    if (stopped()) return report();
    if (NOB + NQB > 0)
        k_boundary_flags<<<blocks(NOB + NQB), kThreads, 0, s>>>(m, ob_cell, ob_face, q_cell, q_face, ob_flag, btype,
                                                                 q_flag, isflow);
    const int nmax = NC > NF ? (NC > NN ? NC : NN) : (NF > NN ? NF : NN);
    k_layers<<<blocks(nmax), kThreads, 0, s>>>(m, NF, acf, h_cell, h_face, btype, b_cell, b_face, b_node, wetdry, fk);
    if (stopped()) return report();

    auto down = [&](void *dst, const void *src, size_t bytes) {
        if (dst && e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
    };
    gom_mesh_geometry &o = *out;
    const size_t F = (size_t)NF;
    down(o.adj_cells_at_node, count, 4 * (size_t)NN);
    down(o.adj_cellnum_at_node, acn, 4 * (size_t)NN * NB);
    down(o.node_count_each_element, ncee, 4 * (size_t)NN * NB);
    down(o.adj_nodes_at_node, an, 4 * (size_t)NN);
    down(o.adj_nodenum_at_node, ann, 4 * (size_t)NN * (NB + 1));
    down(o.bottom_layer_at_node, b_node, 4 * (size_t)NN);
    down(o.initial_wetdry_node, wetdry, 4 * (size_t)NN);
    down(o.x_cell, x_cell, 8 * (size_t)NC);
    down(o.y_cell, y_cell, 8 * (size_t)NC);
    down(o.h_cell, h_cell, 8 * (size_t)NC);
    down(o.area, area, 8 * (size_t)NC);
    down(o.facenum_at_cell, fac, 16 * (size_t)NC);
    down(o.adj_cellnum_at_cell, acc, 16 * (size_t)NC);
    down(o.sign_in_outflow, sign_io, 16 * (size_t)NC);
    down(o.bottom_layer_at_element, b_cell, 4 * (size_t)NC);
    down(o.ob_element_flag, ob_flag, 4 * (size_t)NC);
    down(o.qb_element_flag, q_flag, 4 * (size_t)NC);
    down(o.x_face, x_face, 8 * F);
    down(o.y_face, y_face, 8 * F);
    down(o.h_face, h_face, 8 * F);
    down(o.face_length, flen, 8 * F);
    down(o.delta_j, dj, 8 * F);
    down(o.cos_theta, ct, 8 * F);
    down(o.sin_theta, stt, 8 * F);
    down(o.cos_theta2, ct2, 8 * F);
    down(o.sin_theta2, st2, 8 * F);
    down(o.adj_cellnum_at_face, acf, 8 * F);
    down(o.nodenum_at_face, nof, 8 * F);
    down(o.bottom_layer_at_face, b_face, 4 * F);
    down(o.boundary_type_of_face, btype, 4 * F);
    down(o.isflowside3, isflow, 4 * F);
    down(o.ob_cell_id, ob_cell, 4 * (size_t)NOB);
    down(o.ob_face_id, ob_face, 4 * (size_t)NOB);
    down(o.qb_cell, q_cell, 4 * (size_t)NQB);
    down(o.qb_face, q_face, 4 * (size_t)NQB);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return GOM_E_CUDA;
    o.n_faces = NF;
    return GOM_OK;
}
