// Compact (entity, layer) work lists.
//
// Layered kernels of the mixed path and the flat ELM walk run over the (entity, layer) pairs that
// have work this step instead of over every slot of the (L, entity) arrays: with a shared z-level
// grid most slots of a shallow column are empty, and a lane given an empty slot idles for the
// whole kernel.  A list entry is ((entity << 6) | (layer - 1)) as a 32-bit pattern, entities
// 1-based and in natural order, layers ascending, so layers of one column sit on neighbouring
// lanes.  Built in three launches: count and scan per block of LIST_BLOCK entities, scan of the
// block sums in one block, scatter.  A range functor gives each entity's first and last layer
// (an empty column has last < first).
#pragma once
#include <cuda_runtime.h>

namespace gom {

constexpr int LIST_BLOCK = 1024;
constexpr int LIST_MAX_ENTITIES = 1 << 26;   // entity index fits the 26 high bits of an entry

__device__ __forceinline__ int list_entity(int code) { return (int)((unsigned)code >> 6); }
__device__ __forceinline__ int list_layer(int code) { return (code & 63) + 1; }

// inclusive warp scan, then block totals in warp_tot; returns the exclusive prefix within the block
__device__ __forceinline__ int block_exclusive_scan(int n, int *warp_tot, int &block_total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int v = n;
    for (int o = 1; o < 32; o <<= 1) {
        int u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    if (lane == 31) warp_tot[w] = v;
    __syncthreads();
    if (w == 0) {
        int x = lane < LIST_BLOCK / 32 ? warp_tot[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int u = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += u;
        }
        if (lane < LIST_BLOCK / 32) warp_tot[lane] = x;   // inclusive warp totals
    }
    __syncthreads();
    block_total = warp_tot[LIST_BLOCK / 32 - 1];
    return (w > 0 ? warp_tot[w - 1] : 0) + v - n;
}

template <class Range> __device__ __forceinline__ int range_count(const Range &r, int i) {
    int2 fl = r(i);
    return fl.y >= fl.x ? fl.y - fl.x + 1 : 0;
}

template <class Range>
__global__ void __launch_bounds__(LIST_BLOCK) k_list_scan_blocks(int n_ent, Range r, int *off, int *bsum) {
    __shared__ int warp_tot[LIST_BLOCK / 32];
    const int i = blockIdx.x * LIST_BLOCK + threadIdx.x;   // 0-based entity
    const int n = i < n_ent ? range_count(r, i) : 0;
    int total;
    const int before = block_exclusive_scan(n, warp_tot, total);
    if (i < n_ent) off[i] = before;
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// count[0] = list length; count[1] = 0 (the work-queue counter of kernels that take entries
// dynamically)
template <int Dummy = 0> __global__ void __launch_bounds__(LIST_BLOCK) k_list_scan_sums(int nblocks, int *bsum, int *count) {
    __shared__ int warp_tot[LIST_BLOCK / 32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nblocks; base += LIST_BLOCK) {
        const int i = base + threadIdx.x;
        const int n = i < nblocks ? bsum[i] : 0;
        int total;
        const int excl = carry + block_exclusive_scan(n, warp_tot, total);
        if (i < nblocks) bsum[i] = excl;
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        count[0] = carry;
        count[1] = 0;
    }
}

template <class Range> __global__ void k_list_scatter(int n_ent, Range r, const int *off, const int *bsum, int *list) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_ent) return;
    const int2 fl = r(i);
    if (fl.y < fl.x) return;
    int o = bsum[i / LIST_BLOCK] + off[i];
    const unsigned id = (unsigned)(i + 1) << 6;
    for (int k = fl.x; k <= fl.y; ++k) list[o++] = (int)(id | (unsigned)(k - 1));
}

// off: n_ent ints, bsum: n_ent / LIST_BLOCK + 1 ints, count: 2 ints, list: up to n_ent * L ints
template <class Range>
cudaError_t build_layer_list(int n_ent, const Range &r, int *off, int *bsum, int *list, int *count,
                             cudaStream_t stream) {
    const int nb = (n_ent + LIST_BLOCK - 1) / LIST_BLOCK;
    k_list_scan_blocks<<<nb, LIST_BLOCK, 0, stream>>>(n_ent, r, off, bsum);
    k_list_scan_sums<<<1, LIST_BLOCK, 0, stream>>>(nb, bsum, count);
    k_list_scatter<<<(n_ent + 255) / 256, 256, 0, stream>>>(n_ent, r, off, bsum, list);
    return cudaGetLastError();
}

}   // namespace gom
