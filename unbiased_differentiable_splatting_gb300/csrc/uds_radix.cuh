// Stable LSD radix-sort passes over (key, value) pairs, 8 bits per pass,
// shared by the tree build (Morton keys) and the deterministic per-splat
// gather (splat keys).  Per pass: k_radix_hist counts each tile's digits
// (digit-major over tiles), an exclusive scan of those counts gives every
// (digit, tile) its output base, and k_radix_scatter writes each tile's
// items in item order (per-warp running counts give a stable rank).  The
// item count is N, or *n_dev when that pointer is given (read on the device;
// N then sizes the grid).  Internal linkage: each translation unit that
// includes this header gets its own copy of the kernels.
#pragma once
#include "uds_common.cuh"

namespace uds {
namespace {

constexpr int kSortThreads = 256, kSortItems = 8, kSortTile = kSortThreads * kSortItems;

// Tile of 2048 items per block: warp w owns items [w*256, w*256+256) of the
// tile, lane l holds item w*256 + r*32 + l in round r, so (round, lane) order
// is item order and per-warp running counts give a stable rank.
__global__ void k_radix_hist(int N, const unsigned* __restrict__ n_dev, const uint32_t* __restrict__ keys,
                             int shift, uint32_t* __restrict__ hist) {
    if (n_dev) N = min(N, (int)*n_dev);
    __shared__ unsigned cnt[256];
    for (int d = threadIdx.x; d < 256; d += blockDim.x) cnt[d] = 0;
    __syncthreads();
    size_t base = (size_t)blockIdx.x * kSortTile;
    for (int r = 0; r < kSortItems; ++r) {
        size_t i = base + (size_t)r * kSortThreads + threadIdx.x;
        if (i < (size_t)N) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[(size_t)d * gridDim.x + blockIdx.x] = cnt[d];
}

__global__ void k_radix_scatter(int N, const unsigned* __restrict__ n_dev, const uint32_t* __restrict__ kin,
                                const uint32_t* __restrict__ vin,
                                uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, int shift,
                                const uint32_t* __restrict__ hist) {
    if (n_dev) N = min(N, (int)*n_dev);
    __shared__ unsigned wcnt[kSortThreads / 32][256];
    __shared__ unsigned goff[256];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = lane; d < 256; d += 32) wcnt[warp][d] = 0;
    for (int d = threadIdx.x; d < 256; d += blockDim.x) goff[d] = hist[(size_t)d * gridDim.x + blockIdx.x];
    __syncwarp();
    size_t base = (size_t)blockIdx.x * kSortTile + (size_t)warp * 256;
    uint32_t key[kSortItems], val[kSortItems];
    unsigned rank[kSortItems];
    unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        size_t i = base + (size_t)r * 32 + lane;
        bool ok = i < (size_t)N;
        key[r] = ok ? kin[i] : 0xFFFFFFFFu;
        val[r] = ok ? vin[i] : 0u;
        unsigned dig = ok ? ((key[r] >> shift) & 255u) : 256u;
        unsigned peers = __match_any_sync(0xffffffffu, dig);
        unsigned before = 0;
        if (ok) before = wcnt[warp][dig];
        rank[r] = before + __popc(peers & lt);
        __syncwarp();
        if (ok && (peers & lt) == 0) wcnt[warp][dig] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    if (threadIdx.x < 256) {
        unsigned run = 0;
        for (int w = 0; w < kSortThreads / 32; ++w) {
            unsigned c = wcnt[w][threadIdx.x];
            wcnt[w][threadIdx.x] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        size_t i = base + (size_t)r * 32 + lane;
        if (i < (size_t)N) {
            unsigned dig = (key[r] >> shift) & 255u;
            unsigned pos = goff[dig] + wcnt[warp][dig] + rank[r];
            kout[pos] = key[r];
            vout[pos] = val[r];
        }
    }
}

}  // namespace
}  // namespace uds
