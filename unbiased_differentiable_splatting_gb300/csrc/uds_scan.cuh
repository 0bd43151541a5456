// Exclusive prefix sum of M unsigned counts, out[0..M] with out[M] = total,
// in three launches: per-tile sums, one block scanning the tile sums, and
// per-tile scans that add the tile's offset.  Tiles of 1024 counts; each
// thread loads four consecutive counts, so every warp load is contiguous.
// The kernels have internal linkage: each translation unit that includes
// this header gets its own copy.
#pragma once
#include "uds_common.cuh"

namespace uds {
namespace {

constexpr int kSumThreads = 256, kSumItems = 4, kSumTile = kSumThreads * kSumItems;

__global__ void k_sum_tiles(size_t M, const unsigned* __restrict__ in, unsigned* __restrict__ part) {
    __shared__ unsigned red[kSumThreads / 32];
    size_t base = (size_t)blockIdx.x * kSumTile;
    unsigned s = 0;
    for (int r = 0; r < kSumItems; ++r) {
        size_t i = base + (size_t)r * kSumThreads + threadIdx.x;
        if (i < M) s += in[i];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (int w = 0; w < kSumThreads / 32; ++w) t += red[w];
        part[blockIdx.x] = t;
    }
}

// exclusive scan of the nb tile sums in place, part[nb] = the total
__global__ void k_sum_top(unsigned* part, int nb) {
    __shared__ unsigned buf[1024];
    int t = threadIdx.x;
    int per = (nb + blockDim.x - 1) / blockDim.x;
    int lo = t * per, hi = min(nb, lo + per);
    unsigned s = 0;
    for (int i = lo; i < hi; ++i) s += part[i];
    buf[t] = s;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
        unsigned v = t >= o ? buf[t - o] : 0u;
        __syncthreads();
        buf[t] += v;
        __syncthreads();
    }
    unsigned run = t > 0 ? buf[t - 1] : 0u;
    for (int i = lo; i < hi; ++i) {
        unsigned v = part[i];
        part[i] = run;
        run += v;
    }
    if (t == (int)blockDim.x - 1) part[nb] = buf[t];
}

__global__ void k_sum_down(size_t M, const unsigned* __restrict__ in, const unsigned* __restrict__ part,
                           unsigned* __restrict__ out) {
    __shared__ unsigned wsum[kSumThreads / 32];
    size_t base = (size_t)blockIdx.x * kSumTile + (size_t)threadIdx.x * kSumItems;
    unsigned v[kSumItems], local = 0;
#pragma unroll
    for (int r = 0; r < kSumItems; ++r) {
        size_t i = base + r;
        v[r] = i < M ? in[i] : 0u;
        local += v[r];
    }
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned incl = local;
    for (int o = 1; o < 32; o <<= 1) {
        unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    unsigned woff = 0;
    for (int w = 0; w < warp; ++w) woff += wsum[w];
    unsigned run = part[blockIdx.x] + woff + incl - local;
#pragma unroll
    for (int r = 0; r < kSumItems; ++r) {
        size_t i = base + r;
        if (i < M) out[i] = run;
        run += v[r];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[M] = part[gridDim.x];
}

}  // namespace

// entries of the tile-sum scratch for M counts
static inline size_t scan_part_entries(size_t M) { return M / kSumTile + 2; }

// out (M + 1 entries) = exclusive prefix sums of in (M >= 1 entries); part
// holds scan_part_entries(M) entries; three kernel launches on s
static inline void exclusive_scan(size_t M, const unsigned* in, unsigned* out, unsigned* part, cudaStream_t s) {
    unsigned nb = cdiv(M, kSumTile);
    k_sum_tiles<<<nb, kSumThreads, 0, s>>>(M, in, part);
    k_sum_top<<<1, 1024, 0, s>>>(part, (int)nb);
    k_sum_down<<<nb, kSumThreads, 0, s>>>(M, in, part, out);
}

}  // namespace uds
