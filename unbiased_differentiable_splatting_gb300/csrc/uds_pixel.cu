// Per-sample scatter / per-splat gather (pixelgather.scatter / gather,
// splatting/extensions/pixelGatherCuda.cu:7-152): the consumers of the
// sampled indices right after the render (visibility counting in cleanup.py:41,
// PixelScatterGather in extensions/__init__.py:407-437).
//
// scatter: out (B,W,H,K,C) = values (B,N,C) at each sample's splat, 0 where
//          the index is -1 (or outside [0, N)).
// gather:  out (B,N,C) = sum over the samples of splat j of values (B,W,H,K,C).
//   atomic mode: lanes of a warp that hold the same splat first combine their
//     values (__match_any_sync + shuffles), then one atomic per group and
//     channel; the order of additions is not fixed (like the reference).
//   deterministic mode: the valid samples are compacted in sample order and
//     stably radix-sorted by splat (so each splat's samples stay in sample
//     order, however many there are), bucket offsets come from per-splat
//     counts, and one thread sums its splat's values in that order: the
//     result is bit-identical to a sequential sum in sample order.
#include "uds_common.cuh"
#include "uds_radix.cuh"
#include "uds_scan.cuh"

namespace uds {

// one thread per (sample, channel) would re-read the index C times; one
// thread per sample copies C contiguous floats
__global__ void k_pixel_scatter(size_t S, size_t per_view, int N, int C, const int* __restrict__ idx,
                                 const float* __restrict__ values, float* __restrict__ out) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S) return;
    size_t b = t / per_view;
    int id = idx[t];
    float* o = out + t * (size_t)C;
    if (id < 0 || id >= N) {
        for (int c = 0; c < C; ++c) o[c] = 0.0f;
        return;
    }
    const float* v = values + ((size_t)id + (size_t)N * b) * C;
    for (int c = 0; c < C; ++c) o[c] = v[c];
}

__global__ void k_pixel_gather_atomic(size_t S, size_t per_view, int N, int C, const int* __restrict__ idx,
                                      const float* __restrict__ values, float* __restrict__ out) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool live = t < S;
    int id = live ? idx[t] : -1;
    size_t key = (live && id >= 0 && id < N) ? (size_t)id + (size_t)N * (t / per_view) : ~(size_t)0;
    unsigned peers = __match_any_sync(0xffffffffu, key);
    int lane = threadIdx.x & 31;
    int leader = __ffs(peers) - 1;
    for (int c = 0; c < C; ++c) {
        float v = (key != ~(size_t)0) ? values[t * (size_t)C + c] : 0.0f;
        // sum over the group of lanes with the same splat
        float s = 0.0f;
        unsigned m = peers;
        while (m) {
            int src = __ffs(m) - 1;
            m &= m - 1;
            s += __shfl_sync(peers, v, src);
        }
        if (lane == leader && key != ~(size_t)0) atomicAdd(&out[key * (size_t)C + c], s);
    }
}

// deterministic mode: per-splat counts and the valid-sample flags in one pass
__global__ void k_pixel_count(size_t S, size_t per_view, int N, const int* __restrict__ idx,
                              unsigned* __restrict__ count, unsigned* __restrict__ flag) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S) return;
    int id = idx[t];
    bool ok = id >= 0 && id < N;
    flag[t] = ok ? 1u : 0u;
    if (ok) atomicAdd(&count[(size_t)id + (size_t)N * (t / per_view)], 1u);
}

// the valid samples in sample order: (splat key, sample offset) pairs
__global__ void k_pixel_compact(size_t S, size_t per_view, int N, const int* __restrict__ idx,
                                const unsigned* __restrict__ pos, unsigned* __restrict__ keys,
                                unsigned* __restrict__ samples) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S) return;
    int id = idx[t];
    if (id < 0 || id >= N) return;
    unsigned p = pos[t];
    keys[p] = (unsigned)((size_t)id + (size_t)N * (t / per_view));
    samples[p] = (unsigned)t;
}

// one thread per splat sums its bucket (already in sample order)
__global__ void k_pixel_sum(size_t M, int C, const unsigned* __restrict__ offs, const unsigned* __restrict__ slots,
                            const float* __restrict__ values, float* __restrict__ out) {
    size_t key = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (key >= M) return;
    unsigned lo = offs[key], hi = offs[key + 1];
    for (int c = 0; c < C; ++c) {
        float s = 0.0f;
        for (unsigned i = lo; i < hi; ++i) s = __fadd_rn(s, values[(size_t)slots[i] * C + c]);
        out[key * (size_t)C + c] = s;
    }
}

}  // namespace uds

using namespace uds;

extern "C" int uds_pixel_scatter(int B, int W, int H, int K, const int32_t* indices, int N, int C,
                                 const float* values, float* out, void* stream) {
    if (B <= 0 || W <= 0 || H <= 0 || K <= 0 || N < 0 || C <= 0 || !indices || !out || (N > 0 && !values))
        return UDS_ERR_ARGUMENT;
    size_t per_view = (size_t)W * H * K, S = per_view * B;
    k_pixel_scatter<<<cdiv(S, 256), 256, 0, as_stream(stream)>>>(S, per_view, N, C, indices, values, out);
    return launch_status();
}

// Deterministic-mode scratch: per-splat counts and offsets, sample flags and
// positions, two (key, sample) pair buffers, the radix digit histograms and
// their scan, and the scans' tile sums.
struct GatherWs {
    unsigned *count, *offs, *flag, *pos, *ka, *va, *kb, *vb, *hist, *hscan, *part;
    size_t bytes;
};

static GatherWs gather_layout(size_t M, size_t S, char* base) {
    auto a = [](size_t x) { return (x + 255) & ~(size_t)255; };
    size_t nb = cdiv(S, kSortTile), nh = 256 * nb;
    size_t longest = S > nh ? S : nh;
    size_t parts = scan_part_entries(longest > M ? longest : M);
    GatherWs g{};
    size_t off = 0;
    auto take = [&](size_t n) {
        unsigned* p = base ? reinterpret_cast<unsigned*>(base + off) : nullptr;
        off += a(4 * n);
        return p;
    };
    g.count = take(M);
    g.offs = take(M + 1);
    g.flag = take(S);
    g.pos = take(S + 1);
    g.ka = take(S);
    g.va = take(S);
    g.kb = take(S);
    g.vb = take(S);
    g.hist = take(nh);
    g.hscan = take(nh + 1);
    g.part = take(parts);
    g.bytes = off;
    return g;
}

extern "C" size_t uds_pixel_gather_workspace_size(int B, int W, int H, int K, int N) {
    if (B <= 0 || W <= 0 || H <= 0 || K <= 0 || N < 0) return 0;
    return gather_layout((size_t)B * N, (size_t)B * W * H * K, nullptr).bytes;
}

extern "C" int uds_pixel_gather(int B, int W, int H, int K, const int32_t* indices, int N, int C,
                                const float* values, float* out, int deterministic, void* workspace,
                                size_t workspace_bytes, void* stream) {
    if (B <= 0 || W <= 0 || H <= 0 || K <= 0 || N < 0 || C <= 0 || !indices || !values || (N > 0 && !out))
        return UDS_ERR_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    size_t per_view = (size_t)W * H * K, S = per_view * B, M = (size_t)B * N;
    if (M == 0) return UDS_OK;
    if (S >= (1ull << 32)) return UDS_ERR_ARGUMENT;
    if (!deterministic) {
        cudaError_t e = cudaMemsetAsync(out, 0, sizeof(float) * M * C, s);
        if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
        k_pixel_gather_atomic<<<cdiv(S, 256), 256, 0, s>>>(S, per_view, N, C, indices, values, out);
        return launch_status();
    }
    if (!workspace || workspace_bytes < uds_pixel_gather_workspace_size(B, W, H, K, N)) return UDS_ERR_WORKSPACE;
    GatherWs g = gather_layout(M, S, reinterpret_cast<char*>(workspace));
    cudaError_t e = cudaMemsetAsync(g.count, 0, 4 * M, s);
    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    // bucket offsets from the per-splat counts; the valid samples in sample
    // order, then a stable sort by splat; the number of valid samples
    // (g.pos[S]) stays on the device
    k_pixel_count<<<cdiv(S, 256), 256, 0, s>>>(S, per_view, N, indices, g.count, g.flag);
    exclusive_scan(M, g.count, g.offs, g.part, s);
    exclusive_scan(S, g.flag, g.pos, g.part, s);
    k_pixel_compact<<<cdiv(S, 256), 256, 0, s>>>(S, per_view, N, indices, g.pos, g.ka, g.va);
    int bits = 1;
    while (bits < 32 && (M - 1) >> bits) ++bits;
    unsigned nb = cdiv(S, kSortTile);
    unsigned *ki = g.ka, *vi = g.va, *ko = g.kb, *vo = g.vb;
    int launched = 8;
    for (int shift = 0; shift < bits; shift += 8) {
        k_radix_hist<<<nb, kSortThreads, 0, s>>>((int)S, g.pos + S, ki, shift, g.hist);
        exclusive_scan((size_t)256 * nb, g.hist, g.hscan, g.part, s);
        k_radix_scatter<<<nb, kSortThreads, 0, s>>>((int)S, g.pos + S, ki, vi, ko, vo, shift, g.hscan);
        unsigned* t = ki; ki = ko; ko = t;
        t = vi; vi = vo; vo = t;
        launched += 5;
    }
    k_pixel_sum<<<cdiv(M, 128), 128, 0, s>>>(M, C, g.offs, vi, values, out);
    return launch_status(launched + 1);
}
