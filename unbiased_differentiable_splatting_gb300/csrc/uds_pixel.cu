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
//   deterministic mode: the samples are bucketed per splat (counts, scan,
//     placement), each bucket is ordered by sample offset, and one thread sums
//     its splat's values in that order, so the result is bit-identical to a
//     sequential sum in sample order.
#include "uds_common.cuh"
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

// deterministic mode
__global__ void k_pixel_count(size_t S, size_t per_view, int N, const int* __restrict__ idx,
                              unsigned* __restrict__ count) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S) return;
    int id = idx[t];
    if (id >= 0 && id < N) atomicAdd(&count[(size_t)id + (size_t)N * (t / per_view)], 1u);
}

__global__ void k_pixel_place(size_t S, size_t per_view, int N, const int* __restrict__ idx,
                              const unsigned* __restrict__ offs, unsigned* __restrict__ fill,
                              unsigned* __restrict__ slots) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S) return;
    int id = idx[t];
    if (id < 0 || id >= N) return;
    size_t key = (size_t)id + (size_t)N * (t / per_view);
    unsigned p = offs[key] + atomicAdd(&fill[key], 1u);
    slots[p] = (unsigned)t;
}

// one thread per splat: order its samples (insertion sort, buckets are
// short), then sum in that order
__global__ void k_pixel_sum(size_t M, int C, const unsigned* __restrict__ offs, unsigned* __restrict__ slots,
                            const float* __restrict__ values, float* __restrict__ out) {
    size_t key = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (key >= M) return;
    unsigned lo = offs[key], hi = offs[key + 1];
    for (unsigned i = lo + 1; i < hi; ++i) {
        unsigned x = slots[i];
        unsigned j = i;
        while (j > lo && slots[j - 1] > x) {
            slots[j] = slots[j - 1];
            --j;
        }
        slots[j] = x;
    }
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

extern "C" size_t uds_pixel_gather_workspace_size(int B, int W, int H, int K, int N) {
    if (B <= 0 || W <= 0 || H <= 0 || K <= 0 || N < 0) return 0;
    size_t M = (size_t)B * N, S = (size_t)B * W * H * K;
    auto a = [](size_t x) { return (x + 255) & ~(size_t)255; };
    return a(4 * M) * 2 + a(4 * (M + 1)) + a(4 * S) + a(4 * scan_part_entries(M));
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
    auto a = [](size_t x) { return (x + 255) & ~(size_t)255; };
    char* p = reinterpret_cast<char*>(workspace);
    unsigned* count = reinterpret_cast<unsigned*>(p);
    unsigned* fill = reinterpret_cast<unsigned*>(p + a(4 * M));
    unsigned* offs = reinterpret_cast<unsigned*>(p + 2 * a(4 * M));
    unsigned* slots = reinterpret_cast<unsigned*>(p + 2 * a(4 * M) + a(4 * (M + 1)));
    unsigned* part = reinterpret_cast<unsigned*>(p + 2 * a(4 * M) + a(4 * (M + 1)) + a(4 * S));
    cudaError_t e = cudaMemsetAsync(count, 0, 2 * a(4 * M), s);  // count and fill
    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    k_pixel_count<<<cdiv(S, 256), 256, 0, s>>>(S, per_view, N, indices, count);
    exclusive_scan(M, count, offs, part, s);
    k_pixel_place<<<cdiv(S, 256), 256, 0, s>>>(S, per_view, N, indices, offs, fill, slots);
    k_pixel_sum<<<cdiv(M, 128), 128, 0, s>>>(M, C, offs, slots, values, out);
    return launch_status(6);
}
