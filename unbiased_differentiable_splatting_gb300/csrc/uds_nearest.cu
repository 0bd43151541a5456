// nearestsamples.nearest (nearestSamples.cpp:31-75, nearestSamplesCuda.cu:
// 355-564): for every splat, the numNearest nearest other splats among those
// sampled together with it in pixels where it is the surface splat.
//
// Per pixel the surface splat is the sample with the largest (filtered)
// weight, the first one on ties (fastNearestKernel:375-386); every other
// valid sample of the pixel is a candidate neighbour of it at Euclidean
// distance |p_s - p_c| (camera or world points, (1, N, 3)).  The reference
// merges each pixel's sorted candidates into the splat's list under a spin
// lock, so the list depends on the order in which pixels win the lock and is
// padded with whatever entries of infinite distance were left.  Here the
// result is defined by the candidate set alone: the numNearest distinct
// candidates of smallest distance, ordered by (distance, index), padded with
// -1.  No locks: the (surface, candidate) pairs are bucketed per surface
// splat (count, scan, place) and one thread per splat selects from its
// bucket.  Distances use exact-rounding operations, so the order matches the
// oracle's bit for bit.
#include "uds_common.cuh"
#include "uds_scan.cuh"

namespace uds {

__device__ __forceinline__ float point_distance(const float* __restrict__ pts, int a, int b) {
    float dx = fsub(pts[3 * a], pts[3 * b]);
    float dy = fsub(pts[3 * a + 1], pts[3 * b + 1]);
    float dz = fsub(pts[3 * a + 2], pts[3 * b + 2]);
    return fsqrt(fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz)));
}

__device__ __forceinline__ int surface_sample(const int* __restrict__ idx, const float* __restrict__ w, size_t base,
                                              int K, int N) {
    int s = idx[base];
    float sw = w[base];
    for (int k = 1; k < K; ++k)
        if (w[base + k] > sw) {
            sw = w[base + k];
            s = idx[base + k];
        }
    return (s >= 0 && s < N) ? s : -1;
}

// pass 0: count candidates per surface splat; pass 1: place them
__global__ void k_nearest_pairs(size_t P, int K, int N, const int* __restrict__ idx, const float* __restrict__ w,
                                unsigned* __restrict__ count, const unsigned* __restrict__ offs,
                                unsigned* __restrict__ fill, int* __restrict__ cand, int pass) {
    size_t pix = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= P) return;
    size_t base = pix * K;
    int s = surface_sample(idx, w, base, K, N);
    if (s < 0) return;
    for (int k = 0; k < K; ++k) {
        int c = idx[base + k];
        if (c < 0 || c >= N || c == s) continue;
        if (pass == 0) atomicAdd(&count[s], 1u);
        else cand[offs[s] + atomicAdd(&fill[s], 1u)] = c;
    }
}

constexpr int kMaxNearest = 32;

__global__ void k_nearest_select(int N, int M, const float* __restrict__ pts, const unsigned* __restrict__ offs,
                                 const int* __restrict__ cand, int* __restrict__ out) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    float bd[kMaxNearest];
    int bi[kMaxNearest];
    int m = 0;
    for (unsigned i = offs[s]; i < offs[s + 1]; ++i) {
        int c = cand[i];
        float d = point_distance(pts, s, c);
        // already listed?
        bool dup = false;
        for (int q = 0; q < m; ++q) dup |= bi[q] == c;
        if (dup) continue;
        if (m == M && !(d < bd[M - 1] || (d == bd[M - 1] && c < bi[M - 1]))) continue;
        int q = m < M ? m++ : M - 1;
        while (q > 0 && (d < bd[q - 1] || (d == bd[q - 1] && c < bi[q - 1]))) {
            bd[q] = bd[q - 1];
            bi[q] = bi[q - 1];
            --q;
        }
        bd[q] = d;
        bi[q] = c;
    }
    for (int q = 0; q < M; ++q) out[(size_t)s * M + q] = q < m ? bi[q] : -1;
}

}  // namespace uds

using namespace uds;

extern "C" size_t uds_nearest_workspace_size(int B, int W, int H, int K, int N) {
    if (B <= 0 || W <= 0 || H <= 0 || K <= 0 || N < 0) return 0;
    auto a = [](size_t x) { return (x + 255) & ~(size_t)255; };
    size_t S = (size_t)B * W * H * K;
    return 2 * a(4 * (size_t)N) + a(4 * ((size_t)N + 1)) + a(4 * S) + a(4 * scan_part_entries((size_t)N));
}

extern "C" int uds_nearest_samples(int B, int W, int H, int K, const int32_t* indices, const float* weights, int N,
                                   const float* points, int num_nearest, int32_t* nearest, void* workspace,
                                   size_t workspace_bytes, void* stream) {
    if (B <= 0 || W <= 0 || H <= 0 || K <= 0 || N < 0 || num_nearest < 1 || num_nearest > kMaxNearest ||
        !indices || !weights || (N > 0 && (!points || !nearest)))
        return UDS_ERR_ARGUMENT;
    if (N == 0) return UDS_OK;
    // pair counts, offsets and the scan are 32-bit
    if ((size_t)B * W * H * K >= (1ull << 32)) return UDS_ERR_ARGUMENT;
    if (!workspace || workspace_bytes < uds_nearest_workspace_size(B, W, H, K, N)) return UDS_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    auto a = [](size_t x) { return (x + 255) & ~(size_t)255; };
    char* p = reinterpret_cast<char*>(workspace);
    unsigned* count = reinterpret_cast<unsigned*>(p);
    unsigned* fill = reinterpret_cast<unsigned*>(p + a(4 * (size_t)N));
    unsigned* offs = reinterpret_cast<unsigned*>(p + 2 * a(4 * (size_t)N));
    int* cand = reinterpret_cast<int*>(p + 2 * a(4 * (size_t)N) + a(4 * ((size_t)N + 1)));
    unsigned* part = reinterpret_cast<unsigned*>(p + 2 * a(4 * (size_t)N) + a(4 * ((size_t)N + 1)) +
                                                 a(4 * (size_t)B * W * H * K));
    cudaError_t e = cudaMemsetAsync(count, 0, 2 * a(4 * (size_t)N), s);
    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    size_t P = (size_t)B * W * H;
    // all views' pixels feed one list per splat (points (1, N, 3), as the
    // reference assumes)
    k_nearest_pairs<<<cdiv(P, 256), 256, 0, s>>>(P, K, N, indices, weights, count, nullptr, nullptr, nullptr, 0);
    exclusive_scan((size_t)N, count, offs, part, s);
    k_nearest_pairs<<<cdiv(P, 256), 256, 0, s>>>(P, K, N, indices, weights, nullptr, offs, fill, cand, 1);
    k_nearest_select<<<cdiv(N, 128), 128, 0, s>>>(N, num_nearest, points, offs, cand, nearest);
    return launch_status(6);
}
