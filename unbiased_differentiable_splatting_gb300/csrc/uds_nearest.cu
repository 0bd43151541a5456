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

namespace uds {

// ------------------------------------------------ nearest-sample regulariser
// The two losses of NearestSamplesRegularizer (splatting/regularizier.py:
// 119-175) over the nearest lists, with their gradients, in one pass: one
// thread per splat i walks its M neighbours j (index > 0: the reference's
// mask also drops index 0) and accumulates
//   w_j = exp(-|n_i - n_j|^2 / s^2) exp(-|p_i - p_j|^2 / s^2),
//   A = sum w_j, F = sum w_j n_j, D = sum w_j (p_i - p_j).n_j;
// then plane_i = (D / (A + 1e-4))^2 and normal_i = min(1, #neighbours)
// |F / (|F| + 1e-4) - n_i|^2.  The weights, the neighbours and the filtered
// normal are constants of the loss (computed without gradient in the
// reference), so d plane_i / d p_i = 2 D F / (A + 1e-4)^2 and
// d normal_i / d n_i = -2 min(1, #) (F / (|F| + 1e-4) - n_i); gradients of
// the neighbours' points and normals are zero.  The per-splat losses are
// summed per block in a fixed order (warp trees, then warps), and the block
// sums by one thread in block order: the result does not depend on timing.
constexpr int kRegThreads = 256;

__global__ void __launch_bounds__(kRegThreads) k_nearest_regularizer(
    int N, int M, const int* __restrict__ nearest, const float* __restrict__ pts, const float* __restrict__ nrm,
    float inv_s2, float scale, float* __restrict__ gpts, float* __restrict__ gnrm, float2* __restrict__ part) {
    __shared__ float2 red[kRegThreads / 32];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float normal_loss = 0.0f, plane_loss = 0.0f;
    if (i < N) {
        float p[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        float n[3] = {nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]};
        float A = 0.0f, D = 0.0f, F[3] = {0.0f, 0.0f, 0.0f};
        int cnt = 0;
        for (int m = 0; m < M; ++m) {
            int j = nearest[(size_t)i * M + m];
            if (j <= 0 || j >= N) continue;
            ++cnt;
            float q[3] = {pts[3 * j], pts[3 * j + 1], pts[3 * j + 2]};
            float nj[3] = {nrm[3 * j], nrm[3 * j + 1], nrm[3 * j + 2]};
            float dn2 = 0.0f, dp2 = 0.0f, pd = 0.0f;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float a = n[c] - nj[c], b = p[c] - q[c];
                dn2 += a * a;
                dp2 += b * b;
                pd += b * nj[c];
            }
            float w = expf(-dn2 * inv_s2) * expf(-dp2 * inv_s2);
            A += w;
            D += w * pd;
#pragma unroll
            for (int c = 0; c < 3; ++c) F[c] += w * nj[c];
        }
        float inv = 1.0f / (A + 1e-4f);
        float x = D * inv;
        plane_loss = x * x;
        float fn = 1.0f / (sqrtf(F[0] * F[0] + F[1] * F[1] + F[2] * F[2]) + 1e-4f);
        float mask = cnt > 0 ? 1.0f : 0.0f;
        float gp = scale * 2.0f * x * inv;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            float e = F[c] * fn - n[c];
            normal_loss += e * e;
            gnrm[3 * (size_t)i + c] = -scale * 2.0f * mask * e;
            gpts[3 * (size_t)i + c] = gp * F[c];
        }
        normal_loss *= mask;
    }
    for (int o = 16; o > 0; o >>= 1) {
        normal_loss += __shfl_xor_sync(0xffffffffu, normal_loss, o);
        plane_loss += __shfl_xor_sync(0xffffffffu, plane_loss, o);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_float2(normal_loss, plane_loss);
    __syncthreads();
    if (threadIdx.x == 0) {
        float2 s = make_float2(0.0f, 0.0f);
        for (int w = 0; w < kRegThreads / 32; ++w) {
            s.x += red[w].x;
            s.y += red[w].y;
        }
        part[blockIdx.x] = s;
    }
}

__global__ void k_nearest_regularizer_sum(int nb, const float2* __restrict__ part, float scale,
                                          float* __restrict__ losses) {
    float2 s = make_float2(0.0f, 0.0f);
    for (int b = 0; b < nb; ++b) {
        s.x += part[b].x;
        s.y += part[b].y;
    }
    losses[0] = s.x * scale;
    losses[1] = s.y * scale;
}

}  // namespace uds

extern "C" size_t uds_nearest_regularizer_workspace_size(int N) {
    if (N < 0) return 0;
    return sizeof(float2) * (size_t)cdiv(N > 0 ? N : 1, kRegThreads);
}

extern "C" int uds_nearest_regularizer(int N, int M, const int32_t* nearest, const float* points,
                                       const float* normals, float sigma, int mean, float* losses,
                                       float* grad_points, float* grad_normals, void* workspace,
                                       size_t workspace_bytes, void* stream) {
    if (N < 0 || M < 1 || !(sigma > 0.0f) || !losses || (N > 0 && (!nearest || !points || !normals ||
                                                                   !grad_points || !grad_normals)))
        return UDS_ERR_ARGUMENT;
    if (!workspace || workspace_bytes < uds_nearest_regularizer_workspace_size(N)) return UDS_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    int nb = (int)cdiv(N > 0 ? N : 1, kRegThreads);
    float scale = (mean && N > 0) ? 1.0f / (float)N : 1.0f;
    float2* part = reinterpret_cast<float2*>(workspace);
    k_nearest_regularizer<<<nb, kRegThreads, 0, s>>>(N, M, nearest, points, normals, 1.0f / (sigma * sigma), scale,
                                                      grad_points, grad_normals, part);
    k_nearest_regularizer_sum<<<1, 1, 0, s>>>(nb, part, mean ? 1.0f / (float)(N > 0 ? N : 1) : 1.0f, losses);
    return launch_status(2);
}
