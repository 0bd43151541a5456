// filtering.forward / filtering.backward (zSorting.cpp:24-43,
// zSortingCuda.cu:11-243, alphacompositing.cuh, alphacompositingGrad.cuh):
// per pixel, the depth of each sample along the pixel ray to the splat's
// tangent plane, a stable insertion arg-sort by depth, front-to-back alpha
// blending and its division-based gradient.  The arithmetic follows the
// reference operation by operation (double where it promotes), so the depth
// order is identical to the CPU oracle's.
#include "uds_ewa.cuh"

namespace uds {

constexpr int kFilterThreads = 64;

// -normalize(backproject(pixel)) (alphacompositing.cuh:31-32)
__device__ __forceinline__ void pixel_ray(float W, float H, float f, float px, float py, float* dir) {
    float s[2] = {px, py}, wd[3];
    back_project(W, H, f, s, wd);
    float inv = div_via_double(1.0f, fsqrt(dot3(wd, wd)));
#pragma unroll
    for (int i = 0; i < 3; ++i) dir[i] = fmul(fmul(wd[i], inv), -1.0f);
}

__device__ __forceinline__ float sample_depth(const float* dir, const float* __restrict__ pts,
                                              const float* __restrict__ nrm, int id, int N) {
    if (id < 0 || id >= N) return kZmax;
    float p[3] = {pts[3 * (size_t)id], pts[3 * (size_t)id + 1], pts[3 * (size_t)id + 2]};
    float n[3] = {nrm[3 * (size_t)id], nrm[3 * (size_t)id + 1], nrm[3 * (size_t)id + 2]};
    float d = fdiv(dot3(p, n), dot3(dir, n));
    return d > 0.0f ? d : kZmax;
}

template <int KMAX>
__device__ __forceinline__ void depth_order(int K, const float* dist, int* ord) {
    for (int i = 0; i < K; ++i) ord[i] = i;
    for (int i = 1; i < K; ++i) {
        int index = ord[i];
        float value = dist[index];
        int j = i;
        while (j > 0 && dist[ord[j - 1]] > value) { ord[j] = ord[j - 1]; --j; }
        ord[j] = index;
    }
}

template <int KMAX>
__global__ void k_filter_forward(int B, int W, int H, int K, const int* __restrict__ idx,
                                 const float* __restrict__ w, float f, int pB, int N,
                                 const float* __restrict__ pts, const float* __restrict__ nrm,
                                 float* __restrict__ out) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y, b = blockIdx.z;
    if (j >= H) return;
    size_t e = (size_t)K * ((size_t)j + (size_t)H * ((size_t)i + (size_t)W * b));
    size_t po = pB > 1 ? 3 * (size_t)N * b : 0;
    float dir[3];
    pixel_ray((float)W, (float)H, f, (float)i, (float)j, dir);
    float dist[KMAX];
    int ord[KMAX];
    for (int k = 0; k < K; ++k) dist[k] = sample_depth(dir, pts + po, nrm + po, idx[e + k], N);
    depth_order<KMAX>(K, dist, ord);
    float rem = 1.0f;
    for (int q = 0; q < K; ++q) {
        int id = ord[q];
        float wt = w[e + id];
        out[e + id] = fmul(rem, wt);
        rem = (float)dmul((double)rem, dsub(1.0, (double)wt));
    }
}

template <int KMAX>
__global__ void k_filter_backward(int B, int W, int H, int K, const int* __restrict__ idx,
                                  const float* __restrict__ w, const float* __restrict__ gin, float f,
                                  int pB, int N, const float* __restrict__ pts,
                                  const float* __restrict__ nrm, float* __restrict__ out) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y, b = blockIdx.z;
    if (j >= H) return;
    size_t e = (size_t)K * ((size_t)j + (size_t)H * ((size_t)i + (size_t)W * b));
    size_t po = pB > 1 ? 3 * (size_t)N * b : 0;
    float dir[3];
    pixel_ray((float)W, (float)H, f, (float)i, (float)j, dir);
    float dist[KMAX], fw[KMAX], wl[KMAX];
    int ord[KMAX];
    for (int k = 0; k < K; ++k) {
        dist[k] = sample_depth(dir, pts + po, nrm + po, idx[e + k], N);
        wl[k] = w[e + k];
    }
    depth_order<KMAX>(K, dist, ord);
    float rem = 1.0f;
    for (int q = 0; q < K; ++q) {
        int id = ord[q];
        fw[id] = fmul(rem, wl[id]);
        rem = (float)dmul((double)rem, dsub(1.0, (double)wl[id]));
    }
    const float eps = 1e-4f;
    for (int k = 0; k < K; ++k) {
        int kdx = ord[k];
        float wk = wl[kdx];
        float g = 0.0f;
        for (int q = k; q < K; ++q) {
            int id = ord[q];
            float den = (q == k) ? wk : -fsub(1.0f, wk);
            if (fabsf(den) > eps) g = fadd(g, fdiv(fmul(gin[e + id], fw[id]), den));
        }
        out[e + kdx] = g;
    }
}

}  // namespace uds

using namespace uds;

#define UDS_FILTER_DISPATCH(KERNEL, ...)                                              \
    do {                                                                                \
        dim3 grid(cdiv(H, kFilterThreads), W, B);                                       \
        if (K <= 8) KERNEL<8><<<grid, kFilterThreads, 0, s>>>(__VA_ARGS__);             \
        else if (K <= 16) KERNEL<16><<<grid, kFilterThreads, 0, s>>>(__VA_ARGS__);      \
        else if (K <= 32) KERNEL<32><<<grid, kFilterThreads, 0, s>>>(__VA_ARGS__);      \
        else KERNEL<64><<<grid, kFilterThreads, 0, s>>>(__VA_ARGS__);                   \
    } while (0)

extern "C" int uds_filter_forward(int B, int W, int H, int K, const int32_t* indices,
                                  const float* weights, float focal, int pB, int N,
                                  const float* points, const float* normals, float* out,
                                  void* stream) {
    if (B <= 0 || W <= 0 || H <= 0 || K <= 0 || K > kMaxK || (pB != 1 && pB != B) || N < 0) return UDS_ERR_ARGUMENT;
    if (!indices || !weights || !out) return UDS_ERR_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    UDS_FILTER_DISPATCH(k_filter_forward, B, W, H, K, indices, weights, focal, pB, N, points, normals, out);
    return launch_status();
}

extern "C" int uds_filter_backward(int B, int W, int H, int K, const int32_t* indices,
                                   const float* weights, const float* grad, float focal, int pB,
                                   int N, const float* points, const float* normals,
                                   float* grad_weights, void* stream) {
    if (B <= 0 || W <= 0 || H <= 0 || K <= 0 || K > kMaxK || (pB != 1 && pB != B) || N < 0) return UDS_ERR_ARGUMENT;
    if (!indices || !weights || !grad || !grad_weights) return UDS_ERR_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    UDS_FILTER_DISPATCH(k_filter_backward, B, W, H, K, indices, weights, grad, focal, pB, N, points, normals,
                        grad_weights);
    return launch_status();
}
