// filtering.forward / filtering.backward (zSorting.cpp:24-43,
// zSortingCuda.cu:11-243, alphacompositing.cuh, alphacompositingGrad.cuh):
// per pixel, the depth of each sample along the pixel ray to the splat's
// tangent plane, a stable insertion arg-sort by depth, front-to-back alpha
// blending and its division-based gradient.  The arithmetic follows the
// reference operation by operation (double where it promotes), so the depth
// order is identical to the CPU oracle's.
#include "uds_composite.cuh"

namespace uds {

constexpr int kFilterThreads = 64;

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
    float wl[KMAX], fw[KMAX];
    for (int k = 0; k < K; ++k) wl[k] = w[e + k];
    blend<KMAX>(K, ord, wl, fw);
    for (int k = 0; k < K; ++k) out[e + k] = fw[k];
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
    float dist[KMAX], fw[KMAX], wl[KMAX], gl[KMAX];
    int ord[KMAX];
    for (int k = 0; k < K; ++k) {
        dist[k] = sample_depth(dir, pts + po, nrm + po, idx[e + k], N);
        wl[k] = w[e + k];
        gl[k] = gin[e + k];
    }
    depth_order<KMAX>(K, dist, ord);
    blend<KMAX>(K, ord, wl, fw);
    for (int k = 0; k < K; ++k) out[e + ord[k]] = blend_grad<KMAX>(K, k, ord, wl, fw, gl);
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
