// interpolation.forward / interpolation.backward (interpolation.cpp:31-95,
// interpolationCuda.cu:5-167): image[c] = sum_k w_k attr[idx_k][c] and its
// gradient.  One thread per pixel owns its output row, so the forward needs
// no atomics (the reference uses them); the attribute gradient is a scatter.
#include "uds_common.cuh"

namespace uds {

__global__ void k_interp_forward(int B, int W, int H, int K, const int* __restrict__ idx,
                                 const float* __restrict__ w, int aB, int N, int C,
                                 const float* __restrict__ attr, float* __restrict__ out) {
    size_t pix = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t P = (size_t)W * H;
    if (pix >= P * B) return;
    int b = (int)(pix / P);
    float acc[16];
    for (int c0 = 0; c0 < C; c0 += 16) {
        int cn = min(16, C - c0);
        for (int c = 0; c < cn; ++c) acc[c] = 0.0f;
        for (int s = 0; s < K; ++s) {
            size_t so = (size_t)s + (size_t)K * pix;
            int id = idx[so];
            if (id < 0 || id >= N) continue;
            float wt = w[so];
            const float* a = attr + (size_t)C * ((size_t)id + (aB > 1 ? (size_t)N * b : 0)) + c0;
            for (int c = 0; c < cn; ++c) acc[c] = fadd(acc[c], fmul(wt, a[c]));
        }
        for (int c = 0; c < cn; ++c) out[(size_t)C * pix + c0 + c] = acc[c];
    }
}

__global__ void k_interp_backward(int B, int W, int H, int K, const float* __restrict__ gin,
                                  const int* __restrict__ idx, const float* __restrict__ w, int aB,
                                  int N, int C, const float* __restrict__ attr,
                                  float* __restrict__ gw, float* __restrict__ ga) {
    size_t pix = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t P = (size_t)W * H;
    if (pix >= P * B) return;
    int b = (int)(pix / P);
    const float* g = gin + (size_t)C * pix;
    for (int s = 0; s < K; ++s) {
        size_t so = (size_t)s + (size_t)K * pix;
        int id = idx[so];
        if (id < 0 || id >= N) { gw[so] = 0.0f; continue; }
        float wt = w[so];
        size_t ao = (size_t)C * ((size_t)id + (aB > 1 ? (size_t)N * b : 0));
        float acc = 0.0f;
        for (int c = 0; c < C; ++c) {
            float gi = g[c];
            atomicAdd(&ga[ao + c], gi * wt);
            acc = fadd(acc, fmul(gi, attr[ao + c]));
        }
        gw[so] = acc;
    }
}

}  // namespace uds

using namespace uds;

extern "C" int uds_interp_forward(int B, int W, int H, int K, const int32_t* indices,
                                  const float* weights, int aB, int N, int C, const float* attribute,
                                  float* out, void* stream) {
    if (B <= 0 || W <= 0 || H <= 0 || K <= 0 || C <= 0 || N < 0 || (aB != 1 && aB != B)) return UDS_ERR_ARGUMENT;
    if (!indices || !weights || !out) return UDS_ERR_ARGUMENT;
    size_t total = (size_t)W * H * B;
    k_interp_forward<<<cdiv(total, 128), 128, 0, as_stream(stream)>>>(B, W, H, K, indices, weights, aB, N, C,
                                                                       attribute, out);
    return launch_status();
}

extern "C" int uds_interp_backward(int B, int W, int H, int K, const float* grad,
                                   const int32_t* indices, const float* weights, int aB, int N, int C,
                                   const float* attribute, float* grad_weights, float* grad_attribute,
                                   void* stream) {
    if (B <= 0 || W <= 0 || H <= 0 || K <= 0 || C <= 0 || N < 0 || (aB != 1 && aB != B)) return UDS_ERR_ARGUMENT;
    if (!grad || !indices || !weights || !grad_weights || (N > 0 && !grad_attribute)) return UDS_ERR_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    if (N > 0) {
        cudaError_t e = cudaMemsetAsync(grad_attribute, 0, sizeof(float) * (size_t)aB * N * C, s);
        if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    }
    size_t total = (size_t)W * H * B;
    k_interp_backward<<<cdiv(total, 128), 128, 0, s>>>(B, W, H, K, grad, indices, weights, aB, N, C, attribute,
                                                        grad_weights, grad_attribute);
    return launch_status();
}
