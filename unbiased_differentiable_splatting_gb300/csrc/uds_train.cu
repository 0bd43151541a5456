// Training-step tail, fused (optimization_geometry.py:190-219): the image
// loss with its gradient in one pass, and one Adam step over all splat
// parameters with the constraint projection of the reference's loop
// (normals renormalised, std-devs clamped to their bounds) in the same
// kernel, one thread per splat.
#include "uds_common.cuh"

namespace uds {

// L1 (kind 0) or L2 (kind 1) image loss: loss += scale * sum |x - y| (or
// (x - y)^2), grad = scale * d/dx (sign(x - y) or 2 (x - y)).
__global__ void k_image_loss(size_t n, int kind, const float* __restrict__ x, const float* __restrict__ y,
                             float scale, float* __restrict__ loss, float* __restrict__ grad) {
    __shared__ float red[8];
    float acc = 0.0f;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float d = x[i] - y[i];
        if (kind == 0) {
            acc += fabsf(d);
            grad[i] = scale * (d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f));
        } else {
            acc += d * d;
            grad[i] = scale * 2.0f * d;
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
        atomicAdd(loss, s * scale);
    }
}

__device__ __forceinline__ float adam_update(float p, float g, float& m, float& v, float lr, float b1, float b2,
                                             float eps, float bc1, float bc2) {
    m = b1 * m + (1.0f - b1) * g;
    v = b2 * v + (1.0f - b2) * g * g;
    float denom = sqrtf(v) / sqrtf(bc2) + eps;
    return p - (lr / bc1) * m / denom;
}

// One Adam step for splat s over its position (3), normal (3), colour (C) and
// std-dev (2) parameters; tensor t's moments are m[t], v[t] with the
// parameter's layout.  Then the normal is renormalised (x / (|x| + 1e-4),
// the reference's normalize) and the std-devs clamped to [lo, hi].
struct SplatTensors {
    float* p[4];
    const float* g[4];
    float* m[4];
    float* v[4];
    int width[4];
};

__global__ void k_adam_splats(int N, SplatTensors T, float lr, float b1, float b2, float eps, float bc1, float bc2,
                              float sd_lo, float sd_hi, int project) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    for (int t = 0; t < 4; ++t) {
        if (!T.p[t]) continue;
        int w = T.width[t];
        for (int c = 0; c < w; ++c) {
            size_t i = (size_t)s * w + c;
            float m = T.m[t][i], v = T.v[t][i];
            float p = adam_update(T.p[t][i], T.g[t] ? T.g[t][i] : 0.0f, m, v, lr, b1, b2, eps, bc1, bc2);
            T.m[t][i] = m;
            T.v[t][i] = v;
            if (project && t == 3) p = fminf(fmaxf(p, sd_lo), sd_hi);
            T.p[t][i] = p;
        }
    }
    if (project && T.p[1]) {
        float* n = T.p[1] + (size_t)s * 3;
        float len = sqrtf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]) + 1e-4f;
        n[0] /= len;
        n[1] /= len;
        n[2] /= len;
    }
}

}  // namespace uds

using namespace uds;

extern "C" int uds_image_loss(int kind, size_t n, const float* x, const float* y, float scale, float* loss,
                              float* grad, void* stream) {
    if ((kind != 0 && kind != 1) || !loss || (n > 0 && (!x || !y || !grad))) return UDS_ERR_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    cudaError_t e = cudaMemsetAsync(loss, 0, sizeof(float), s);
    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    if (n == 0) return UDS_OK;
    unsigned blocks = cdiv(n, 256);
    if (blocks > 4096) blocks = 4096;
    k_image_loss<<<blocks, 256, 0, s>>>(n, kind, x, y, scale, loss, grad);
    return launch_status();
}

extern "C" int uds_adam_splats(int N, float* points, const float* g_points, float* normals, const float* g_normals,
                               float* colors, const float* g_colors, int C, float* std_devs, const float* g_std_devs,
                               float* m, float* v, int step, float lr, float beta1, float beta2, float eps,
                               float sd_lo, float sd_hi, int project, void* stream) {
    if (N < 0 || C < 0 || step < 1 || !m || !v) return UDS_ERR_ARGUMENT;
    if (N == 0) return UDS_OK;
    SplatTensors T{};
    float* ps[4] = {points, normals, colors, std_devs};
    const float* gs[4] = {g_points, g_normals, g_colors, g_std_devs};
    int ws[4] = {3, 3, C, 2};
    size_t off = 0;
    for (int t = 0; t < 4; ++t) {
        T.p[t] = ws[t] > 0 ? ps[t] : nullptr;
        T.g[t] = gs[t];
        T.width[t] = ws[t];
        // moments of all four tensors packed in m / v: N*3, N*3, N*C, N*2
        T.m[t] = m + off;
        T.v[t] = v + off;
        off += (size_t)N * ws[t];
    }
    float bc1 = 1.0f - powf(beta1, (float)step), bc2 = 1.0f - powf(beta2, (float)step);
    k_adam_splats<<<cdiv(N, 128), 128, 0, as_stream(stream)>>>(N, T, lr, beta1, beta2, eps, bc1, bc2, sd_lo, sd_hi,
                                                               project);
    return launch_status();
}
