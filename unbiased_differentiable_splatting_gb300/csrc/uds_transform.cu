// Batched 4x4 affine / linear transform of splat vectors and its backward
// (transform.cpp:33-86, transformCuda.cu:11-117, transformation.cuh:8-27).
#include "uds_common.cuh"

namespace uds {

// Camera-space transform with the reference's summation order
// ((0 + m0 p0) + m1 p1) + m2 p2 (+ m3), exact rounding: the result feeds the
// bit-exact sampler.
template <bool Affine>
__global__ void k_transform_forward(int B, const float* __restrict__ M, int vB, int N,
                                    const float* __restrict__ v, float* __restrict__ out) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int b = blockIdx.y;
    if (x >= N) return;
    const float* T = M + 16 * b;
    const float* p = v + 3 * ((size_t)x + (vB > 1 ? (size_t)N * b : 0));
    float p0 = p[0], p1 = p[1], p2 = p[2];
    float* o = out + 3 * ((size_t)x + (size_t)N * b);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float s = fadd(fadd(fadd(0.0f, fmul(T[4 * i], p0)), fmul(T[4 * i + 1], p1)), fmul(T[4 * i + 2], p2));
        if (Affine) s = fadd(s, T[4 * i + 3]);
        o[i] = s;
    }
}

// gM[b] = sum_x g_x (v_x, 1)^T (row 3 stays zero); block-reduced then one
// atomic per entry and block.  gv[x] = sum_b M_b^T g_bx (loops over b when
// the vectors are broadcast, so no atomics on gv).
template <bool Affine>
__global__ void k_transform_backward(int B, const float* __restrict__ grad,
                                     const float* __restrict__ M, int vB, int N,
                                     const float* __restrict__ v, float* __restrict__ gM,
                                     float* __restrict__ gv) {
    __shared__ float red[12][32];
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int b = blockIdx.y;
    float acc[12];
#pragma unroll
    for (int i = 0; i < 12; ++i) acc[i] = 0.0f;
    if (x < N) {
        const float* g = grad + 3 * ((size_t)x + (size_t)N * b);
        const float* p = v + 3 * ((size_t)x + (vB > 1 ? (size_t)N * b : 0));
        float g0 = g[0], g1 = g[1], g2 = g[2];
        float gg[3] = {g0, g1, g2};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            acc[4 * i + 0] = gg[i] * p[0];
            acc[4 * i + 1] = gg[i] * p[1];
            acc[4 * i + 2] = gg[i] * p[2];
            acc[4 * i + 3] = Affine ? gg[i] : 0.0f;
        }
        if (vB > 1 || B == 1) {
            const float* T = M + 16 * b;
            float* o = gv + 3 * ((size_t)x + (vB > 1 ? (size_t)N * b : 0));
#pragma unroll
            for (int j = 0; j < 3; ++j) o[j] = g0 * T[j] + g1 * T[4 + j] + g2 * T[8 + j];
        } else if (b == 0) {
            float r[3] = {0.0f, 0.0f, 0.0f};
            for (int bb = 0; bb < B; ++bb) {
                const float* T = M + 16 * bb;
                const float* gb = grad + 3 * ((size_t)x + (size_t)N * bb);
#pragma unroll
                for (int j = 0; j < 3; ++j) r[j] += gb[0] * T[j] + gb[1] * T[4 + j] + gb[2] * T[8 + j];
            }
            float* o = gv + 3 * (size_t)x;
#pragma unroll
            for (int j = 0; j < 3; ++j) o[j] = r[j];
        }
    }
    // block reduction: warp shuffle, then across warps
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < 12; ++i) {
        float a = acc[i];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) red[i][warp] = a;
    }
    __syncthreads();
    if (threadIdx.x < 12) {
        float a = 0.0f;
        int nw = blockDim.x >> 5;
        for (int w = 0; w < nw; ++w) a += red[threadIdx.x][w];
        int i = threadIdx.x;
        if (Affine || (i & 3) != 3) atomicAdd(&gM[16 * b + i], a);
    }
}

// world2Camera (utils.py:11-49): quaternion (x, y, z, w) and position to the
// view matrix [R | t; 0 0 0 1], R by the Euler-Rodrigues formula, with every
// product and sum rounded as the reference's tensor operations round them
// (left to right), so the matrix is the same bit for bit.  One thread per
// view; the backward is the analytic derivative of R in the quaternion.
__global__ void k_view_matrix_forward(int B, const float* __restrict__ pos, const float* __restrict__ quat,
                                      float* __restrict__ M) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    float x = quat[4 * b], y = quat[4 * b + 1], z = quat[4 * b + 2], w = quat[4 * b + 3];
    float x2 = fmul(x, x), y2 = fmul(y, y), z2 = fmul(z, z), w2 = fmul(w, w);
    float xy = fmul(x, y), zw = fmul(z, w), xz = fmul(x, z), yw = fmul(y, w), yz = fmul(y, z), xw = fmul(x, w);
    float* m = M + 16 * (size_t)b;
    m[0] = fadd(fsub(fsub(x2, y2), z2), w2);
    m[1] = fmul(2.0f, fsub(xy, zw));
    m[2] = fmul(2.0f, fadd(xz, yw));
    m[3] = pos[3 * b];
    m[4] = fmul(2.0f, fadd(xy, zw));
    m[5] = fadd(fsub(fadd(-x2, y2), z2), w2);
    m[6] = fmul(2.0f, fsub(yz, xw));
    m[7] = pos[3 * b + 1];
    m[8] = fmul(2.0f, fsub(xz, yw));
    m[9] = fmul(2.0f, fadd(yz, xw));
    m[10] = fadd(fadd(fsub(-x2, y2), z2), w2);
    m[11] = pos[3 * b + 2];
    m[12] = 0.0f;
    m[13] = 0.0f;
    m[14] = 0.0f;
    m[15] = 1.0f;
}

__global__ void k_view_matrix_backward(int B, const float* __restrict__ G, const float* __restrict__ quat,
                                       float* __restrict__ gpos, float* __restrict__ gquat) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    float x = quat[4 * b], y = quat[4 * b + 1], z = quat[4 * b + 2], w = quat[4 * b + 3];
    const float* g = G + 16 * (size_t)b;
    gpos[3 * b] = g[3];
    gpos[3 * b + 1] = g[7];
    gpos[3 * b + 2] = g[11];
    // dR_ij / d(x, y, z, w), row-major i, j
    const float d[9][4] = {{2 * x, -2 * y, -2 * z, 2 * w}, {2 * y, 2 * x, -2 * w, -2 * z},
                           {2 * z, 2 * w, 2 * x, 2 * y},   {2 * y, 2 * x, 2 * w, 2 * z},
                           {-2 * x, 2 * y, -2 * z, 2 * w}, {-2 * w, 2 * z, 2 * y, -2 * x},
                           {2 * z, -2 * w, 2 * x, -2 * y}, {2 * w, 2 * z, 2 * y, 2 * x},
                           {-2 * x, -2 * y, 2 * z, 2 * w}};
    float gq[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int e = 0; e < 9; ++e) {
        float ge = g[4 * (e / 3) + e % 3];
#pragma unroll
        for (int k = 0; k < 4; ++k) gq[k] += ge * d[e][k];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) gquat[4 * b + k] = gq[k];
}

// BackfaceCulling (render.py:193-205): a splat whose camera-space normal
// points away from the camera (z > 0) gets its camera-space normal and, when
// given, its world normal negated; everything else is copied.  One thread per
// (view, splat); world normals (nB,N,3) with nB in {1, B}.
__global__ void k_backface_forward(int B, int N, const float* __restrict__ cam, int nB,
                                   const float* __restrict__ world, float* __restrict__ out_cam,
                                   float* __restrict__ out_world) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int b = blockIdx.y;
    if (x >= N) return;
    size_t o = 3 * ((size_t)x + (size_t)N * b);
    float c0 = cam[o], c1 = cam[o + 1], c2 = cam[o + 2];
    bool flip = c2 > 0.0f;
    out_cam[o] = flip ? -c0 : c0;
    out_cam[o + 1] = flip ? -c1 : c1;
    out_cam[o + 2] = flip ? -c2 : c2;
    if (world) {
        const float* w = world + 3 * ((size_t)x + (nB > 1 ? (size_t)N * b : 0));
#pragma unroll
        for (int k = 0; k < 3; ++k) out_world[o + k] = flip ? -w[k] : w[k];
    }
}

// Gradients of the flips: the camera-space one per (view, splat); the world
// one summed over the views in view order when the normals are shared.
__global__ void k_backface_backward(int B, int N, const float* __restrict__ cam, const float* __restrict__ g_cam,
                                    int nB, const float* __restrict__ g_world, float* __restrict__ gcam_out,
                                    float* __restrict__ gworld_out) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= N) return;
    float acc[3] = {0.0f, 0.0f, 0.0f};
    for (int b = 0; b < B; ++b) {
        size_t o = 3 * ((size_t)x + (size_t)N * b);
        float sgn = cam[o + 2] > 0.0f ? -1.0f : 1.0f;
        if (g_cam) {
#pragma unroll
            for (int k = 0; k < 3; ++k) gcam_out[o + k] = sgn * g_cam[o + k];
        }
        if (g_world) {
            if (nB > 1) {
#pragma unroll
                for (int k = 0; k < 3; ++k) gworld_out[o + k] = sgn * g_world[o + k];
            } else {
#pragma unroll
                for (int k = 0; k < 3; ++k) acc[k] += sgn * g_world[o + k];
            }
        }
    }
    if (g_world && nB == 1) {
#pragma unroll
        for (int k = 0; k < 3; ++k) gworld_out[3 * (size_t)x + k] = acc[k];
    }
}

}  // namespace uds

using namespace uds;

extern "C" int uds_backface_forward(int B, int N, const float* cam_normals, int nB, const float* normals,
                                    float* flipped_cam, float* flipped_normals, void* stream) {
    if (B <= 0 || N < 0 || (normals && nB != 1 && nB != B) || (N > 0 && (!cam_normals || !flipped_cam)) ||
        (normals && !flipped_normals))
        return UDS_ERR_ARGUMENT;
    if (N == 0) return UDS_OK;
    k_backface_forward<<<dim3(cdiv(N, 256), B), 256, 0, as_stream(stream)>>>(B, N, cam_normals, nB, normals,
                                                                             flipped_cam, flipped_normals);
    return launch_status();
}

extern "C" int uds_backface_backward(int B, int N, const float* cam_normals, const float* grad_flipped_cam, int nB,
                                     const float* grad_flipped_normals, float* grad_cam, float* grad_normals,
                                     void* stream) {
    if (B <= 0 || N < 0 || (grad_flipped_normals && nB != 1 && nB != B) || (N > 0 && !cam_normals) ||
        (grad_flipped_cam && !grad_cam) || (grad_flipped_normals && !grad_normals))
        return UDS_ERR_ARGUMENT;
    if (N == 0) return UDS_OK;
    k_backface_backward<<<cdiv(N, 256), 256, 0, as_stream(stream)>>>(B, N, cam_normals, grad_flipped_cam, nB,
                                                                     grad_flipped_normals, grad_cam, grad_normals);
    return launch_status();
}

extern "C" int uds_transform_forward(int affine, int B, const float* M, int vB, int N,
                                     const float* v, float* out, void* stream) {
    if (B <= 0 || N < 0 || (vB != 1 && vB != B) || !M || (N > 0 && (!v || !out))) return UDS_ERR_ARGUMENT;
    if (N == 0) return UDS_OK;
    dim3 grid(cdiv(N, 256), B);
    if (affine) k_transform_forward<true><<<grid, 256, 0, as_stream(stream)>>>(B, M, vB, N, v, out);
    else k_transform_forward<false><<<grid, 256, 0, as_stream(stream)>>>(B, M, vB, N, v, out);
    return launch_status();
}

extern "C" int uds_transform_backward(int affine, int B, const float* grad, const float* M, int vB,
                                      int N, const float* v, float* gM, float* gv, void* stream) {
    if (B <= 0 || N < 0 || (vB != 1 && vB != B) || !M || !gM || (N > 0 && (!grad || !v || !gv)))
        return UDS_ERR_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    cudaError_t e = cudaMemsetAsync(gM, 0, sizeof(float) * 16 * (size_t)B, s);
    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    if (N == 0) return UDS_OK;
    dim3 grid(cdiv(N, 256), B);
    if (affine) k_transform_backward<true><<<grid, 256, 0, s>>>(B, grad, M, vB, N, v, gM, gv);
    else k_transform_backward<false><<<grid, 256, 0, s>>>(B, grad, M, vB, N, v, gM, gv);
    return launch_status();
}

extern "C" int uds_view_matrix_forward(int B, const float* positions, const float* quaternions, float* matrices,
                                       void* stream) {
    if (B < 0 || (B > 0 && (!positions || !quaternions || !matrices))) return UDS_ERR_ARGUMENT;
    if (B == 0) return UDS_OK;
    k_view_matrix_forward<<<cdiv((size_t)B, 128), 128, 0, as_stream(stream)>>>(B, positions, quaternions, matrices);
    return launch_status();
}

extern "C" int uds_view_matrix_backward(int B, const float* grad, const float* quaternions, float* grad_positions,
                                        float* grad_quaternions, void* stream) {
    if (B < 0 || (B > 0 && (!grad || !quaternions || !grad_positions || !grad_quaternions))) return UDS_ERR_ARGUMENT;
    if (B == 0) return UDS_OK;
    k_view_matrix_backward<<<cdiv((size_t)B, 128), 128, 0, as_stream(stream)>>>(B, grad, quaternions,
                                                                                  grad_positions, grad_quaternions);
    return launch_status();
}
