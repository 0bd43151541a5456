// splatting.forward / splatting.backward (splatting.cpp:43-129,
// splattingCuda.cu:18-233) restructured for the GPU:
//   forward : per-splat Gaussian constants once (the part of the reference's
//             per-sample work that does not depend on the pixel), then one
//             thread per pixel evaluates its K samples;
//   backward: per sample only the sufficient statistics of the gradient
//             (sum g*G, sum g*G*d, sum g*G*d d^T, d = pixel - screen point)
//             are scattered, then one thread per splat applies the chain
//             rule through covariance, Jacobian, tangent plane and
//             projection once.  The reference instead runs the full chain
//             (ewaSplattingGrad.cuh:163-206) per sample and scatters 8 floats.
// The fused render kernels at the end of this file run EWA weights, depth
// compositing and attribute interpolation (and their backward passes) per
// pixel in one kernel each way.
#include "uds_composite.cuh"

namespace uds {

__global__ void k_ewa_consts(int B, int N, float W, float H, float f,
                             const float* __restrict__ pts, const float* __restrict__ nrm,
                             const float* __restrict__ sd, int sdB, float sm,
                             const unsigned char* __restrict__ used, float4* __restrict__ consts) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int b = blockIdx.y;
    if (x >= N) return;
    size_t o = (size_t)x + (size_t)N * b;
    if (!used[o]) return;  // no pixel of view b samples splat x
    float p[3] = {pts[3 * o], pts[3 * o + 1], pts[3 * o + 2]};
    float n[3] = {nrm[3 * o], nrm[3 * o + 1], nrm[3 * o + 2]};
    size_t so = sdB > 1 ? o : (size_t)x;
    float s[2] = {sd[2 * so], sd[2 * so + 1]};
    EwaFrame F;
    ewa_frame(W, H, f, p, n, s, sm, F);
    float4 a, c;
    ewa_gauss_consts(F, a, c);
    consts[2 * o] = a;
    consts[2 * o + 1] = c;
}

// Flag the (view, splat) pairs that some pixel samples: only those need the
// Gaussian constants (their frame takes double-precision divisions, which
// are slow on this GPU), and only those receive gradient, as in the
// reference, whose kernels visit sampled pairs only.
__global__ void k_ewa_mark(int B, int W, int H, int K, const int* __restrict__ idx, int N,
                           unsigned char* __restrict__ used) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y;
    int b = blockIdx.z;
    if (j >= H) return;
    size_t pix = (size_t)j + (size_t)H * ((size_t)i + (size_t)W * b);
    for (int s = 0; s < K; ++s) {
        int id = idx[(size_t)s + (size_t)K * pix];
        if (id >= 0 && id < N) used[(size_t)id + (size_t)N * b] = 1;
    }
}

// One thread per pixel (x = i, y = j), K samples.
__global__ void k_ewa_forward(int B, int W, int H, int K, const int* __restrict__ idx,
                              const float4* __restrict__ consts, int N, float* __restrict__ w) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y;
    int b = blockIdx.z;
    if (j >= H) return;
    size_t pix = (size_t)j + (size_t)H * ((size_t)i + (size_t)W * b);
    float px = (float)i, py = (float)j;
    for (int s = 0; s < K; ++s) {
        size_t off = (size_t)s + (size_t)K * pix;
        int id = idx[off];
        float out = 0.0f;
        if (id >= 0 && id < N) {
            size_t o = (size_t)id + (size_t)N * b;
            float4 a = consts[2 * o], c = consts[2 * o + 1];
            out = fminf(ewa_gauss(a, c, px, py), 1.0f);
        }
        w[off] = out;
    }
}

// Sufficient statistics of the EWA gradient, gated on the unclamped weight
// <= 1 like gradEwaKernel (splattingCuda.cu:173).
__global__ void k_ewa_stats(int B, int W, int H, int K, const float* __restrict__ grad,
                            const int* __restrict__ idx, const float4* __restrict__ consts, int N,
                            float4* __restrict__ stats) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y;
    int b = blockIdx.z;
    if (j >= H) return;
    size_t pix = (size_t)j + (size_t)H * ((size_t)i + (size_t)W * b);
    float px = (float)i, py = (float)j;
    for (int s = 0; s < K; ++s) {
        size_t off = (size_t)s + (size_t)K * pix;
        int id = idx[off];
        if (id < 0 || id >= N) continue;
        size_t o = (size_t)id + (size_t)N * b;
        float4 a = consts[2 * o], c = consts[2 * o + 1];
        float dx, dy;
        float G = ewa_gauss(a, c, px, py, &dx, &dy);
        if (!(G <= 1.0f)) continue;
        float g = grad[off] * G;
        if (g == 0.0f) continue;
        atomicAdd(&stats[2 * o], make_float4(g, g * dx, g * dy, g * dx * dx));
        atomicAdd(reinterpret_cast<float2*>(&stats[2 * o + 1]), make_float2(g * dx * dy, g * dy * dy));
    }
}

__device__ __forceinline__ void cross3(const float* a, const float* b, float* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ float dot3c(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// Reverse-mode chain of the EWA weight for one splat from its statistics.
__global__ void k_ewa_chain(int B, int N, float W, float H, float f, const float* __restrict__ pts,
                            const float* __restrict__ nrm, const float* __restrict__ sd, int sdB,
                            float sm, const float4* __restrict__ stats, float* __restrict__ gp_out,
                            float* __restrict__ gn_out, float* __restrict__ gs_out) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int b = blockIdx.y;
    if (x >= N) return;
    size_t o = (size_t)x + (size_t)N * b;
    float4 st0 = stats[2 * o], st1 = stats[2 * o + 1];
    float S0 = st0.x, S1x = st0.y, S1y = st0.z, S2xx = st0.w, S2xy = st1.x, S2yy = st1.y;
    size_t so = sdB > 1 ? o : (size_t)x;
    if (S0 == 0.0f && S1x == 0.0f && S1y == 0.0f && S2xx == 0.0f && S2xy == 0.0f && S2yy == 0.0f) {
        gp_out[3 * o] = 0.0f; gp_out[3 * o + 1] = 0.0f; gp_out[3 * o + 2] = 0.0f;
        gn_out[3 * o] = 0.0f; gn_out[3 * o + 1] = 0.0f; gn_out[3 * o + 2] = 0.0f;
        if (sdB > 1) { gs_out[2 * so] = 0.0f; gs_out[2 * so + 1] = 0.0f; }
        return;
    }
    float p[3] = {pts[3 * o], pts[3 * o + 1], pts[3 * o + 2]};
    float n[3] = {nrm[3 * o], nrm[3 * o + 1], nrm[3 * o + 2]};
    float sdv[2] = {sd[2 * so], sd[2 * so + 1]};
    // forward quantities (same sequence as the frame)
    float sp[2];
    screen_point(W, H, f, p, sp);
    float y0[2] = {add_via_double(sp[0], 1.0f), sp[1]};
    float y1[2] = {sp[0], add_via_double(sp[1], 1.0f)};
    float x0[3], x1[3], t0[3], t1[3];
    back_project(W, H, f, y0, x0);
    back_project(W, H, f, y1, x1);
    float c = dot3(p, n);
    float D0 = dot3(x0, n), D1 = dot3(x1, n);
    float k0 = fdiv(c, D0), k1 = fdiv(c, D1);
    tangent(x0, p, n, t0);
    tangent(x1, p, n, t1);
    float al = fsqrt(dot3(t0, t0));
    float invNorm = div_via_double(1.0f, al);
    float u0[3] = {t0[0] * invNorm, t0[1] * invNorm, t0[2] * invNorm};
    float u1[3];
    cross3(u0, n, u1);
    float be = dot3c(t1, u0), ga = dot3c(t1, u1);
    float J00 = 1.0f / al, J01 = -be / (al * ga), J11 = 1.0f / ga;
    float Sg0 = sdv[0] * sdv[0], Sg1 = sdv[1] * sdv[1];
    float V00 = J00 * J00 * Sg0 + J01 * J01 * Sg1 + sm;
    float V01 = J01 * J11 * Sg1;
    float V11 = J11 * J11 * Sg1 + sm;
    float vdet = V00 * V11 - V01 * V01;
    float I00 = V11 / vdet, I01 = -V01 / vdet, I11 = V00 / vdet;
    // moments of q = V^-1 d
    float M1x = I00 * S1x + I01 * S1y, M1y = I01 * S1x + I11 * S1y;
    float A00 = I00 * S2xx + I01 * S2xy, A01 = I00 * S2xy + I01 * S2yy;
    float A10 = I01 * S2xx + I11 * S2xy, A11 = I01 * S2xy + I11 * S2yy;
    float Q00 = A00 * I00 + A01 * I01, Q01 = A00 * I01 + A01 * I11, Q11 = A10 * I01 + A11 * I11;
    float gV00 = 0.5f * (Q00 - S0 * I00), gV01 = 0.5f * (Q01 - S0 * I01), gV11 = 0.5f * (Q11 - S0 * I11);
    float gJ00 = 2.0f * (gV00 * J00 * Sg0);
    float gJ01 = 2.0f * (gV00 * J01 * Sg1 + gV01 * J11 * Sg1);
    float gJ11 = 2.0f * (gV01 * J01 * Sg1 + gV11 * J11 * Sg1);
    float gsd0 = 2.0f * sdv[0] * (J00 * J00 * gV00);
    float gsd1 = 2.0f * sdv[1] * (J01 * J01 * gV00 + 2.0f * J01 * J11 * gV01 + J11 * J11 * gV11);
    float gal = -gJ00 / (al * al) + gJ01 * be / (al * al * ga) - S0 / al;
    float gbe = -gJ01 / (al * ga);
    float gga = gJ01 * be / (al * ga * ga) - gJ11 / (ga * ga) - S0 / ga;
    float nxt1[3], t1xu0[3], gt1[3], gu0[3], gnv[3];
    cross3(n, t1, nxt1);
    cross3(t1, u0, t1xu0);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        gt1[i] = gbe * u0[i] + gga * u1[i];
        gu0[i] = gbe * t1[i] + gga * nxt1[i];
        gnv[i] = gga * t1xu0[i];
    }
    float gdu = dot3c(gu0, u0), gt0[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) gt0[i] = (gu0[i] - gdu * u0[i]) / al + gal * u0[i];
    float gpv[3] = {-gt0[0] - gt1[0], -gt0[1] - gt1[1], -gt0[2] - gt1[2]};
    float gk0 = dot3c(gt0, x0), gk1 = dot3c(gt1, x1);
    float gc = gk0 / D0 + gk1 / D1;
    float gD0 = -gk0 * c / (D0 * D0), gD1 = -gk1 * c / (D1 * D1);
    float gx00 = k0 * gt0[0] + gD0 * n[0], gx01 = k0 * gt0[1] + gD0 * n[1];
    float gx10 = k1 * gt1[0] + gD1 * n[0], gx11 = k1 * gt1[1] + gD1 * n[1];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        gnv[i] += gD0 * x0[i] + gD1 * x1[i] + gc * p[i];
        gpv[i] += gc * n[i];
    }
    float gS0 = M1x - (gx00 + gx10) / f;
    float gS1 = M1y + (gx01 + gx11) / f;
    float iz = 1.0f / p[2];
    gpv[0] += gS0 * (-f * iz);
    gpv[1] += gS1 * (f * iz);
    gpv[2] += (gS0 * p[0] - gS1 * p[1]) * f * iz * iz;
    gp_out[3 * o] = gpv[0]; gp_out[3 * o + 1] = gpv[1]; gp_out[3 * o + 2] = gpv[2];
    gn_out[3 * o] = gnv[0]; gn_out[3 * o + 1] = gnv[1]; gn_out[3 * o + 2] = gnv[2];
    if (sdB > 1) {
        gs_out[2 * so] = gsd0;
        gs_out[2 * so + 1] = gsd1;
    } else {
        atomicAdd(&gs_out[2 * so], gsd0);
        atomicAdd(&gs_out[2 * so + 1], gsd1);
    }
}

// ----------------------------------------------------- fused render pass
// One thread per pixel runs splatting.forward, filtering.forward and
// interpolation.forward on its K samples (splattingCuda.cu:18-66,
// zSortingCuda.cu:11-62, interpolationCuda.cu:5-46): EWA weight of each
// sample from its pair's Gaussian constants, depth along the pixel ray,
// stable depth order, front-to-back blend, and the blended attributes.  The
// same device functions in the same order as the three separate kernels, so
// weights, depth weights and image are bit-identical to them; the (B,W,H,K)
// intermediates are written once (the autograd needs them) and never read
// back.
constexpr int kRenderThreads = 64;

template <int KMAX>
__global__ void __launch_bounds__(kRenderThreads) k_render_forward(
    int B, int W, int H, int K, const int* __restrict__ idx, const float4* __restrict__ consts, int N, float f,
    const float* __restrict__ pts, const float* __restrict__ nrm, int aB, int C, const float* __restrict__ attr,
    float* __restrict__ w_out, float* __restrict__ dw_out, float* __restrict__ img) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y, b = blockIdx.z;
    if (j >= H) return;
    size_t pix = (size_t)j + (size_t)H * ((size_t)i + (size_t)W * b);
    size_t e = (size_t)K * pix;
    float px = (float)i, py = (float)j;
    const float* bp = pts + 3 * (size_t)N * b;
    const float* bn = nrm + 3 * (size_t)N * b;
    float dir[3];
    pixel_ray((float)W, (float)H, f, px, py, dir);
    int id[KMAX], ord[KMAX];
    float wl[KMAX], dist[KMAX], fw[KMAX];
    for (int k = 0; k < K; ++k) {
        int s = idx[e + k];
        bool ok = s >= 0 && s < N;
        id[k] = ok ? s : -1;
        float wv = 0.0f;
        if (ok) {
            size_t o = (size_t)s + (size_t)N * b;
            wv = fminf(ewa_gauss(consts[2 * o], consts[2 * o + 1], px, py), 1.0f);
        }
        wl[k] = wv;
        w_out[e + k] = wv;
        dist[k] = sample_depth(dir, bp, bn, s, N);
    }
    depth_order<KMAX>(K, dist, ord);
    blend<KMAX>(K, ord, wl, fw);
    for (int k = 0; k < K; ++k) dw_out[e + k] = fw[k];
    const size_t aoff = aB > 1 ? (size_t)N * b : 0;
    for (int c0 = 0; c0 < C; c0 += 4) {
        int cn = min(4, C - c0);
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int k = 0; k < K; ++k) {
            if (id[k] < 0) continue;
            const float* a = attr + (size_t)C * ((size_t)id[k] + aoff) + c0;
#pragma unroll
            for (int c = 0; c < 4; ++c)
                if (c < cn) acc[c] = fadd(acc[c], fmul(fw[k], a[c]));
        }
#pragma unroll
        for (int c = 0; c < 4; ++c)
            if (c < cn) img[(size_t)C * pix + c0 + c] = acc[c];
    }
}

// The backward of the fused pass per pixel: interpolation.backward (weight
// gradient per sample, attribute gradient scattered), plus any gradient that
// reaches the depth weights directly; filtering.backward through the
// recomputed depth order and blend; and the EWA gradient statistics of
// k_ewa_stats (gated on the unclamped weight <= 1), plus any gradient that
// reaches the EWA weights directly.  k_ewa_chain then finishes the splat
// gradients.  Same arithmetic per sample as the separate kernels; the
// scattered sums are atomic, as there.
template <int KMAX>
__global__ void __launch_bounds__(kRenderThreads) k_render_backward(
    int B, int W, int H, int K, const float* __restrict__ gimg, const float* __restrict__ gdw_in,
    const float* __restrict__ gw_in, const int* __restrict__ idx, const float* __restrict__ w,
    const float4* __restrict__ consts, int N, float f, const float* __restrict__ pts, const float* __restrict__ nrm,
    int aB, int C, const float* __restrict__ attr, float* __restrict__ ga, float4* __restrict__ stats) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y, b = blockIdx.z;
    if (j >= H) return;
    size_t pix = (size_t)j + (size_t)H * ((size_t)i + (size_t)W * b);
    size_t e = (size_t)K * pix;
    float px = (float)i, py = (float)j;
    const float* bp = pts + 3 * (size_t)N * b;
    const float* bn = nrm + 3 * (size_t)N * b;
    float dir[3];
    pixel_ray((float)W, (float)H, f, px, py, dir);
    int id[KMAX], ord[KMAX];
    float wl[KMAX], dist[KMAX], fw[KMAX], gd[KMAX];
    for (int k = 0; k < K; ++k) {
        int s = idx[e + k];
        id[k] = (s >= 0 && s < N) ? s : -1;
        wl[k] = w[e + k];
        dist[k] = sample_depth(dir, bp, bn, s, N);
    }
    depth_order<KMAX>(K, dist, ord);
    blend<KMAX>(K, ord, wl, fw);
    // interpolation.backward with the depth weights fw
    const float* g = gimg + (size_t)C * pix;
    const size_t aoff = aB > 1 ? (size_t)N * b : 0;
    for (int k = 0; k < K; ++k) {
        float acc = 0.0f;
        if (id[k] >= 0) {
            size_t ao = (size_t)C * ((size_t)id[k] + aoff);
            for (int c = 0; c < C; ++c) {
                float gi = g[c];
                atomicAdd(&ga[ao + c], gi * fw[k]);
                acc = fadd(acc, fmul(gi, attr[ao + c]));
            }
        }
        gd[k] = gdw_in ? fadd(acc, gdw_in[e + k]) : acc;
    }
    // filtering.backward, then the EWA statistics in sample order
    float ge[KMAX];
    for (int k = 0; k < K; ++k) ge[ord[k]] = blend_grad<KMAX>(K, k, ord, wl, fw, gd);
    for (int k = 0; k < K; ++k) {
        if (id[k] < 0) continue;
        size_t o = (size_t)id[k] + (size_t)N * b;
        float dx, dy;
        float G = ewa_gauss(consts[2 * o], consts[2 * o + 1], px, py, &dx, &dy);
        if (!(G <= 1.0f)) continue;
        float gk = gw_in ? fadd(ge[k], gw_in[e + k]) : ge[k];
        float gg = gk * G;
        if (gg == 0.0f) continue;
        atomicAdd(&stats[2 * o], make_float4(gg, gg * dx, gg * dy, gg * dx * dx));
        atomicAdd(reinterpret_cast<float2*>(&stats[2 * o + 1]), make_float2(gg * dx * dy, gg * dy * dy));
    }
}

}  // namespace uds

using namespace uds;

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Workspace: Gaussian constants (2 float4 per pair), gradient statistics (2
// float4 per pair), one flag byte per pair.
extern "C" size_t uds_splat_workspace_size(int B, int N) {
    return align256(sizeof(float4) * 2 * (size_t)B * N) * 2 + align256((size_t)B * N);
}

static int check_splat_args(int B, int W, int H, int K, int std_batch, int N) {
    if (B <= 0 || W <= 0 || H <= 0 || K <= 0 || N < 0) return UDS_ERR_ARGUMENT;
    if (std_batch != 1 && std_batch != B) return UDS_ERR_ARGUMENT;
    return UDS_OK;
}

extern "C" int uds_splat_forward(int B, int W, int H, int K, float focal, const int32_t* indices,
                                 const float* points, const float* normals, int std_batch, int N,
                                 const float* std_devs, float smoothing, float* weights,
                                 void* workspace, size_t workspace_bytes, void* stream) {
    int st = check_splat_args(B, W, H, K, std_batch, N);
    if (st) return st;
    if (!indices || !weights) return UDS_ERR_ARGUMENT;
    if (workspace_bytes < uds_splat_workspace_size(B, N) || (N > 0 && !workspace)) return UDS_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    float4* consts = reinterpret_cast<float4*>(workspace);
    if (N > 0) {
        unsigned char* used = reinterpret_cast<unsigned char*>(workspace) +
                              2 * align256(sizeof(float4) * 2 * (size_t)B * N);
        cudaError_t e = cudaMemsetAsync(used, 0, (size_t)B * N, s);
        if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
        k_ewa_mark<<<dim3(cdiv(H, 64), W, B), 64, 0, s>>>(B, W, H, K, indices, N, used);
        k_ewa_consts<<<dim3(cdiv(N, 128), B), 128, 0, s>>>(B, N, (float)W, (float)H, focal, points, normals,
                                                          std_devs, std_batch, smoothing, used, consts);
        if ((st = launch_status(2))) return st;
    }
    k_ewa_forward<<<dim3(cdiv(H, 64), W, B), 64, 0, s>>>(B, W, H, K, indices, consts, N, weights);
    return launch_status();
}

extern "C" int uds_splat_backward(int B, int W, int H, int K, float focal, const float* grad,
                                  const int32_t* indices, const float* points, const float* normals,
                                  int std_batch, int N, const float* std_devs, float smoothing,
                                  float* grad_points, float* grad_normals, float* grad_std_devs,
                                  void* workspace, size_t workspace_bytes, void* stream) {
    int st = check_splat_args(B, W, H, K, std_batch, N);
    if (st) return st;
    if (!grad || !indices) return UDS_ERR_ARGUMENT;
    if (workspace_bytes < uds_splat_workspace_size(B, N) || (N > 0 && !workspace)) return UDS_ERR_WORKSPACE;
    if (N == 0) return UDS_OK;
    cudaStream_t s = as_stream(stream);
    float4* consts = reinterpret_cast<float4*>(workspace);
    float4* stats = reinterpret_cast<float4*>(reinterpret_cast<char*>(workspace) +
                                              align256(sizeof(float4) * 2 * (size_t)B * N));
    cudaError_t e = cudaMemsetAsync(stats, 0, sizeof(float4) * 2 * (size_t)B * N, s);
    if (e == cudaSuccess && std_batch == 1)
        e = cudaMemsetAsync(grad_std_devs, 0, sizeof(float) * 2 * (size_t)N, s);
    unsigned char* used = reinterpret_cast<unsigned char*>(workspace) +
                          2 * align256(sizeof(float4) * 2 * (size_t)B * N);
    if (e == cudaSuccess) e = cudaMemsetAsync(used, 0, (size_t)B * N, s);
    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    k_ewa_mark<<<dim3(cdiv(H, 64), W, B), 64, 0, s>>>(B, W, H, K, indices, N, used);
    k_ewa_consts<<<dim3(cdiv(N, 128), B), 128, 0, s>>>(B, N, (float)W, (float)H, focal, points, normals,
                                                      std_devs, std_batch, smoothing, used, consts);
    if ((st = launch_status(2))) return st;
    k_ewa_stats<<<dim3(cdiv(H, 64), W, B), 64, 0, s>>>(B, W, H, K, grad, indices, consts, N, stats);
    if ((st = launch_status())) return st;
    k_ewa_chain<<<dim3(cdiv(N, 128), B), 128, 0, s>>>(B, N, (float)W, (float)H, focal, points, normals,
                                                     std_devs, std_batch, smoothing, stats, grad_points,
                                                     grad_normals, grad_std_devs);
    return launch_status();
}

#define UDS_RENDER_DISPATCH(KERNEL, ...)                                               \
    do {                                                                                 \
        dim3 grid(cdiv(H, kRenderThreads), W, B);                                        \
        if (K <= 8) KERNEL<8><<<grid, kRenderThreads, 0, s>>>(__VA_ARGS__);              \
        else if (K <= 16) KERNEL<16><<<grid, kRenderThreads, 0, s>>>(__VA_ARGS__);       \
        else if (K <= 32) KERNEL<32><<<grid, kRenderThreads, 0, s>>>(__VA_ARGS__);       \
        else KERNEL<64><<<grid, kRenderThreads, 0, s>>>(__VA_ARGS__);                    \
    } while (0)

// Sampled-pair flags and Gaussian constants in the splat workspace (the
// first step of uds_splat_forward / backward).
static int render_consts(int B, int W, int H, int K, float focal, const int32_t* indices, const float* points,
                         const float* normals, int std_batch, int N, const float* std_devs, float smoothing,
                         void* workspace, cudaStream_t s) {
    float4* consts = reinterpret_cast<float4*>(workspace);
    unsigned char* used = reinterpret_cast<unsigned char*>(workspace) + 2 * align256(sizeof(float4) * 2 * (size_t)B * N);
    cudaError_t e = cudaMemsetAsync(used, 0, (size_t)B * N, s);
    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    k_ewa_mark<<<dim3(cdiv(H, 64), W, B), 64, 0, s>>>(B, W, H, K, indices, N, used);
    k_ewa_consts<<<dim3(cdiv(N, 128), B), 128, 0, s>>>(B, N, (float)W, (float)H, focal, points, normals, std_devs,
                                                      std_batch, smoothing, used, consts);
    return launch_status(2);
}

extern "C" int uds_render_fused_forward(int B, int W, int H, int K, float focal, const int32_t* indices,
                                        const float* points, const float* normals, int std_batch, int N,
                                        const float* std_devs, float smoothing, int aB, int C,
                                        const float* attribute, float* weights, float* depth_weights, float* image,
                                        void* workspace, size_t workspace_bytes, void* stream) {
    int st = check_splat_args(B, W, H, K, std_batch, N);
    if (st) return st;
    if (K > kMaxK || C <= 0 || (aB != 1 && aB != B) || !indices || !weights || !depth_weights || !image ||
        (N > 0 && (!points || !normals || !std_devs || !attribute)))
        return UDS_ERR_ARGUMENT;
    if (workspace_bytes < uds_splat_workspace_size(B, N) || (N > 0 && !workspace)) return UDS_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    if (N > 0 && (st = render_consts(B, W, H, K, focal, indices, points, normals, std_batch, N, std_devs, smoothing,
                                     workspace, s)))
        return st;
    const float4* consts = reinterpret_cast<const float4*>(workspace);
    UDS_RENDER_DISPATCH(k_render_forward, B, W, H, K, indices, consts, N, focal, points, normals, aB, C, attribute,
                        weights, depth_weights, image);
    return launch_status();
}

extern "C" int uds_render_fused_backward(int B, int W, int H, int K, float focal, const float* grad_image,
                                         const float* grad_depth_weights, const float* grad_weights,
                                         const int32_t* indices, const float* weights, const float* points,
                                         const float* normals, int std_batch, int N, const float* std_devs,
                                         float smoothing, int aB, int C, const float* attribute, float* grad_points,
                                         float* grad_normals, float* grad_std_devs, float* grad_attribute,
                                         void* workspace, size_t workspace_bytes, void* stream) {
    int st = check_splat_args(B, W, H, K, std_batch, N);
    if (st) return st;
    if (K > kMaxK || C <= 0 || (aB != 1 && aB != B) || !grad_image || !indices || !weights) return UDS_ERR_ARGUMENT;
    if (N > 0 && (!points || !normals || !std_devs || !attribute || !grad_points || !grad_normals || !grad_std_devs ||
                  !grad_attribute))
        return UDS_ERR_ARGUMENT;
    if (workspace_bytes < uds_splat_workspace_size(B, N) || (N > 0 && !workspace)) return UDS_ERR_WORKSPACE;
    if (N == 0) return UDS_OK;
    cudaStream_t s = as_stream(stream);
    float4* stats = reinterpret_cast<float4*>(reinterpret_cast<char*>(workspace) +
                                              align256(sizeof(float4) * 2 * (size_t)B * N));
    cudaError_t e = cudaMemsetAsync(stats, 0, sizeof(float4) * 2 * (size_t)B * N, s);
    if (e == cudaSuccess && std_batch == 1) e = cudaMemsetAsync(grad_std_devs, 0, sizeof(float) * 2 * (size_t)N, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(grad_attribute, 0, sizeof(float) * (size_t)aB * N * C, s);
    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    if ((st = render_consts(B, W, H, K, focal, indices, points, normals, std_batch, N, std_devs, smoothing, workspace,
                            s)))
        return st;
    const float4* consts = reinterpret_cast<const float4*>(workspace);
    UDS_RENDER_DISPATCH(k_render_backward, B, W, H, K, grad_image, grad_depth_weights, grad_weights, indices, weights,
                        consts, N, focal, points, normals, aB, C, attribute, grad_attribute, stats);
    if ((st = launch_status())) return st;
    k_ewa_chain<<<dim3(cdiv(N, 128), B), 128, 0, s>>>(B, N, (float)W, (float)H, focal, points, normals, std_devs,
                                                     std_batch, smoothing, stats, grad_points, grad_normals,
                                                     grad_std_devs);
    return launch_status();
}
