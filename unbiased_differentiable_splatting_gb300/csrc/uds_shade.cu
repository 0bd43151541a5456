// shading.forward / backward / forwardSh / backwardSh (shading.cpp:51-199,
// shadingCuda.cu:12-330, diffuseShading.cuh, diffuseShadingGrad.cuh):
// deferred Lambert with L directional lights and deferred order-2 spherical
// harmonics irradiance (Ramamoorthi & Hanrahan 2001) on per-pixel normals and
// albedo.  Light and coefficient gradients are reduced within the warp first
// and then added with one atomic per warp.
#include "uds_common.cuh"

namespace uds {

constexpr int kShadeThreads = 128;

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void k_shade_forward(int B, int P, int L, const float* __restrict__ dirs,
                                const float* __restrict__ I, int IB, const float* __restrict__ nrm,
                                const float* __restrict__ dif, float* __restrict__ out) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)P * B) return;
    int b = (int)(t / P);
    const float* n = nrm + 3 * t;
    const float* d = dif + 3 * t;
    float r[3] = {0.0f, 0.0f, 0.0f};
    for (int l = 0; l < L; ++l) {
        const float* dir = dirs + 3 * ((size_t)l + (size_t)L * b);
        const float* col = I + 3 * ((size_t)l + (IB > 1 ? (size_t)L * b : 0));
        float cs = fadd(fadd(fadd(0.0f, fmul(dir[0], n[0])), fmul(dir[1], n[1])), fmul(dir[2], n[2]));
        cs = fmaxf(0.0f, cs);
#pragma unroll
        for (int i = 0; i < 3; ++i)
            r[i] = fadd(r[i], (float)dmul(dmul(ddiv((double)d[i], kPi), (double)col[i]), (double)cs));
    }
    out[3 * t] = r[0]; out[3 * t + 1] = r[1]; out[3 * t + 2] = r[2];
}

// Light gradients (dirs: B*L*3, intensities: IB*L*3) accumulate across
// pixels; normals / diffuse gradients are per pixel.
__global__ void k_shade_backward(int B, int P, int L, const float* __restrict__ gin,
                                 const float* __restrict__ dirs, const float* __restrict__ I, int IB,
                                 const float* __restrict__ nrm, const float* __restrict__ dif,
                                 float* __restrict__ gdirs, float* __restrict__ gI,
                                 float* __restrict__ gn, float* __restrict__ gd) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool live = t < (size_t)P * B;
    // all lanes of a warp belong to the same view when P is a multiple of 32;
    // otherwise fall back to per-lane atomics
    int b = live ? (int)(t / P) : 0;
    int b0 = __shfl_sync(0xffffffffu, b, 0);
    bool uniform = __all_sync(0xffffffffu, !live || b == b0);
    const float pif = (float)kPi;
    float n[3] = {0, 0, 0}, d[3] = {0, 0, 0}, g[3] = {0, 0, 0}, an[3] = {0, 0, 0}, ad[3] = {0, 0, 0};
    if (live) {
#pragma unroll
        for (int i = 0; i < 3; ++i) { n[i] = nrm[3 * t + i]; d[i] = dif[3 * t + i]; g[i] = gin[3 * t + i]; }
    }
    for (int l = 0; l < L; ++l) {
        float gdir[3] = {0, 0, 0}, gcol[3] = {0, 0, 0};
        if (live) {
            const float* dir = dirs + 3 * ((size_t)l + (size_t)L * b);
            const float* col = I + 3 * ((size_t)l + (IB > 1 ? (size_t)L * b : 0));
            float cs = 0.0f, dc[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) { cs += dir[i] * n[i]; dc[i] = d[i] * col[i]; }
            if (cs > 0.0f) {
                float scaling = (float)((double)cs / kPi);
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    float a = 0.0f, c = 0.0f;
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        a += g[i] * ((dc[i] * n[j]) / pif);
                        c += g[i] * ((dc[i] * dir[j]) / pif);
                    }
                    gdir[j] = a;
                    an[j] += c;
                    gcol[j] = g[j] * (d[j] * scaling);
                    ad[j] += g[j] * (col[j] * scaling);
                }
            }
        }
        size_t dl = 3 * ((size_t)l + (size_t)L * b);
        size_t il = 3 * ((size_t)l + (IB > 1 ? (size_t)L * b : 0));
        if (uniform) {
#pragma unroll
            for (int j = 0; j < 3; ++j) { gdir[j] = warp_sum(gdir[j]); gcol[j] = warp_sum(gcol[j]); }
            if ((threadIdx.x & 31) == 0 && b0 < B) {
                size_t dl0 = 3 * ((size_t)l + (size_t)L * b0);
                size_t il0 = 3 * ((size_t)l + (IB > 1 ? (size_t)L * b0 : 0));
#pragma unroll
                for (int j = 0; j < 3; ++j) { atomicAdd(&gdirs[dl0 + j], gdir[j]); atomicAdd(&gI[il0 + j], gcol[j]); }
            }
        } else if (live) {
#pragma unroll
            for (int j = 0; j < 3; ++j) { atomicAdd(&gdirs[dl + j], gdir[j]); atomicAdd(&gI[il + j], gcol[j]); }
        }
    }
    if (live) {
#pragma unroll
        for (int j = 0; j < 3; ++j) { gn[3 * t + j] = an[j]; gd[3 * t + j] = ad[j]; }
    }
}

// buildShMatrix (diffuseShading.cuh:39-71); M(i,j) = m[4i+j]
__device__ __forceinline__ void sh_matrix(const float* c, float* M) {
    const float c1 = 0.429043f, c2 = 0.511664f, c3 = 0.743125f, c4 = 0.886227f, c5 = 0.247708f;
    M[0] = c1 * c[8]; M[4] = c1 * c[4]; M[8] = c1 * c[7]; M[12] = c2 * c[3];
    M[1] = c1 * c[4]; M[5] = -c1 * c[8]; M[9] = c1 * c[5]; M[13] = c2 * c[1];
    M[2] = c1 * c[7]; M[6] = c1 * c[5]; M[10] = c3 * c[6]; M[14] = c2 * c[2];
    M[3] = c2 * c[3]; M[7] = c2 * c[1]; M[11] = c2 * c[2]; M[15] = fsub(fmul(c4, c[0]), fmul(c5, c[6]));
}

__device__ __forceinline__ float sh_unit(const float* n, float* v) {
    float norm = fsqrt(fadd(fadd(fadd(0.0f, fmul(n[0], n[0])), fmul(n[1], n[1])), fmul(n[2], n[2])));
    v[0] = 0.0f; v[1] = 0.0f; v[2] = 0.0f; v[3] = 1.0f;
    if (norm > 1e-5f) {
        float inv = div_via_double(1.0f, norm);
        v[0] = fmul(n[0], inv); v[1] = fmul(n[1], inv); v[2] = fmul(n[2], inv); v[3] = fmul(norm, inv);
    }
    return norm;
}

__device__ __forceinline__ float sh_quad(const float* M, const float* v) {
    float r = 0.0f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float y = 0.0f;
#pragma unroll
        for (int j = 0; j < 4; ++j) y = fadd(y, fmul(v[j], M[4 * j + i]));
        r = fadd(r, fmul(y, v[i]));
    }
    return r;
}

__global__ void k_shade_sh_forward(int B, int P, const float* __restrict__ coef, int cB,
                                   const float* __restrict__ nrm, const float* __restrict__ dif,
                                   float* __restrict__ out) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)P * B) return;
    int b = (int)(t / P);
    float n[3] = {nrm[3 * t], nrm[3 * t + 1], nrm[3 * t + 2]}, v[4];
    sh_unit(n, v);
    for (int i = 0; i < 3; ++i) {
        float M[16];
        sh_matrix(coef + (cB > 1 ? 9 * (i + 3 * b) : 9 * i), M);
        out[3 * t + i] = (float)ddiv((double)fmul(dif[3 * t + i], sh_quad(M, v)), kPi);
    }
}

// shadingShBackwardKernel (shadingCuda.cu:244-293): channel i's normal
// gradient keeps only component i of that channel's gradient.
__global__ void k_shade_sh_backward(int B, int P, const float* __restrict__ gin,
                                    const float* __restrict__ coef, int cB,
                                    const float* __restrict__ nrm, const float* __restrict__ dif,
                                    float* __restrict__ gc, float* __restrict__ gn,
                                    float* __restrict__ gd) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool live = t < (size_t)P * B;
    int b = live ? (int)(t / P) : 0;
    int b0 = __shfl_sync(0xffffffffu, b, 0);
    bool uniform = __all_sync(0xffffffffu, !live || b == b0);
    const float c1 = 0.429043f, c2 = 0.511664f, c3 = 0.743125f, c4 = 0.886227f, c5 = 0.247708f;
    float n[3] = {0, 0, 0}, v[4] = {0, 0, 0, 1}, norm = 0.0f;
    if (live) {
        n[0] = nrm[3 * t]; n[1] = nrm[3 * t + 1]; n[2] = nrm[3 * t + 2];
        norm = sh_unit(n, v);
    }
    for (int i = 0; i < 3; ++i) {
        float gsh[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        size_t co = cB > 1 ? 9 * (i + 3 * b) : 9 * i;
        if (live) {
            float M[16];
            sh_matrix(coef + co, M);
            float irr = sh_quad(M, v);
            float gv[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                float a = 0.0f, tt = 0.0f;
#pragma unroll
                for (int j = 0; j < 4; ++j) { a += M[4 * r + j] * v[j]; tt += M[4 * j + r] * v[j]; }
                gv[r] = a + tt;
            }
            float gM[16];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int j = 0; j < 4; ++j) gM[4 * r + j] = v[r] * v[j];
            float g = gin[3 * t + i], dd = dif[3 * t + i];
            float s = g * dd / (float)kPi;
            gsh[0] = s * (c4 * gM[15]);
            gsh[1] = s * (c2 * (gM[7] + gM[13]));
            gsh[2] = s * (c2 * (gM[14] + gM[11]));
            gsh[3] = s * (c2 * (gM[12] + gM[3]));
            gsh[4] = s * (c1 * (gM[4] + gM[1]));
            gsh[5] = s * (c1 * (gM[9] + gM[6]));
            gsh[6] = s * (c3 * gM[10] - c5 * gM[15]);
            gsh[7] = s * (c1 * (gM[8] + gM[2]));
            gsh[8] = s * (c1 * (gM[0] - gM[5]));
            float gni = 0.0f;
            if (norm > 1e-5f) {
                float inv = (float)(1.0 / (double)norm);
                float inv3 = inv * inv * inv;
#pragma unroll
                for (int j = 0; j < 3; ++j) gni += (((i == j) ? inv : 0.0f) - n[i] * n[j] * inv3) * gv[j];
            }
            gd[3 * t + i] = (float)((double)(g * irr) / kPi);
            gn[3 * t + i] = (float)((double)(g * dd * gni) / kPi);
        }
        if (uniform) {
#pragma unroll
            for (int j = 0; j < 9; ++j) gsh[j] = warp_sum(gsh[j]);
            if ((threadIdx.x & 31) == 0) {
                size_t co0 = cB > 1 ? 9 * (i + 3 * b0) : 9 * i;
#pragma unroll
                for (int j = 0; j < 9; ++j) atomicAdd(&gc[co0 + j], gsh[j]);
            }
        } else if (live) {
#pragma unroll
            for (int j = 0; j < 9; ++j) atomicAdd(&gc[co + j], gsh[j]);
        }
    }
}

// Per-splat Lambert of the forward shading mode (shading.py:12-29, a chain
// of broadcasting tensor operations in the reference), fused:
//   out = ambient * d + sum_l (I_l * clamp(<dir_l, n>, 0, 1)) * (d / pi)
// with normals (B, N, 3), diffuse d (dB, N, 3), dirs (B, L, 3), intensities
// (IB, L, 3), ambient (aB, 3); dB, IB, aB are 1 or B.  Each product and sum
// is rounded as the tensor operations round it (the division by pi is a
// multiplication by the float reciprocal, as PyTorch divides by a scalar).
constexpr int kLambertMaxL = 4;
constexpr float kInvPiF = (float)(1.0 / kPi);

__global__ void k_lambert_forward(int B, int N, int L, const float* __restrict__ amb, int aB,
                                  const float* __restrict__ dirs, const float* __restrict__ I, int IB,
                                  const float* __restrict__ nrm, const float* __restrict__ dif, int dB,
                                  float* __restrict__ out) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)N * B) return;
    int b = (int)(t / N);
    size_t n = t - (size_t)b * N;
    const float* nv = nrm + 3 * t;
    const float* d = dif + 3 * ((dB > 1 ? (size_t)b * N : 0) + n);
    const float* a = amb + 3 * (aB > 1 ? b : 0);
    float S[3] = {0.0f, 0.0f, 0.0f};
    for (int l = 0; l < L; ++l) {
        const float* dl = dirs + 3 * ((size_t)b * L + l);
        const float* il = I + 3 * ((IB > 1 ? (size_t)b * L : 0) + l);
        float c = fadd(fadd(fmul(dl[0], nv[0]), fmul(dl[1], nv[1])), fmul(dl[2], nv[2]));
        c = fminf(fmaxf(c, 0.0f), 1.0f);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float tk = fmul(fmul(il[k], c), fmul(d[k], kInvPiF));
            S[k] = l ? fadd(S[k], tk) : tk;
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) out[3 * t + k] = fadd(fmul(a[k], d[k]), S[k]);
}

// One thread per splat, looping over the views: the normal gradients per
// (view, splat), the diffuse gradient summed over the views in registers
// when diffuse is shared, and the light / ambient gradients reduced over the
// warp, then the block (shared memory), then one atomic per block and value.
__global__ void k_lambert_backward(int B, int N, int L, const float* __restrict__ g,
                                   const float* __restrict__ amb, int aB, const float* __restrict__ dirs,
                                   const float* __restrict__ I, int IB, const float* __restrict__ nrm,
                                   const float* __restrict__ dif, int dB, float* __restrict__ gamb,
                                   float* __restrict__ gdirs, float* __restrict__ gI, float* __restrict__ gn,
                                   float* __restrict__ gd) {
    extern __shared__ float red[];  // gdirs (B L 3), gI (IB L 3), gamb (aB 3)
    float* rD = red;
    float* rI = rD + 3 * B * L;
    float* rA = rI + 3 * IB * L;
    int nred = 3 * B * L + 3 * IB * L + 3 * aB;
    for (int i = threadIdx.x; i < nred; i += blockDim.x) red[i] = 0.0f;
    __syncthreads();
    size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool live = n < (size_t)N;
    int lane = threadIdx.x & 31;
    float gds[3] = {0.0f, 0.0f, 0.0f};  // diffuse gradient summed over the views (dB == 1)
    for (int b = 0; b < B; ++b) {
        float gv[3] = {0, 0, 0}, nv[3] = {0, 0, 0}, d[3] = {0, 0, 0};
        const float* a = amb + 3 * (aB > 1 ? b : 0);
        if (live) {
            size_t t = (size_t)b * N + n;
            const float* dp = dif + 3 * ((dB > 1 ? (size_t)b * N : 0) + n);
#pragma unroll
            for (int k = 0; k < 3; ++k) { gv[k] = g[3 * t + k]; nv[k] = nrm[3 * t + k]; d[k] = dp[k]; }
        }
        float gnv[3] = {0.0f, 0.0f, 0.0f}, gdv[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) gdv[k] = fmul(gv[k], a[k]);
        // ambient: g * d
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float v = fmul(gv[k], d[k]);
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) atomicAdd(&rA[3 * (aB > 1 ? b : 0) + k], v);
        }
        for (int l = 0; l < L; ++l) {
            const float* dl = dirs + 3 * ((size_t)b * L + l);
            const float* il = I + 3 * ((IB > 1 ? (size_t)b * L : 0) + l);
            float s = fadd(fadd(fmul(dl[0], nv[0]), fmul(dl[1], nv[1])), fmul(dl[2], nv[2]));
            float c = fminf(fmaxf(s, 0.0f), 1.0f);
            bool pass = s >= 0.0f && s <= 1.0f;  // clamp passes the gradient inside [0, 1]
            float gs = 0.0f;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                float brdf = fmul(d[k], kInvPiF);
                gs += gv[k] * il[k] * brdf;
                gdv[k] += gv[k] * il[k] * c * kInvPiF;
                float vI = gv[k] * c * brdf;
                for (int o = 16; o > 0; o >>= 1) vI += __shfl_xor_sync(0xffffffffu, vI, o);
                if (lane == 0) atomicAdd(&rI[3 * ((IB > 1 ? b : 0) * L + l) + k], vI);
            }
            if (!pass) gs = 0.0f;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                gnv[k] += gs * dl[k];
                float vD = gs * nv[k];
                for (int o = 16; o > 0; o >>= 1) vD += __shfl_xor_sync(0xffffffffu, vD, o);
                if (lane == 0) atomicAdd(&rD[3 * (b * L + l) + k], vD);
            }
        }
        if (live) {
            size_t t = (size_t)b * N + n;
#pragma unroll
            for (int k = 0; k < 3; ++k) gn[3 * t + k] = gnv[k];
            if (dB > 1) {
#pragma unroll
                for (int k = 0; k < 3; ++k) gd[3 * t + k] = gdv[k];
            } else {
#pragma unroll
                for (int k = 0; k < 3; ++k) gds[k] += gdv[k];
            }
        }
    }
    if (live && dB == 1) {
#pragma unroll
        for (int k = 0; k < 3; ++k) gd[3 * n + k] = gds[k];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nred; i += blockDim.x) {
        float v = red[i];
        if (v != 0.0f) {
            if (i < 3 * B * L) atomicAdd(&gdirs[i], v);
            else if (i < 3 * B * L + 3 * IB * L) atomicAdd(&gI[i - 3 * B * L], v);
            else atomicAdd(&gamb[i - 3 * B * L - 3 * IB * L], v);
        }
    }
}

}  // namespace uds

using namespace uds;

extern "C" int uds_shade_forward(int B, int P, int L, const float* dirs, const float* intensities, int IB,
                                 const float* normals, const float* diffuse, float* out, void* stream) {
    if (B <= 0 || P < 0 || L < 0 || (IB != 1 && IB != B)) return UDS_ERR_ARGUMENT;
    if (P == 0) return UDS_OK;
    k_shade_forward<<<cdiv((size_t)P * B, kShadeThreads), kShadeThreads, 0, as_stream(stream)>>>(
        B, P, L, dirs, intensities, IB, normals, diffuse, out);
    return launch_status();
}

extern "C" int uds_shade_backward(int B, int P, int L, const float* grad, const float* dirs,
                                  const float* intensities, int IB, const float* normals,
                                  const float* diffuse, float* grad_dirs, float* grad_intensities,
                                  float* grad_normals, float* grad_diffuse, void* stream) {
    if (B <= 0 || P < 0 || L < 0 || (IB != 1 && IB != B)) return UDS_ERR_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    cudaError_t e = cudaSuccess;
    if (L > 0) {
        e = cudaMemsetAsync(grad_dirs, 0, sizeof(float) * 3 * (size_t)L * B, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(grad_intensities, 0, sizeof(float) * 3 * (size_t)L * IB, s);
    }
    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    if (P == 0) return UDS_OK;
    k_shade_backward<<<cdiv((size_t)P * B, kShadeThreads), kShadeThreads, 0, s>>>(
        B, P, L, grad, dirs, intensities, IB, normals, diffuse, grad_dirs, grad_intensities, grad_normals,
        grad_diffuse);
    return launch_status();
}

extern "C" int uds_shade_sh_forward(int B, int P, const float* coeffs, int cB, const float* normals,
                                    const float* diffuse, float* out, void* stream) {
    if (B <= 0 || P < 0 || (cB != 1 && cB != B)) return UDS_ERR_ARGUMENT;
    if (P == 0) return UDS_OK;
    k_shade_sh_forward<<<cdiv((size_t)P * B, kShadeThreads), kShadeThreads, 0, as_stream(stream)>>>(
        B, P, coeffs, cB, normals, diffuse, out);
    return launch_status();
}

extern "C" int uds_shade_sh_backward(int B, int P, const float* grad, const float* coeffs, int cB,
                                     const float* normals, const float* diffuse, float* grad_coeffs,
                                     float* grad_normals, float* grad_diffuse, void* stream) {
    if (B <= 0 || P < 0 || (cB != 1 && cB != B)) return UDS_ERR_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    cudaError_t e = cudaMemsetAsync(grad_coeffs, 0, sizeof(float) * 27 * (size_t)cB, s);
    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    if (P == 0) return UDS_OK;
    k_shade_sh_backward<<<cdiv((size_t)P * B, kShadeThreads), kShadeThreads, 0, s>>>(
        B, P, grad, coeffs, cB, normals, diffuse, grad_coeffs, grad_normals, grad_diffuse);
    return launch_status();
}

static size_t lambert_shared(int B, int L, int IB, int aB) {
    return sizeof(float) * (3 * (size_t)B * L + 3 * (size_t)IB * L + 3 * (size_t)aB);
}

extern "C" int uds_lambert_forward(int B, int N, int L, const float* ambient, int aB, const float* dirs,
                                   const float* intensities, int IB, const float* normals,
                                   const float* diffuse, int dB, float* out, void* stream) {
    if (B <= 0 || N < 0 || L < 0 || L > kLambertMaxL || (aB != 1 && aB != B) || (IB != 1 && IB != B) ||
        (dB != 1 && dB != B) || !ambient || (L > 0 && (!dirs || !intensities)))
        return UDS_ERR_ARGUMENT;
    if (N == 0) return UDS_OK;
    if (!normals || !diffuse || !out) return UDS_ERR_ARGUMENT;
    k_lambert_forward<<<cdiv((size_t)N * B, kShadeThreads), kShadeThreads, 0, as_stream(stream)>>>(
        B, N, L, ambient, aB, dirs, intensities, IB, normals, diffuse, dB, out);
    return launch_status();
}

extern "C" int uds_lambert_backward(int B, int N, int L, const float* grad, const float* ambient, int aB,
                                    const float* dirs, const float* intensities, int IB, const float* normals,
                                    const float* diffuse, int dB, float* grad_ambient, float* grad_dirs,
                                    float* grad_intensities, float* grad_normals, float* grad_diffuse,
                                    void* stream) {
    if (B <= 0 || N < 0 || L < 0 || L > kLambertMaxL || (aB != 1 && aB != B) || (IB != 1 && IB != B) ||
        (dB != 1 && dB != B) || !ambient || !grad_ambient || (L > 0 && (!dirs || !intensities || !grad_dirs ||
                                                                        !grad_intensities)))
        return UDS_ERR_ARGUMENT;
    size_t shm = lambert_shared(B, L, IB, aB);
    if (shm > 48 * 1024) return UDS_ERR_ARGUMENT;
    cudaStream_t s = as_stream(stream);
    cudaError_t e = cudaMemsetAsync(grad_ambient, 0, sizeof(float) * 3 * (size_t)aB, s);
    if (e == cudaSuccess && L > 0) e = cudaMemsetAsync(grad_dirs, 0, sizeof(float) * 3 * (size_t)B * L, s);
    if (e == cudaSuccess && L > 0) e = cudaMemsetAsync(grad_intensities, 0, sizeof(float) * 3 * (size_t)IB * L, s);
    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    if (N == 0) return UDS_OK;
    if (!grad || !normals || !diffuse || !grad_normals || !grad_diffuse) return UDS_ERR_ARGUMENT;
    k_lambert_backward<<<cdiv((size_t)N, kShadeThreads), kShadeThreads, shm, s>>>(
        B, N, L, grad, ambient, aB, dirs, intensities, IB, normals, diffuse, dB, grad_ambient, grad_dirs,
        grad_intensities, grad_normals, grad_diffuse);
    return launch_status();
}
