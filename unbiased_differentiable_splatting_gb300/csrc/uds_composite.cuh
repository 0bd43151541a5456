// Depth compositing helpers shared by filtering.forward / backward and the
// fused render kernels (zSortingCuda.cu:11-243, alphacompositing.cuh):
// the pixel ray, each sample's depth along it to the splat's tangent plane,
// the stable insertion arg-sort by depth, and front-to-back blending.  The
// arithmetic follows the reference operation by operation (double where it
// promotes), so the depth order is identical to the CPU oracle's.
#pragma once
#include "uds_blendrem.cuh"
#include "uds_ewa.cuh"

namespace uds {

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

// front-to-back blend (alphacompositing.cuh:58-68): fw[id] = rem * w[id],
// rem *= (1 - w[id]) in double, in depth order; the double update is done on
// the exact integer product (uds_blendrem.cuh) wherever that gives the same
// float, so the FP64 pipe only sees the rare inputs off that path
template <int KMAX>
__device__ __forceinline__ void blend(int K, const int* ord, const float* w, float* fw) {
    float rem = 1.0f;
    for (int q = 0; q < K; ++q) {
        int id = ord[q];
        fw[id] = fmul(rem, w[id]);
        float next;
        if (!blend_rem(rem, w[id], &next)) next = (float)dmul((double)rem, dsub(1.0, (double)w[id]));
        rem = next;
    }
}

// gradBlending (alphacompositingGrad.cuh:7-26): the gradient of the EWA
// weight of the sample at depth rank k, terms whose divisor is within 1e-4
// of zero dropped as in the reference
template <int KMAX>
__device__ __forceinline__ float blend_grad(int K, int k, const int* ord, const float* w, const float* fw,
                                            const float* g) {
    const float eps = 1e-4f;
    int kdx = ord[k];
    float wk = w[kdx];
    float acc = 0.0f;
    for (int q = k; q < K; ++q) {
        int id = ord[q];
        float den = (q == k) ? wk : -fsub(1.0f, wk);
        if (fabsf(den) > eps) acc = fadd(acc, fdiv(fmul(g[id], fw[id]), den));
    }
    return acc;
}

}  // namespace uds
