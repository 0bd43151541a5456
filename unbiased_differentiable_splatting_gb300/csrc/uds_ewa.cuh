// EWA screen-space Gaussian of a camera-space surfel: per-splat frame with
// the reference's float/double operation sequence (transformation.cuh:29-58,
// ewaSplatting.cuh:8-91, linalg.cuh), and its reverse-mode derivative.
#pragma once
#include "uds_common.cuh"
#include "uds_backproject.cuh"

namespace uds {

__device__ __forceinline__ float dot3(const float* a, const float* b) {
    return fadd(fadd(fadd(0.0f, fmul(a[0], b[0])), fmul(a[1], b[1])), fmul(a[2], b[2]));
}

// toScreenspace: -(x f)/z + W/2.0 (the addend is double; W/2 is a float)
__device__ __forceinline__ void screen_point(float W, float H, float f, const float* p, float* s) {
    s[0] = add_via_double(fdiv(-fmul(p[0], f), p[2]), fmul(W, 0.5f));
    s[1] = add_via_double(fdiv(fmul(p[1], f), p[2]), fmul(H, 0.5f));
}

// backproject (double arithmetic, rounded to float): the same numbers from
// the exact integer quotient where it applies, else the double sequence
__device__ __forceinline__ void back_project(float W, float H, float f, const float* s, float* x) {
    float q;
    if (bp_quotient(fmul(W, 0.5f), s[0], f, &q)) x[0] = q;
    else x[0] = (float)ddiv(dsub((double)W, dmul(2.0, (double)s[0])), dmul(2.0, (double)f));
    if (bp_quotient(fmul(H, 0.5f), s[1], f, &q)) x[1] = -q;
    else x[1] = (float)ddiv(-dsub((double)H, dmul(2.0, (double)s[1])), dmul(2.0, (double)f));
    x[2] = 1.0f;
}

// projectOntoPlane(x, p, n) - p
__device__ __forceinline__ void tangent(const float* x, const float* p, const float* n, float* t) {
    float xts = fdiv(dot3(p, n), dot3(x, n));
#pragma unroll
    for (int i = 0; i < 3; ++i) t[i] = fsub(fmul(x[i], xts), p[i]);
}

struct EwaFrame {
    float sp[2];
    float invJ[4];
    float V[4];
};

__device__ __forceinline__ void ewa_frame(float W, float H, float f, const float* p, const float* n,
                                          const float* sd, float sm, EwaFrame& F) {
    screen_point(W, H, f, p, F.sp);
    float y0[2] = {add_via_double(F.sp[0], 1.0f), F.sp[1]};
    float y1[2] = {F.sp[0], add_via_double(F.sp[1], 1.0f)};
    float x0[3], x1[3], t0[3], t1[3];
    back_project(W, H, f, y0, x0);
    back_project(W, H, f, y1, x1);
    tangent(x0, p, n, t0);
    tangent(x1, p, n, t1);
    float nt0 = fsqrt(dot3(t0, t0));
    float invNorm = div_via_double(1.0f, nt0);
    float u0[3] = {fmul(t0[0], invNorm), fmul(t0[1], invNorm), fmul(t0[2], invNorm)};
    float u1[3] = {fsub(fmul(u0[1], n[2]), fmul(u0[2], n[1])), fsub(fmul(u0[2], n[0]), fmul(u0[0], n[2])),
                   fsub(fmul(u0[0], n[1]), fmul(u0[1], n[0]))};
    F.invJ[0] = nt0;
    F.invJ[1] = dot3(t1, u0);
    F.invJ[2] = 0.0f;
    F.invJ[3] = dot3(t1, u1);
    const float* iJ = F.invJ;
    float det = fsub(fmul(iJ[0], iJ[3]), fmul(iJ[1], iJ[2]));
    float invDet = div_via_double(1.0f, det);
    float J[4] = {fmul(iJ[3], invDet), fmul(-iJ[1], invDet), fmul(-iJ[2], invDet), fmul(iJ[0], invDet)};
    float D[4] = {fmul(sd[0], sd[0]), 0.0f, 0.0f, fmul(sd[1], sd[1])};
    float T[4], U[4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int k = 0; k < 2; ++k)
            T[2 * i + k] = fadd(fadd(0.0f, fmul(J[2 * i], D[k])), fmul(J[2 * i + 1], D[2 + k]));
    float Jt[4] = {J[0], J[2], J[1], J[3]};
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int k = 0; k < 2; ++k)
            U[2 * i + k] = fadd(fadd(0.0f, fmul(T[2 * i], Jt[k])), fmul(T[2 * i + 1], Jt[2 + k]));
    F.V[0] = fadd(U[0], sm);
    F.V[1] = fadd(U[1], 0.0f);
    F.V[2] = fadd(U[2], 0.0f);
    F.V[3] = fadd(U[3], sm);
}

// Per-splat constants of the Gaussian: {sp.x, sp.y, iV0, iV1, iV2, iV3, Z, 0}
// with weight = exp(-0.5 e) / Z, e = (x iV) . x, x = pixel - sp, and Z the
// normalisation 2 pi sqrt(det V) |det invJ| rounded to float like the
// reference's evaluteGaussian (ewaSplatting.cuh:128-137).
__device__ __forceinline__ void ewa_gauss_consts(const EwaFrame& F, float4& a, float4& b) {
    const float* V = F.V;
    float vdet = fsub(fmul(V[0], V[3]), fmul(V[1], V[2]));
    float inv = div_via_double(1.0f, vdet);
    float jdet = fsub(fmul(F.invJ[0], F.invJ[3]), fmul(F.invJ[1], F.invJ[2]));
    float norm = (float)dmul(dmul(2.0 * kPi, (double)fsqrt(vdet)), (double)fabsf(jdet));
    a = make_float4(F.sp[0], F.sp[1], fmul(V[3], inv), fmul(-V[1], inv));
    b = make_float4(fmul(-V[2], inv), fmul(V[0], inv), norm, 0.0f);
}

// Unclamped Gaussian at a pixel from the per-splat constants.
__device__ __forceinline__ float ewa_gauss(const float4& a, const float4& b, float px, float py,
                                           float* dx = nullptr, float* dy = nullptr) {
    float x0 = fsub(px, a.x), x1 = fsub(py, a.y);
    float y0 = fadd(fmul(x0, a.z), fmul(x1, b.x));
    float y1 = fadd(fmul(x0, a.w), fmul(x1, b.y));
    float e = fadd(fmul(y0, x0), fmul(y1, x1));
    if (dx) { *dx = x0; *dy = x1; }
    return fdiv(expf(fmul(-0.5f, e)), b.z);
}

}  // namespace uds
