// Shared device helpers of libuds.so: status plumbing, exact-rounding float
// arithmetic, the deterministic exp / log used on the sampling path, Philox
// uniforms, and the tree layout in HBM.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/uds.h"

namespace uds {

// ----------------------------------------------------------------- status
void set_last_error(cudaError_t e);
int launch_status(int launches = 1);  // UDS_OK or UDS_ERR_LAUNCH after `launches` kernel launches

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

constexpr int kMaxK = 64;        // samples per pixel supported by the sampler
constexpr int kMaxLeaf = 64;     // largest leaf size of the Poisson descent
constexpr int kMaxRounds = 8;    // ceil(sqrt(64))
constexpr int kTrace = 64;       // descent trace entries (reference STACKSIZE)
constexpr int kMaxDegree = 16;   // reference MAXDEGREE
constexpr float kZmax = 10000.0f;  // depth of invalid samples (alphacompositing.cuh:16)
constexpr double kPi = 3.14159265358979323846;

inline int num_rounds(int K) {
    // for (i = 0; i < sqrt(K); i++) in the reference host driver
    int R = 0;
    while (R * R < K) ++R;
    return R;
}

inline unsigned cdiv(size_t a, unsigned b) { return (unsigned)((a + b - 1) / b); }

// ------------------------------------------------- exact-rounding float ops
// The sampling path must round exactly like the CPU oracle (which is built
// with contraction off), so those kernels spell out every operation.
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// One double operation on float operands, rounded to float, is the float
// operation itself: rounding to 53 bits and then to 24 is innocuous for +, -,
// *, / and sqrt because 53 >= 2 * 24 + 2 (S. A. Figueroa, "When is double
// rounding innocuous?", SIGNUM Newsletter 30(3), 1995); overflow and
// subnormal results round the same way too.  So the reference's
// (float)(1.0 / (double)x) or (float)((double)x + 1.0) runs here as a float
// operation with the identical result, off the slow FP64 pipe.
__device__ __forceinline__ float div_via_double(float a, float b) { return fdiv(a, b); }
__device__ __forceinline__ float add_via_double(float a, float b) { return fadd(a, b); }
__device__ __forceinline__ float sub_via_double(float a, float b) { return fsub(a, b); }

// --------------------------------------------- deterministic exp and log
// exp: Cody & Waite (1980) reduction x = k ln2 + r with ln2 split in a high
// and a low part, degree-7 Taylor polynomial of e^r in Horner form with
// fused multiply-adds, exact scaling by 2^k.  log: x = m 2^e with m in
// [sqrt(1/2), sqrt(2)], log m = 2 atanh((m-1)/(m+1)) by its odd series to the
// 13th power.  Only IEEE-exact operations, so the C oracle reproduces them.
#define UDS_LN2_HI 0.693145751953125f
#define UDS_LN2_LO 1.428606765330187e-06f

__device__ __forceinline__ float scale_pow2(float p, int n) {
    if (n > 127) { p = fmul(p, 0x1p127f); n -= 127; }
    if (n < -126) {
        p = fmul(p, 0x1p-126f); n += 126;
        if (n < -126) { p = fmul(p, 0x1p-126f); n += 126; }
    }
    return fmul(p, __uint_as_float((unsigned)(n + 127) << 23));
}

__device__ __forceinline__ float det_expf(float x) {
    if (x != x) return x;
    if (x > 88.72283935546875f) return __int_as_float(0x7f800000);
    if (x < -103.972084f) return 0.0f;
    float k = rintf(fmul(x, 1.44269502f));
    float r = __fmaf_rn(-k, UDS_LN2_HI, x);
    r = __fmaf_rn(-k, UDS_LN2_LO, r);
    float p = 1.0f / 5040.0f;
    p = __fmaf_rn(p, r, 1.0f / 720.0f);
    p = __fmaf_rn(p, r, 1.0f / 120.0f);
    p = __fmaf_rn(p, r, 1.0f / 24.0f);
    p = __fmaf_rn(p, r, 1.0f / 6.0f);
    p = __fmaf_rn(p, r, 0.5f);
    p = __fmaf_rn(p, r, 1.0f);
    p = __fmaf_rn(p, r, 1.0f);
    return scale_pow2(p, (int)k);
}

__device__ __forceinline__ float det_logf(float x) {
    if (x != x) return x;
    if (x < 0.0f) return __int_as_float(0x7fc00000);
    if (x == 0.0f) return __int_as_float(0xff800000);
    if (x == __int_as_float(0x7f800000)) return x;
    unsigned u = __float_as_uint(x);
    int e = 0;
    if (u < 0x00800000u) { x = fmul(x, 0x1p23f); u = __float_as_uint(x); e = -23; }
    e += (int)(u >> 23) - 127;
    float m = __uint_as_float((u & 0x007FFFFFu) | 0x3F800000u);
    if (m > 1.41421356f) { m = fmul(m, 0.5f); e += 1; }
    float s = fdiv(fsub(m, 1.0f), fadd(m, 1.0f));
    float s2 = fmul(s, s);
    float q = 1.0f / 13.0f;
    q = __fmaf_rn(q, s2, 1.0f / 11.0f);
    q = __fmaf_rn(q, s2, 1.0f / 9.0f);
    q = __fmaf_rn(q, s2, 1.0f / 7.0f);
    q = __fmaf_rn(q, s2, 1.0f / 5.0f);
    q = __fmaf_rn(q, s2, 1.0f / 3.0f);
    float lm = fmul(2.0f, __fmaf_rn(fmul(s, s2), q, s));
    float fe = (float)e;
    return __fmaf_rn(fe, UDS_LN2_HI, __fmaf_rn(fe, UDS_LN2_LO, lm));
}

__device__ __forceinline__ float ipowf(float x, unsigned n) {
    float r = 1.0f;
    for (unsigned i = 0; i < n; ++i) r = fmul(r, x);
    return r;
}

// n! as the reference's sequential float product (hermitefmm.cuh fac)
__device__ __forceinline__ float facf(unsigned n) {
    float p = 1.0f;
    for (unsigned i = 1; i <= n; ++i) p = fmul(p, (float)i);
    return p;
}

// ------------------------------------------------------------ Philox4x32-10
// Salmon, Moraes, Dror & Shaw, "Parallel random numbers: as easy as 1, 2, 3"
// (SC'11).  counter = (pixel, view, round*ceil(K/4)+group, 0), key = seed.
__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
        uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
}
// u in (0, 1], exactly ((x >> 8) + 1) * 2^-24
__device__ __forceinline__ float bits_to_uniform(uint32_t x) {
    return (float)((x >> 8) + 1u) * 0x1p-24f;
}

// ---------------------------------------------------------- tree in HBM
// Node v in [0, n-2] is internal (0 = root), node n-1+i is the leaf of the
// i-th splat in Morton order.  Structure-of-arrays, 16-byte records:
//   lnk[v]  = {left, right, first leaf position, leaf count}
//   par[v]  = parent (-1 at the root)
//   box[v]  = {lo.x, lo.y, hi.x, hi.y} screen-space bounding box
//   cen[v]  = {centre.x, centre.y, truncation radius, meta}
//             meta (int bits) = (coefficient offset << 5) | (degree + 1)
//   leaf_xy[i], leaf_id[i]: screen position and splat id of sorted leaf i
struct TreeView {
    const int4* lnk;
    const int* par;
    const float4* box;
    const float4* cen;
    const float* coef;
    const float2* leaf_xy;
    const int* leaf_id;
    const int* n_ptr;  // device scalar: number of leaves
    float h;           // unused when h_ptr is set
    const float* h_ptr;
};

__device__ __forceinline__ int meta_degree(float w) { return (__float_as_int(w) & 31) - 1; }
__device__ __forceinline__ int meta_offset(float w) { return __float_as_int(w) >> 5; }
__device__ __forceinline__ float make_meta(int offset, int degree) {
    return __int_as_float((offset << 5) | (degree + 1));
}

}  // namespace uds
