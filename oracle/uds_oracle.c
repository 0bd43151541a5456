/* CPU oracle for the Poisson-sampled EWA splatting path.
 *
 * TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and the CPU legs
 * of bench.py load this library to check or to time the CUDA path; the
 * product never does.
 *
 * A C restatement of the reference (paths below are inside the reference
 * project).  Compiled with -ffp-contract=off so that every a*b+c rounds twice
 * unless fmaf is written out; results are identical on x86-64 and aarch64.
 * Where the reference mixes double constants into float code the same
 * promotions are written out explicitly.
 */
#include "uds_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846
#define ORC_MAXDEGREE 16   /* radixTree.cuh:8 */
#define ORC_STACK 64       /* transformRadixTree.cuh:12 STACKSIZE */
#define ORC_ZMAX 10000.0f  /* alphacompositing.cuh:16 */

static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* ------------------------------------------------------------------------
 * Deterministic elementary functions.  Exponential: Cody & Waite (1980)
 * argument reduction x = n ln2 + r, |r| <= ln2/2, with ln2 split in a high
 * and a low part, then the degree-7 Taylor polynomial of e^r in Horner form
 * with fused multiply-adds (truncation error r^8/8! < 6e-9 relative), then an
 * exact scaling by 2^n.  Logarithm: x = m 2^e with m in [sqrt(1/2), sqrt(2)],
 * log m = 2 atanh(s), s = (m-1)/(m+1), odd series to s^13.  Only IEEE
 * add/mul/div/sqrt and fmaf are used, so CUDA and C give the same bits.
 * ---------------------------------------------------------------------- */
#define LN2_HI 0.693145751953125f
#define LN2_LO 1.428606765330187e-06f

static inline float scale_pow2(float p, int n) {
    if (n > 127) { p *= 0x1p127f; n -= 127; }
    if (n < -126) {
        p *= 0x1p-126f; n += 126;
        if (n < -126) { p *= 0x1p-126f; n += 126; }
    }
    return p * u2f((uint32_t)(n + 127) << 23);
}

float orc_det_expf(float x) {
    if (x != x) return x;
    if (x > 88.72283935546875f) return INFINITY;
    if (x < -103.972084f) return 0.0f;
    float k = rintf(x * 1.44269502f);
    float r = fmaf(-k, LN2_HI, x);
    r = fmaf(-k, LN2_LO, r);
    float p = 1.0f / 5040.0f;
    p = fmaf(p, r, 1.0f / 720.0f);
    p = fmaf(p, r, 1.0f / 120.0f);
    p = fmaf(p, r, 1.0f / 24.0f);
    p = fmaf(p, r, 1.0f / 6.0f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    return scale_pow2(p, (int)k);
}

float orc_det_logf(float x) {
    if (x != x) return x;
    if (x < 0.0f) return NAN;
    if (x == 0.0f) return -INFINITY;
    if (x == INFINITY) return x;
    uint32_t u = f2u(x);
    int e = 0;
    if (u < 0x00800000u) { x *= 0x1p23f; u = f2u(x); e = -23; }
    e += (int)(u >> 23) - 127;
    float m = u2f((u & 0x007FFFFFu) | 0x3F800000u);
    if (m > 1.41421356f) { m *= 0.5f; e += 1; }
    float s = (m - 1.0f) / (m + 1.0f);
    float s2 = s * s;
    float q = 1.0f / 13.0f;
    q = fmaf(q, s2, 1.0f / 11.0f);
    q = fmaf(q, s2, 1.0f / 9.0f);
    q = fmaf(q, s2, 1.0f / 7.0f);
    q = fmaf(q, s2, 1.0f / 5.0f);
    q = fmaf(q, s2, 1.0f / 3.0f);
    float lm = 2.0f * fmaf(s * s2, q, s);
    float fe = (float)e;
    return fmaf(fe, LN2_HI, fmaf(fe, LN2_LO, lm));
}

static inline float xexpf(float x, int fl) { return fl == ORC_LIBM ? expf(x) : orc_det_expf(x); }
static inline float xlogf(float x, int fl) { return fl == ORC_LIBM ? logf(x) : orc_det_logf(x); }
static inline float ipowf(float x, unsigned n) {
    float r = 1.0f;
    for (unsigned i = 0; i < n; ++i) r *= x;
    return r;
}
static inline float xpowi(float x, unsigned n, int fl) { return fl == ORC_LIBM ? powf(x, (float)n) : ipowf(x, n); }
/* fac (hermitefmm.cuh:14-21) */
static inline float facf(unsigned n) {
    float p = 1.0f;
    for (unsigned i = 1; i <= n; ++i) p *= (float)i;
    return p;
}

/* ------------------------------------------------------------------------
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) counter-based uniforms.
 * counter = (pixel, view, round * ceil(K/4) + group, 0), key = seed.
 * u = ((x >> 8) + 1) * 2^-24 lies in (0, 1] like curand_uniform.
 * ---------------------------------------------------------------------- */
static void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
}

void orc_philox_uniforms(uint64_t seed, uint32_t view, uint32_t pixel, uint32_t round, int K,
                         float* out) {
    int G = (K + 3) / 4;
    for (int g = 0; g < G; ++g) {
        uint32_t c[4] = {pixel, view, round * (uint32_t)G + (uint32_t)g, 0u};
        philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
        for (int q = 0; q < 4 && 4 * g + q < K; ++q)
            out[4 * g + q] = (float)((c[q] >> 8) + 1u) * 0x1p-24f;
    }
}

int orc_num_rounds(int K) {
    /* sequentialPoissonDynamicTree.cuh:251: for (i = 0; i < sqrt(K); i++) */
    int R = 0;
    while ((double)R < sqrt((double)K)) ++R;
    return R;
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------
 * Transform (transformation.cuh:8-27, transformationGrad.cuh:5-40)
 * ---------------------------------------------------------------------- */
void orc_transform_forward(int affine, int B, const float* M, int vB, int N, const float* v,
                           float* out) {
    for (int b = 0; b < B; ++b) {
        const float* T = &M[16 * b];
        for (int x = 0; x < N; ++x) {
            const float* p = &v[vB > 1 ? 3 * ((size_t)x + (size_t)N * b) : 3 * (size_t)x];
            float* o = &out[3 * ((size_t)x + (size_t)N * b)];
            for (int i = 0; i < 3; ++i) {
                float s = 0.0f;
                for (int j = 0; j < 3; ++j) s += T[4 * i + j] * p[j];
                if (affine) s += T[4 * i + 3];
                o[i] = s;
            }
        }
    }
}

void orc_transform_backward(int affine, int B, const float* gin, const float* M, int vB, int N,
                            const float* v, float* gM, float* gv) {
    for (int b = 0; b < B; ++b) {
        const float* T = &M[16 * b];
        double acc[16] = {0};
        for (int x = 0; x < N; ++x) {
            size_t vo = vB > 1 ? 3 * ((size_t)x + (size_t)N * b) : 3 * (size_t)x;
            const float* p = &v[vo];
            const float* g = &gin[3 * ((size_t)x + (size_t)N * b)];
            for (int i = 0; i < 3; ++i) {
                for (int j = 0; j < 3; ++j) acc[4 * i + j] += (double)g[i] * p[j];
                if (affine) acc[4 * i + 3] += g[i];
            }
            for (int j = 0; j < 3; ++j) {
                double s = 0.0;
                for (int i = 0; i < 3; ++i) s += (double)g[i] * T[4 * i + j];
                gv[vo + j] += (float)s;
            }
        }
        for (int i = 0; i < 16; ++i) gM[16 * b + i] += (float)acc[i];
    }
}

/* ------------------------------------------------------------------------
 * EWA weight, float arithmetic in the reference's order
 * (transformation.cuh:29-58, ewaSplatting.cuh:8-91, linalg.cuh).
 * ---------------------------------------------------------------------- */
static inline float dot3f(const float* a, const float* b) {
    float x = 0.0f;
    for (int i = 0; i < 3; ++i) x += a[i] * b[i];
    return x;
}
static inline float norm3f(const float* a) { return sqrtf(dot3f(a, a)); }

static inline void screenf(float W, float H, float f, const float* p, float* s) {
    s[0] = (float)((double)(-(p[0] * f) / p[2]) + (double)W / 2.0);
    s[1] = (float)((double)((p[1] * f) / p[2]) + (double)H / 2.0);
}
static inline void backprojf(float W, float H, float f, const float* s, float* x) {
    x[0] = (float)(((double)W - 2.0 * (double)s[0]) / (2.0 * (double)f));
    x[1] = (float)(-((double)H - 2.0 * (double)s[1]) / (2.0 * (double)f));
    x[2] = 1.0f;
}
/* projectOntoPlane(x, p, n) - p */
static inline void tangentf(const float* x, const float* p, const float* n, float* t) {
    float na = dot3f(p, n);
    float xts = na / dot3f(x, n);
    for (int i = 0; i < 3; ++i) t[i] = x[i] * xts - p[i];
}
typedef struct {
    float sp[2], invJ[4], V[4];
} ewa_frame;

static void ewa_framef(float W, float H, float f, const float* p, const float* n, const float* sd,
                       float sm, ewa_frame* F) {
    screenf(W, H, f, p, F->sp);
    float y0[2] = {(float)((double)F->sp[0] + 1.0), F->sp[1]};
    float y1[2] = {F->sp[0], (float)((double)F->sp[1] + 1.0)};
    float x0[3], x1[3], t0[3], t1[3];
    backprojf(W, H, f, y0, x0);
    backprojf(W, H, f, y1, x1);
    tangentf(x0, p, n, t0);
    tangentf(x1, p, n, t1);
    float invNorm = (float)(1.0 / (double)norm3f(t0));
    float u0[3] = {t0[0] * invNorm, t0[1] * invNorm, t0[2] * invNorm};
    float u1[3] = {u0[1] * n[2] - u0[2] * n[1], u0[2] * n[0] - u0[0] * n[2], u0[0] * n[1] - u0[1] * n[0]};
    float* iJ = F->invJ;
    iJ[0] = norm3f(t0);
    iJ[1] = dot3f(t1, u0);
    iJ[2] = 0.0f;
    iJ[3] = dot3f(t1, u1);
    /* buildCovariance: Jk * D^2 * Jk^T + smoothing I */
    float det = iJ[0] * iJ[3] - iJ[1] * iJ[2];
    float invDet = (float)(1.0 / (double)det);
    float J[4] = {iJ[3] * invDet, -iJ[1] * invDet, -iJ[2] * invDet, iJ[0] * invDet};
    float D[4] = {sd[0] * sd[0], 0.0f * 0.0f, 0.0f * 0.0f, sd[1] * sd[1]};
    float T[4], U[4];
    for (int i = 0; i < 2; ++i)
        for (int k = 0; k < 2; ++k) {
            float m = 0.0f;
            for (int j = 0; j < 2; ++j) m += J[2 * i + j] * D[2 * j + k];
            T[2 * i + k] = m;
        }
    float Jt[4] = {J[0], J[2], J[1], J[3]};
    for (int i = 0; i < 2; ++i)
        for (int k = 0; k < 2; ++k) {
            float m = 0.0f;
            for (int j = 0; j < 2; ++j) m += T[2 * i + j] * Jt[2 * j + k];
            U[2 * i + k] = m;
        }
    F->V[0] = U[0] + sm;
    F->V[1] = U[1] + 0.0f;
    F->V[2] = U[2] + 0.0f;
    F->V[3] = U[3] + sm;
}

/* evaluteGaussian (ewaSplatting.cuh:56-67) */
static float ewa_gaussf(const float* pixel, const ewa_frame* F) {
    float x[2] = {pixel[0] - F->sp[0], pixel[1] - F->sp[1]};
    const float* V = F->V;
    float vdet = V[0] * V[3] - V[1] * V[2];
    float inv = (float)(1.0 / (double)vdet);
    float iV[4] = {V[3] * inv, -V[1] * inv, -V[2] * inv, V[0] * inv};
    float y0 = x[0] * iV[0] + x[1] * iV[2];
    float y1 = x[0] * iV[1] + x[1] * iV[3];
    float e = y0 * x[0] + y1 * x[1];
    float jdet = F->invJ[0] * F->invJ[3] - F->invJ[1] * F->invJ[2];
    float normalization = (float)(2.0 * ORC_PI * (double)sqrtf(vdet) * (double)fabsf(jdet));
    float ex = expf((float)(-0.5 * (double)e));
    return ex / normalization;
}

void orc_to_screenspace(int n, float W, float H, float f, const float* pts, float* out) {
    for (int i = 0; i < n; ++i) screenf(W, H, f, &pts[3 * (size_t)i], &out[2 * (size_t)i]);
}

float orc_ewa_weight(const float* pixel, float W, float H, float f, const float* p,
                     const float* nrm, const float* sd, float smoothing, float* unclamped) {
    ewa_frame F;
    ewa_framef(W, H, f, p, nrm, sd, smoothing, &F);
    float g = ewa_gaussf(pixel, &F);
    if (unclamped) *unclamped = g;
    return (float)fmin((double)g, 1.0);
}

/* ------------------------------------------------------------------------
 * EWA gradient: reverse-mode derivative of the weight in FP64, derived
 * directly from the forward definition (ewaSplatting.cuh:8-91):
 *   s = screen(p), x0/x1 = back-projected s+e_x / s+e_y, t0/t1 their
 *   projections onto the tangent plane minus p, invJ = [[|t0|, t1.u0],
 *   [0, t1.(u0 x n)]], V = J diag(sd^2) J^T + smoothing I,
 *   G = exp(-d^T V^-1 d / 2) / (2 pi sqrt(det V) |det invJ|), d = pixel - s.
 * Cross-checked against the reference's gradEWAWeight
 * (ewaSplattingGrad.cuh:163-206) and against central differences.
 * ---------------------------------------------------------------------- */
static inline double dot3d(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline void cross3d(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

void orc_ewa_grad(const float* pixel, float W, float H, float f, const float* pf, const float* nf,
                  const float* sdf, float smoothing, double* gp, double* gn, double* gs) {
    double p[3] = {pf[0], pf[1], pf[2]}, n[3] = {nf[0], nf[1], nf[2]};
    double sd[2] = {sdf[0], sdf[1]}, F = f, sm = smoothing;
    /* forward */
    double s0 = -(p[0] * F) / p[2] + W / 2.0, s1 = (p[1] * F) / p[2] + H / 2.0;
    double a0 = (W - 2.0 * s0) / (2.0 * F), a1 = -(H - 2.0 * s1) / (2.0 * F);
    double x0[3] = {a0 - 1.0 / F, a1, 1.0}, x1[3] = {a0, a1 + 1.0 / F, 1.0};
    double c = dot3d(p, n);
    double D0 = dot3d(x0, n), D1 = dot3d(x1, n);
    double k0 = c / D0, k1 = c / D1;
    double t0[3], t1[3];
    for (int i = 0; i < 3; ++i) { t0[i] = k0 * x0[i] - p[i]; t1[i] = k1 * x1[i] - p[i]; }
    double al = sqrt(dot3d(t0, t0));
    double u0[3] = {t0[0] / al, t0[1] / al, t0[2] / al};
    double u1[3];
    cross3d(u0, n, u1);
    double be = dot3d(t1, u0), ga = dot3d(t1, u1);
    /* J = inv([[al, be], [0, ga]]) */
    double J00 = 1.0 / al, J01 = -be / (al * ga), J11 = 1.0 / ga;
    double S0 = sd[0] * sd[0], S1 = sd[1] * sd[1];
    double V00 = J00 * J00 * S0 + J01 * J01 * S1 + sm;
    double V01 = J01 * J11 * S1;
    double V11 = J11 * J11 * S1 + sm;
    double vdet = V00 * V11 - V01 * V01;
    double I00 = V11 / vdet, I01 = -V01 / vdet, I11 = V00 / vdet;
    double d0 = pixel[0] - s0, d1 = pixel[1] - s1;
    double q0 = I00 * d0 + I01 * d1, q1 = I01 * d0 + I11 * d1; /* V^-1 d */
    double e = d0 * q0 + d1 * q1;
    double G = exp(-0.5 * e) / (2.0 * ORC_PI * sqrt(vdet) * fabs(al * ga));
    /* backward: dG/dV (symmetric), dG/ds, direct |det invJ| terms */
    double gV00 = 0.5 * G * (q0 * q0 - I00), gV01 = 0.5 * G * (q0 * q1 - I01), gV11 = 0.5 * G * (q1 * q1 - I11);
    double gs0 = G * q0, gs1 = G * q1; /* dG/ds (d = pixel - s) */
    /* V = J S J^T + sm I, J upper triangular {J00, J01, J11} */
    double gJ00 = 2.0 * (gV00 * J00 * S0);
    double gJ01 = 2.0 * (gV00 * J01 * S1 + gV01 * J11 * S1);
    double gJ11 = 2.0 * (gV01 * J01 * S1 + gV11 * J11 * S1);
    gs[0] = 2.0 * sd[0] * (J00 * J00 * gV00);
    gs[1] = 2.0 * sd[1] * (J01 * J01 * gV00 + 2.0 * J01 * J11 * gV01 + J11 * J11 * gV11);
    /* J from invJ = [[al, be], [0, ga]] */
    double gal = -gJ00 / (al * al) + gJ01 * be / (al * al * ga) - G / al;
    double gbe = -gJ01 / (al * ga);
    double gga = gJ01 * be / (al * ga * ga) - gJ11 / (ga * ga) - G / ga;
    /* be = t1.u0, ga = t1.(u0 x n) */
    double gt1[3], gu0[3], gnv[3], nxt1[3], t1xu0[3];
    cross3d(n, t1, nxt1);
    cross3d(t1, u0, t1xu0);
    for (int i = 0; i < 3; ++i) {
        gt1[i] = gbe * u0[i] + gga * u1[i];
        gu0[i] = gbe * t1[i] + gga * nxt1[i];
        gnv[i] = gga * t1xu0[i];
    }
    /* u0 = t0 / al, al = |t0| */
    double gdotu = dot3d(gu0, u0), gt0[3];
    for (int i = 0; i < 3; ++i) gt0[i] = (gu0[i] - gdotu * u0[i]) / al + gal * u0[i];
    /* t = k x - p, k = c / (x.n), c = p.n */
    double gpv[3] = {-gt0[0] - gt1[0], -gt0[1] - gt1[1], -gt0[2] - gt1[2]};
    double gx0[3], gx1[3];
    double gk0 = dot3d(gt0, x0), gk1 = dot3d(gt1, x1);
    double gc = gk0 / D0 + gk1 / D1;
    double gD0 = -gk0 * c / (D0 * D0), gD1 = -gk1 * c / (D1 * D1);
    for (int i = 0; i < 3; ++i) {
        gx0[i] = k0 * gt0[i] + gD0 * n[i];
        gx1[i] = k1 * gt1[i] + gD1 * n[i];
        gnv[i] += gD0 * x0[i] + gD1 * x1[i] + gc * p[i];
        gpv[i] += gc * n[i];
    }
    /* x0 = (a0 - 1/f, a1, 1), x1 = (a0, a1 + 1/f, 1), a0 = (W - 2 s0)/(2f), a1 = (2 s1 - H)/(2f) */
    double ga0 = gx0[0] + gx1[0], ga1 = gx0[1] + gx1[1];
    double gS0 = gs0 - ga0 / F, gS1 = gs1 + ga1 / F; /* dG/ds = G V^-1 d */
    gpv[0] += gS0 * (-F / p[2]);
    gpv[1] += gS1 * (F / p[2]);
    gpv[2] += gS0 * (p[0] * F / (p[2] * p[2])) - gS1 * (p[1] * F / (p[2] * p[2]));
    for (int i = 0; i < 3; ++i) { gp[i] = gpv[i]; gn[i] = gnv[i]; }
}

/* ewaKernel (splattingCuda.cu:18-66) */
void orc_splat_forward(int B, int W, int H, int K, float f, const int* idx, const float* pts,
                       const float* nrm, const float* sd, int sdB, int N, float smoothing,
                       float* w) {
    size_t P = (size_t)W * H;
#pragma omp parallel for schedule(dynamic, 64)
    for (long long pb = 0; pb < (long long)(P * B); ++pb) {
        int b = (int)(pb / P);
        size_t pix = (size_t)pb % P;
        int i = (int)(pix / H), j = (int)(pix % H);
        float pixel[2] = {(float)i, (float)j};
        for (int s = 0; s < K; ++s) {
            size_t off = (size_t)s + (size_t)K * (size_t)pb;
            int index = idx[off];
            if (index < 0) { w[off] = 0.0f; continue; }
            size_t po = 3 * ((size_t)index + (size_t)N * b);
            size_t so = sdB > 1 ? 2 * ((size_t)index + (size_t)N * b) : 2 * (size_t)index;
            w[off] = orc_ewa_weight(pixel, (float)W, (float)H, f, &pts[po], &nrm[po], &sd[so], smoothing, NULL);
        }
    }
}

/* gradEwaKernel (splattingCuda.cu:114-193): gradient only where the
 * unclamped weight is <= 1; FP64 accumulation, then rounded once. */
void orc_splat_backward(int B, int W, int H, int K, float f, const float* gin, const int* idx,
                        const float* pts, const float* nrm, const float* sd, int sdB, int N,
                        float smoothing, float* gp, float* gn, float* gs) {
    size_t nP = (size_t)N * B * 3, nS = (size_t)(sdB > 1 ? N * B : N) * 2;
    double* ap = (double*)calloc(nP, sizeof(double));
    double* an = (double*)calloc(nP, sizeof(double));
    double* as = (double*)calloc(nS, sizeof(double));
    size_t P = (size_t)W * H;
    for (int b = 0; b < B; ++b)
        for (size_t pix = 0; pix < P; ++pix) {
            int i = (int)(pix / H), j = (int)(pix % H);
            float pixel[2] = {(float)i, (float)j};
            for (int s = 0; s < K; ++s) {
                size_t off = (size_t)s + (size_t)K * (pix + P * b);
                int index = idx[off];
                if (index < 0) continue;
                size_t po = 3 * ((size_t)index + (size_t)N * b);
                size_t so = sdB > 1 ? 2 * ((size_t)index + (size_t)N * b) : 2 * (size_t)index;
                float raw;
                orc_ewa_weight(pixel, (float)W, (float)H, f, &pts[po], &nrm[po], &sd[so], smoothing, &raw);
                if (!(raw <= 1.0f)) continue;
                double a[3], c[3], d[2];
                orc_ewa_grad(pixel, (float)W, (float)H, f, &pts[po], &nrm[po], &sd[so], smoothing, a, c, d);
                double g = gin[off];
                for (int k = 0; k < 3; ++k) { ap[po + k] += a[k] * g; an[po + k] += c[k] * g; }
                as[so] += d[0] * g;
                as[so + 1] += d[1] * g;
            }
        }
    for (size_t i = 0; i < nP; ++i) { gp[i] = (float)ap[i]; gn[i] = (float)an[i]; }
    for (size_t i = 0; i < nS; ++i) gs[i] = (float)as[i];
    free(ap); free(an); free(as);
}

/* ------------------------------------------------------------------------
 * Depth compositing (alphacompositing.cuh:6-68, alphacompositingGrad.cuh)
 * ---------------------------------------------------------------------- */
static void signed_distances(float* dist, const float* pixel, float W, float H, float f, int K,
                             const int* idx, const float* pts, const float* nrm) {
    float wd[3], dir[3];
    backprojf(W, H, f, pixel, wd);
    float invNorm = (float)(1.0 / (double)norm3f(wd));
    for (int i = 0; i < 3; ++i) dir[i] = (wd[i] * invNorm) * -1.0f;
    for (int k = 0; k < K; ++k) {
        dist[k] = ORC_ZMAX;
        int id = idx[k];
        if (id < 0) continue;
        const float* p = &pts[3 * (size_t)id];
        const float* n = &nrm[3 * (size_t)id];
        float d = dot3f(p, n) / dot3f(dir, n);
        if (d > 0.0f) dist[k] = d;
    }
}

static void arg_sort(int* order, const float* v, int K) {
    for (int i = 0; i < K; ++i) order[i] = i;
    for (int i = 1; i < K; ++i) {
        int index = order[i];
        float value = v[index];
        int j = i;
        while (j > 0 && v[order[j - 1]] > value) { order[j] = order[j - 1]; --j; }
        order[j] = index;
    }
}

static void blend(float* out, const int* order, const float* w, int K) {
    float rem = 1.0f;
    for (int i = 0; i < K; ++i) {
        int id = order[i];
        float wt = w[id];
        out[id] = rem * wt;
        rem = (float)((double)rem * (1.0 - (double)wt));
    }
}

void orc_filter_forward(int B, int W, int H, int K, const int* idx, const float* w, float f,
                        int pB, int N, const float* pts, const float* nrm, float* out,
                        int* order) {
    size_t P = (size_t)W * H;
#pragma omp parallel for schedule(static)
    for (long long pb = 0; pb < (long long)(P * B); ++pb) {
        int b = (int)(pb / P);
        size_t pix = (size_t)pb % P;
        float pixel[2] = {(float)(pix / H), (float)(pix % H)};
        size_t e = (size_t)K * (size_t)pb;
        size_t po = pB > 1 ? 3 * (size_t)N * b : 0;
        int ord[64];
        float dist[64];
        signed_distances(dist, pixel, (float)W, (float)H, f, K, &idx[e], &pts[po], &nrm[po]);
        arg_sort(ord, dist, K);
        blend(&out[e], ord, &w[e], K);
        if (order)
            for (int k = 0; k < K; ++k) order[e + k] = ord[k];
    }
}

void orc_filter_backward(int B, int W, int H, int K, const int* idx, const float* w,
                         const float* gin, float f, int pB, int N, const float* pts,
                         const float* nrm, float* out) {
    size_t P = (size_t)W * H;
#pragma omp parallel for schedule(static)
    for (long long pb = 0; pb < (long long)(P * B); ++pb) {
        int b = (int)(pb / P);
        size_t pix = (size_t)pb % P;
        float pixel[2] = {(float)(pix / H), (float)(pix % H)};
        size_t e = (size_t)K * (size_t)pb;
        size_t po = pB > 1 ? 3 * (size_t)N * b : 0;
        int ord[64];
        float dist[64], fw[64];
        signed_distances(dist, pixel, (float)W, (float)H, f, K, &idx[e], &pts[po], &nrm[po]);
        arg_sort(ord, dist, K);
        blend(fw, ord, &w[e], K);
        const float eps = 1e-4f;
        for (int k = 0; k < K; ++k) {
            int kdx = ord[k];
            float g = 0.0f;
            for (int i = k; i < K; ++i) {
                int id = ord[i];
                float den = (i == k) ? w[e + kdx] : -(1.0f - w[e + kdx]);
                if (fabsf(den) > eps) g += gin[e + id] * fw[id] / den;
            }
            out[e + kdx] = g;
        }
    }
}

/* ------------------------------------------------------------------------
 * Interpolation (interpolationCuda.cu:5-129)
 * ---------------------------------------------------------------------- */
void orc_interp_forward(int B, int W, int H, int K, const int* idx, const float* w, int aB, int N,
                        int C, const float* attr, float* out) {
    size_t P = (size_t)W * H;
#pragma omp parallel for schedule(static)
    for (long long pb = 0; pb < (long long)(P * B); ++pb) {
        int b = (int)(pb / P);
        float* o = &out[(size_t)C * (size_t)pb];
        for (int c = 0; c < C; ++c) o[c] = 0.0f;
        for (int s = 0; s < K; ++s) {
            size_t so = (size_t)s + (size_t)K * (size_t)pb;
            int id = idx[so];
            if (id < 0) continue;
            const float* a = &attr[aB > 1 ? (size_t)C * ((size_t)id + (size_t)N * b) : (size_t)C * id];
            for (int c = 0; c < C; ++c) o[c] += w[so] * a[c];
        }
    }
}

void orc_interp_backward(int B, int W, int H, int K, const float* gin, const int* idx,
                         const float* w, int aB, int N, int C, const float* attr, float* gw,
                         float* ga) {
    size_t P = (size_t)W * H;
    size_t nA = (size_t)(aB > 1 ? N * B : N) * C;
    double* acc = (double*)calloc(nA, sizeof(double));
    for (size_t pb = 0; pb < P * B; ++pb) {
        int b = (int)(pb / P);
        for (int s = 0; s < K; ++s) {
            size_t so = (size_t)s + (size_t)K * pb;
            int id = idx[so];
            gw[so] = 0.0f;
            if (id < 0) continue;
            size_t ao = aB > 1 ? (size_t)C * ((size_t)id + (size_t)N * b) : (size_t)C * id;
            float g = 0.0f;
            for (int c = 0; c < C; ++c) {
                float gi = gin[(size_t)C * pb + c];
                acc[ao + c] += (double)gi * w[so];
                g += gi * attr[ao + c];
            }
            gw[so] = g;
        }
    }
    for (size_t i = 0; i < nA; ++i) ga[i] = (float)acc[i];
    free(acc);
}

/* ------------------------------------------------------------------------
 * The EWA -> compositing -> interpolation chain in FP64 for fixed indices:
 * the reference for central differences of the CUDA backward kernels.  The
 * formulas are those of the FP32 functions above, every operation in double:
 * the weight (ewaSplatting.cuh:8-91, clamped at 1 as ewaSplatting.cuh:90),
 * the signed distance along the pixel ray (alphacompositing.cuh:6-30), the
 * stable insertion sort (alphacompositing.cuh:32-56), the front-to-back blend
 * (alphacompositing.cuh:58-68) and the weighted attribute sum
 * (interpolationCuda.cu:5-46).
 * ---------------------------------------------------------------------- */
static double ewa_weight64(const double* pixel, double W, double H, double F, const double* p, const double* n,
                           const double* sd, double sm) {
    double s0 = -(p[0] * F) / p[2] + W / 2.0, s1 = (p[1] * F) / p[2] + H / 2.0;
    double a0 = (W - 2.0 * s0) / (2.0 * F), a1 = -(H - 2.0 * s1) / (2.0 * F);
    double x0[3] = {a0 - 1.0 / F, a1, 1.0}, x1[3] = {a0, a1 + 1.0 / F, 1.0};
    double c = dot3d(p, n);
    double k0 = c / dot3d(x0, n), k1 = c / dot3d(x1, n);
    double t0[3], t1[3];
    for (int i = 0; i < 3; ++i) { t0[i] = k0 * x0[i] - p[i]; t1[i] = k1 * x1[i] - p[i]; }
    double al = sqrt(dot3d(t0, t0));
    double u0[3] = {t0[0] / al, t0[1] / al, t0[2] / al}, u1[3];
    cross3d(u0, n, u1);
    double be = dot3d(t1, u0), ga = dot3d(t1, u1);
    double J00 = 1.0 / al, J01 = -be / (al * ga), J11 = 1.0 / ga;
    double S0 = sd[0] * sd[0], S1 = sd[1] * sd[1];
    double V00 = J00 * J00 * S0 + J01 * J01 * S1 + sm, V01 = J01 * J11 * S1, V11 = J11 * J11 * S1 + sm;
    double vdet = V00 * V11 - V01 * V01;
    double d0 = pixel[0] - s0, d1 = pixel[1] - s1;
    double e = (d0 * (V11 * d0 - V01 * d1) + d1 * (V00 * d1 - V01 * d0)) / vdet;
    double G = exp(-0.5 * e) / (2.0 * ORC_PI * sqrt(vdet) * fabs(al * ga));
    return G < 1.0 ? G : 1.0;
}

void orc_chain64_forward(int W, int H, int K, double f, const int* idx, int N, const double* pts,
                         const double* nrm, const double* sd, double smoothing, int C, const double* attr,
                         double* img) {
    (void)N;
#pragma omp parallel for schedule(static)
    for (long long pix = 0; pix < (long long)W * H; ++pix) {
        int i = (int)(pix / H), j = (int)(pix % H);
        double pixel[2] = {(double)i, (double)j};
        const int* ix = &idx[(size_t)K * pix];
        double w[64], dist[64], out[64];
        int ord[64];
        double wd[3] = {((double)W - 2.0 * i) / (2.0 * f), -((double)H - 2.0 * j) / (2.0 * f), 1.0};
        double nw = sqrt(dot3d(wd, wd));
        double dir[3] = {-wd[0] / nw, -wd[1] / nw, -wd[2] / nw};
        for (int k = 0; k < K; ++k) {
            w[k] = 0.0;
            dist[k] = (double)ORC_ZMAX;
            int id = ix[k];
            if (id < 0) continue;
            const double* p = &pts[3 * (size_t)id];
            const double* n = &nrm[3 * (size_t)id];
            w[k] = ewa_weight64(pixel, W, H, f, p, n, &sd[2 * (size_t)id], smoothing);
            double d = dot3d(p, n) / dot3d(dir, n);
            if (d > 0.0) dist[k] = d;
        }
        for (int k = 0; k < K; ++k) ord[k] = k;
        for (int k = 1; k < K; ++k) {
            int index = ord[k];
            int m = k;
            while (m > 0 && dist[ord[m - 1]] > dist[index]) { ord[m] = ord[m - 1]; --m; }
            ord[m] = index;
        }
        double rem = 1.0;
        for (int k = 0; k < K; ++k) {
            out[ord[k]] = rem * w[ord[k]];
            rem *= 1.0 - w[ord[k]];
        }
        double* o = &img[(size_t)C * pix];
        for (int c = 0; c < C; ++c) o[c] = 0.0;
        for (int k = 0; k < K; ++k) {
            int id = ix[k];
            if (id < 0) continue;
            for (int c = 0; c < C; ++c) o[c] += out[k] * attr[(size_t)C * id + c];
        }
    }
}

/* ------------------------------------------------------------------------
 * Shading (diffuseShading.cuh, diffuseShadingGrad.cuh, shadingCuda.cu)
 * ---------------------------------------------------------------------- */
void orc_shade_forward(int B, int P, int L, const float* dirs, const float* I, int IB,
                       const float* nrm, const float* dif, float* out) {
    for (int b = 0; b < B; ++b)
        for (int p = 0; p < P; ++p) {
            size_t o = 3 * ((size_t)p + (size_t)P * b);
            const float* n = &nrm[o];
            const float* d = &dif[o];
            float r[3] = {0.0f, 0.0f, 0.0f};
            for (int l = 0; l < L; ++l) {
                const float* dir = &dirs[3 * ((size_t)l + (size_t)L * b)];
                const float* col = &I[3 * ((size_t)l + (IB > 1 ? (size_t)L * b : 0))];
                float cs = 0.0f;
                for (int i = 0; i < 3; ++i) cs += dir[i] * n[i];
                cs = fmaxf(0.0f, cs);
                for (int i = 0; i < 3; ++i) r[i] += (float)((double)d[i] / ORC_PI * (double)col[i] * (double)cs);
            }
            for (int i = 0; i < 3; ++i) out[o + i] = r[i];
        }
}

void orc_shade_backward(int B, int P, int L, const float* gin, const float* dirs, const float* I,
                        int IB, const float* nrm, const float* dif, float* gdirs, float* gI,
                        float* gn, float* gd) {
    const float pif = (float)ORC_PI;
    for (int b = 0; b < B; ++b)
        for (int p = 0; p < P; ++p) {
            size_t o = 3 * ((size_t)p + (size_t)P * b);
            const float* n = &nrm[o];
            const float* d = &dif[o];
            const float* g = &gin[o];
            for (int l = 0; l < L; ++l) {
                size_t dl = 3 * ((size_t)l + (size_t)L * b);
                size_t il = 3 * ((size_t)l + (IB > 1 ? (size_t)L * b : 0));
                const float* dir = &dirs[dl];
                const float* col = &I[il];
                float cs = 0.0f, dc[3];
                for (int i = 0; i < 3; ++i) { cs += dir[i] * n[i]; dc[i] = d[i] * col[i]; }
                if (!(cs > 0.0f)) continue;
                float scaling = (float)((double)fmaxf(0.0f, cs) / ORC_PI);
                float gdc = 0.0f; /* sum_i g_i * dc_i */
                for (int i = 0; i < 3; ++i) gdc += g[i] * dc[i];
                for (int j = 0; j < 3; ++j) {
                    float gdir = 0.0f, gnn = 0.0f;
                    for (int i = 0; i < 3; ++i) {
                        gdir += g[i] * ((dc[i] * n[j]) / pif);
                        gnn += g[i] * ((dc[i] * dir[j]) / pif);
                    }
                    gdirs[dl + j] += gdir;
                    gn[o + j] += gnn;
                    gI[il + j] += g[j] * (d[j] * scaling);
                    gd[o + j] += g[j] * (col[j] * scaling);
                }
                (void)gdc;
            }
        }
}

/* buildShMatrix (diffuseShading.cuh:39-71), row-major M(i,j) = m[4i+j] */
static void sh_matrix(const float* c, float* M) {
    const float c1 = 0.429043f, c2 = 0.511664f, c3 = 0.743125f, c4 = 0.886227f, c5 = 0.247708f;
    M[0] = c1 * c[8]; M[4] = c1 * c[4]; M[8] = c1 * c[7]; M[12] = c2 * c[3];
    M[1] = c1 * c[4]; M[5] = -c1 * c[8]; M[9] = c1 * c[5]; M[13] = c2 * c[1];
    M[2] = c1 * c[7]; M[6] = c1 * c[5]; M[10] = c3 * c[6]; M[14] = c2 * c[2];
    M[3] = c2 * c[3]; M[7] = c2 * c[1]; M[11] = c2 * c[2]; M[15] = c4 * c[0] - c5 * c[6];
}

static void sh_unit(const float* n, float* v, float* normOut) {
    const float eps = 1e-5f;
    float norm = norm3f(n);
    v[0] = 0.0f; v[1] = 0.0f; v[2] = 0.0f; v[3] = 1.0f;
    if (norm > eps) {
        float inv = (float)(1.0 / (double)norm);
        v[0] = n[0] * inv; v[1] = n[1] * inv; v[2] = n[2] * inv; v[3] = norm * inv;
    }
    *normOut = norm;
}

static float sh_eval(const float* c, const float* n) {
    float M[16], v[4], norm, y[4];
    sh_matrix(c, M);
    sh_unit(n, v, &norm);
    for (int i = 0; i < 4; ++i) {
        y[i] = 0.0f;
        for (int j = 0; j < 4; ++j) y[i] += v[j] * M[4 * j + i];
    }
    float r = 0.0f;
    for (int i = 0; i < 4; ++i) r += y[i] * v[i];
    return r;
}

void orc_shade_sh_forward(int B, int P, const float* coef, int cB, const float* nrm,
                          const float* dif, float* out) {
    for (int b = 0; b < B; ++b)
        for (int p = 0; p < P; ++p) {
            size_t o = 3 * ((size_t)p + (size_t)P * b);
            for (int i = 0; i < 3; ++i) {
                const float* c = &coef[cB > 1 ? 9 * (i + 3 * b) : 9 * i];
                out[o + i] = (float)((double)(dif[o + i] * sh_eval(c, &nrm[o])) / ORC_PI);
            }
        }
}

/* shadingShBackwardKernel (shadingCuda.cu:244-293): the normal gradient of
 * channel i keeps only component i of that channel's normal gradient. */
void orc_shade_sh_backward(int B, int P, const float* gin, const float* coef, int cB,
                           const float* nrm, const float* dif, float* gc, float* gn, float* gd) {
    const float c1 = 0.429043f, c2 = 0.511664f, c3 = 0.743125f, c4 = 0.886227f, c5 = 0.247708f;
    for (int b = 0; b < B; ++b)
        for (int p = 0; p < P; ++p) {
            size_t o = 3 * ((size_t)p + (size_t)P * b);
            const float* n = &nrm[o];
            for (int i = 0; i < 3; ++i) {
                size_t co = cB > 1 ? 9 * (i + 3 * b) : 9 * i;
                const float* c = &coef[co];
                float M[16], v[4], norm;
                sh_matrix(c, M);
                sh_unit(n, v, &norm);
                float irr = sh_eval(c, n);
                /* dE/dv = (M + M^T) v ; dE/dM = v v^T */
                float gv[4];
                for (int r = 0; r < 4; ++r) {
                    float a = 0.0f, t = 0.0f;
                    for (int j = 0; j < 4; ++j) { a += M[4 * r + j] * v[j]; t += M[4 * j + r] * v[j]; }
                    gv[r] = a + t;
                }
                float gM[16];
                for (int r = 0; r < 4; ++r)
                    for (int j = 0; j < 4; ++j) gM[4 * r + j] = v[r] * v[j];
                float gsh[9];
                gsh[0] = c4 * gM[15];
                gsh[1] = c2 * (gM[7] + gM[13]);
                gsh[2] = c2 * (gM[14] + gM[11]);
                gsh[3] = c2 * (gM[12] + gM[3]);
                gsh[4] = c1 * (gM[4] + gM[1]);
                gsh[5] = c1 * (gM[9] + gM[6]);
                gsh[6] = c3 * gM[10] - c5 * gM[15];
                gsh[7] = c1 * (gM[8] + gM[2]);
                gsh[8] = c1 * (gM[0] - gM[5]);
                /* normalisation Jacobian (I - n n^T / |n|^2) / |n| */
                float gnv[3] = {0.0f, 0.0f, 0.0f};
                if (norm > 1e-5f) {
                    float inv = (float)(1.0 / (double)norm);
                    float inv3 = inv * inv * inv;
                    for (int r = 0; r < 3; ++r) {
                        float s = 0.0f;
                        for (int j = 0; j < 3; ++j) {
                            float Jrj = ((r == j) ? inv : 0.0f) - n[r] * n[j] * inv3;
                            s += Jrj * gv[j];
                        }
                        gnv[r] = s;
                    }
                }
                float g = gin[o + i], dd = dif[o + i];
                gd[o + i] = (float)((double)(g * irr) / ORC_PI);
                gn[o + i] = (float)((double)(g * dd * gnv[i]) / ORC_PI);
                for (int j = 0; j < 9; ++j) gc[co + j] += (float)((double)(g * dd * gsh[j]) / ORC_PI);
            }
        }
}

/* ------------------------------------------------------------------------
 * FMM sampler
 * ---------------------------------------------------------------------- */

/* IsotropicEigenFunctor (samplingCuda.cu:133-162): per-splat isotropic
 * std-dev, float/double mixture as written. */
static float splat_bandwidth(float W, float H, float f, const float* p, const float* n,
                             const float* sd, float sm) {
    ewa_frame F;
    ewa_framef(W, H, f, p, n, sd, sm, &F);
    const float* V = F.V;
    float det = V[0] * V[3] - V[1] * V[2];
    float inv = (float)(1.0 / (double)det);
    float iV[4] = {V[3] * inv, -V[1] * inv, -V[2] * inv, V[0] * inv};
    float tr = iV[0] + iV[3];
    float idet = iV[0] * iV[3] - iV[1] * iV[2];
    float root = sqrtf((float)(0.25 * (double)(tr * tr) - (double)idet));
    float l1 = (float)(0.5 * (double)tr + (double)root);
    float l2 = (float)(0.5 * (double)tr - (double)root);
    float lk = fminf(l1, l2);
    return (float)fmin(1.0, 1.0 / (double)sqrtf(lk));
}

/* Mean of the per-splat bandwidths over all N splats of the view
 * (MeanFunctor, samplingCuda.cu:165-195).  Summed in 2^-32 fixed point so
 * that the result does not depend on the summation order. */
float orc_view_bandwidth(int W, int H, float f, int N, const float* pts, const float* nrm,
                         const float* sd, float smoothing) {
    unsigned long long sum = 0;
    long long count = 0;
    for (int i = 0; i < N; ++i) {
        float hk = splat_bandwidth((float)W, (float)H, f, &pts[3 * (size_t)i], &nrm[3 * (size_t)i], &sd[2 * (size_t)i], smoothing);
        if (isfinite(hk)) {
            sum += (unsigned long long)llrint((double)hk * 4294967296.0);
            count += 1;
        }
    }
    if (count == 0) return NAN;
    return (float)((double)sum / 4294967296.0 / (double)count);
}

/* samplingCuda.cu:251-252 */
float orc_cull_radius(float h, float precision, int flavour) {
    float norm = (float)(2.0 * ORC_PI * (double)sqrtf(h));
    double a = flavour == ORC_LIBM ? -log((double)precision) : -(double)orc_det_logf(precision);
    double b = (double)xlogf(norm, flavour);
    return (float)(sqrt(2.0) * (double)h * sqrt(a - b));
}

struct orc_tree {
    int n;
    unsigned* keys;
    int* ids;
    float* leafxy;
    int *left, *right, *parent, *count, *first, *last, *degree;
    long* offset;
    float *box, *centre, *trunc;
    float* coef;
    long ncoef;
    float h, precision;
    int demoted;
};

void orc_tree_free(orc_tree* t) {
    if (!t) return;
    free(t->keys); free(t->ids); free(t->leafxy);
    free(t->left); free(t->right); free(t->parent); free(t->count); free(t->first); free(t->last);
    free(t->degree); free(t->offset); free(t->box); free(t->centre); free(t->trunc); free(t->coef);
    free(t);
}

int orc_tree_size(const orc_tree* t) { return t ? t->n : 0; }
long orc_tree_num_coefs(const orc_tree* t) { return t ? t->ncoef : 0; }

/* expandBits (buildRadixTree.cuh:18-28) */
static inline unsigned expand_bits(unsigned v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}
static inline unsigned morton_coord(float s, float lo, float hi) {
    float src = (s - lo) / (hi - lo);
    float c = fminf(fmaxf(src * 1024.0f, 0.0f), 1023.0f);
    return (unsigned)c;
}
static inline int clz64(unsigned long long x) {
    if (x == 0) return 64;
    int n = 0;
    while (!(x & 0x8000000000000000ull)) { x <<= 1; ++n; }
    return n;
}
static inline unsigned long long key64(const unsigned* keys, int i) {
    return ((unsigned long long)keys[i] << 32) | (unsigned)i;
}
static inline int cpref(const unsigned* keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    return clz64(key64(keys, i) ^ key64(keys, j));
}

/* Karras (2012) radix tree over the unique 64-bit keys (key << 32 | rank):
 * determineRange / findSplit (buildRadixTree.cuh:76-167) and the child
 * links of HierarchyFunctor (buildDynamicRadixTree.cuh:91-123). */
static void karras(const unsigned* keys, int n, int* left, int* right, int* parent, int* first, int* last,
                   int* count) {
    int L0 = n - 1;
    for (int idx = 0; idx < n - 1; ++idx) {
        int lo, hi;
        if (idx == 0) { lo = 0; hi = n - 1; }
        else {
            int dL = cpref(keys, n, idx, idx - 1), dR = cpref(keys, n, idx, idx + 1);
            int d = (dR > dL) ? 1 : -1;
            int dmin = dL < dR ? dL : dR;
            int lmax = 2;
            while (cpref(keys, n, idx, idx + d * lmax) > dmin) lmax <<= 1;
            int l = 0;
            for (int s = lmax >> 1; s > 0; s >>= 1)
                if (cpref(keys, n, idx, idx + (l + s) * d) > dmin) l += s;
            int j = idx + l * d;
            lo = d < 0 ? j : idx;
            hi = d < 0 ? idx : j;
        }
        int dnode = cpref(keys, n, lo, hi);
        int split = lo, stride = hi - lo;
        do {
            stride = (stride + 1) >> 1;
            int mid = split + stride;
            if (mid < hi && cpref(keys, n, lo, mid) > dnode) split = mid;
        } while (stride > 1);
        int lc = split, rc = split + 1;
        if (lo == split) lc += L0;
        if (hi == split + 1) rc += L0;
        left[idx] = lc; right[idx] = rc;
        if (parent) { parent[lc] = idx; parent[rc] = idx; }
        if (first) first[idx] = lo;
        if (last) last[idx] = hi;
        if (count) count[idx] = hi - lo + 1;
    }
}

void orc_karras_from_keys(int n, const unsigned* keys, int* left, int* right) {
    karras(keys, n, left, right, NULL, NULL, NULL, NULL);
}

unsigned orc_expand_bits(unsigned v) { return expand_bits(v); }

/* hermiteError (hermitefmm.cuh:184-195) */
static float hermite_error(float r, float nr, unsigned ph, int fl) {
    if (r >= 1.0f) return r;
    float a, b;
    if (fl == ORC_LIBM) {
        a = nr / powf(1.0f - r, 2.0f);
        b = powf(r, (float)ph) / sqrtf(facf(ph));
        float c = b * b;
        float d = 2.0f * (1.0f - powf(r, (float)ph)) * b;
        return a * (c + d);
    }
    float om = 1.0f - r;
    a = nr / (om * om);
    float rp = ipowf(r, ph);
    b = rp / sqrtf(facf(ph));
    float c = b * b;
    float d = 2.0f * (1.0f - rp) * b;
    return a * (c + d);
}

/* hermiteFunction (hermitefmm.cuh:35-47) */
void orc_hermite_function(float t, int ph, int fl, float* out) {
    float e = xexpf(-(t * t), fl);
    out[0] = e;
    out[1] = (2.0f * t) * e;
    for (int n = 2; n <= ph; ++n) out[n] = (2.0f * t) * out[n - 1] - (2.0f * (float)(n - 1)) * out[n - 2];
}

float orc_hermite_error(float r, float nr, int ph, int fl) { return hermite_error(r, nr, (unsigned)ph, fl); }

static int cmp_key_id(const void* a, const void* b) {
    const unsigned long long* x = (const unsigned long long*)a;
    const unsigned long long* y = (const unsigned long long*)b;
    return (*x > *y) - (*x < *y);
}

orc_tree* orc_tree_build(int W, int H, float f, int N, const float* pts, float h, float radius,
                         float precision, int maxDegree, long coefPool, int fl) {
    orc_tree* t = (orc_tree*)calloc(1, sizeof(orc_tree));
    if (!t) return NULL;
    t->h = h;
    t->precision = precision;
    float bounds[4] = {-radius, (float)W + radius, -radius, (float)H + radius};
    /* culling (CullingFunctor, samplingCuda.cu:41-54) in ascending id order */
    unsigned long long* kv = (unsigned long long*)malloc(sizeof(unsigned long long) * (size_t)(N > 0 ? N : 1));
    float* sxy = (float*)malloc(sizeof(float) * 2 * (size_t)(N > 0 ? N : 1));
    int n = 0;
    for (int i = 0; i < N; ++i) {
        const float* p = &pts[3 * (size_t)i];
        float s[2];
        screenf((float)W, (float)H, f, p, s);
        int vis = (p[2] <= 0.0f);
        for (int a = 0; a < 2; ++a) { vis &= (bounds[2 * a] <= s[a]); vis &= (bounds[2 * a + 1] >= s[a]); }
        if (!vis) continue;
        /* MortonTransformFunctor (buildRadixTree.cuh:231-246): x weight 2, y weight 1 */
        unsigned key = 2u * expand_bits(morton_coord(s[0], bounds[0], bounds[1])) +
                       expand_bits(morton_coord(s[1], bounds[2], bounds[3]));
        kv[n] = ((unsigned long long)key << 32) | (unsigned)i;
        sxy[2 * (size_t)i] = s[0];
        sxy[2 * (size_t)i + 1] = s[1];
        ++n;
    }
    /* stable sort by key == sort by (key, id) since ids ascend */
    qsort(kv, (size_t)n, sizeof(unsigned long long), cmp_key_id);
    t->n = n;
    int M = n > 0 ? 2 * n - 1 : 1;
    t->keys = (unsigned*)malloc(sizeof(unsigned) * (size_t)(n > 0 ? n : 1));
    t->ids = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    t->leafxy = (float*)malloc(sizeof(float) * 2 * (size_t)(n > 0 ? n : 1));
    t->left = (int*)malloc(sizeof(int) * M);
    t->right = (int*)malloc(sizeof(int) * M);
    t->parent = (int*)malloc(sizeof(int) * M);
    t->count = (int*)malloc(sizeof(int) * M);
    t->first = (int*)malloc(sizeof(int) * M);
    t->last = (int*)malloc(sizeof(int) * M);
    t->degree = (int*)malloc(sizeof(int) * M);
    t->offset = (long*)malloc(sizeof(long) * M);
    t->box = (float*)malloc(sizeof(float) * 4 * M);
    t->centre = (float*)malloc(sizeof(float) * 2 * M);
    t->trunc = (float*)malloc(sizeof(float) * M);
    for (int i = 0; i < n; ++i) {
        t->keys[i] = (unsigned)(kv[i] >> 32);
        t->ids[i] = (int)(unsigned)(kv[i] & 0xFFFFFFFFu);
        t->leafxy[2 * i] = sxy[2 * (size_t)t->ids[i]];
        t->leafxy[2 * i + 1] = sxy[2 * (size_t)t->ids[i] + 1];
    }
    free(kv);
    free(sxy);
    t->ncoef = 0;
    t->coef = (float*)malloc(sizeof(float));
    if (n == 0) return t;
    int L0 = n - 1; /* first leaf node */
    for (int i = 0; i < M; ++i) t->parent[i] = -1;
    /* leaves (LeafNodeFunctor, buildDynamicRadixTree.cuh:46-73) */
    for (int i = 0; i < n; ++i) {
        int v = L0 + i;
        t->left[v] = -1; t->right[v] = -1; t->count[v] = 1; t->degree[v] = 0;
        t->first[v] = i; t->last[v] = i;
        float x = t->leafxy[2 * i], y = t->leafxy[2 * i + 1];
        t->box[4 * v] = x; t->box[4 * v + 1] = y; t->box[4 * v + 2] = x; t->box[4 * v + 3] = y;
        t->centre[2 * v] = x; t->centre[2 * v + 1] = y;
    }
    /* Karras hierarchy (determineRange / findSplit, buildRadixTree.cuh:76-167) */
    karras(t->keys, n, t->left, t->right, t->parent, t->first, t->last, t->count);
    /* bottom-up (InternalNodeFunctor, buildDynamicRadixTree.cuh:155-221) in
     * post order; centres indexed [2*child] */
    if (n > 1) {
        int* stack = (int*)malloc(sizeof(int) * 2 * (size_t)M);
        int* post = (int*)malloc(sizeof(int) * (size_t)M);
        int sp = 0, np = 0;
        stack[sp++] = 0;
        while (sp) {
            int v = stack[--sp];
            if (v >= L0) continue;
            post[np++] = v;
            stack[sp++] = t->left[v];
            stack[sp++] = t->right[v];
        }
        for (int q = np - 1; q >= 0; --q) {
            int v = post[q];
            int a = t->left[v], b = t->right[v];
            t->box[4 * v] = fminf(t->box[4 * a], t->box[4 * b]);
            t->box[4 * v + 1] = fminf(t->box[4 * a + 1], t->box[4 * b + 1]);
            t->box[4 * v + 2] = fmaxf(t->box[4 * a + 2], t->box[4 * b + 2]);
            t->box[4 * v + 3] = fmaxf(t->box[4 * a + 3], t->box[4 * b + 3]);
            unsigned ca = (unsigned)t->count[a], cb = (unsigned)t->count[b], nc = ca + cb;
            for (int k = 0; k < 2; ++k)
                t->centre[2 * v + k] = ((float)ca * t->centre[2 * a + k] + (float)cb * t->centre[2 * b + k]) / (float)nc;
            float mn = 0.0f;
            for (int k = 0; k < 2; ++k) {
                float x = fmaxf(t->centre[2 * v + k] - t->box[4 * v + k], t->box[4 * v + 2 + k] - t->centre[2 * v + k]);
                mn = fmaxf(mn, x);
            }
            float r = mn / h;
            int d0 = t->degree[a] > t->degree[b] ? t->degree[a] : t->degree[b];
            unsigned deg = (unsigned)(d0 > 0 ? d0 : 0);
            while (deg <= (unsigned)maxDegree && hermite_error(r, (float)nc, deg, fl) > precision && r < 1.0f) deg += 1;
            t->degree[v] = (r < 1.0f && deg <= (unsigned)maxDegree) ? (int)deg : -1;
        }
        free(stack);
        free(post);
    }
    /* coefficient offsets in node order; internal nodes only (a leaf's
     * single coefficient is the constant 1).  Nodes past the pool fall back
     * to degree -1: offsets are the exclusive scan of all internal nodes'
     * sizes, and a node is demoted iff offset + size exceeds the pool. */
    long total = 0, kept = 0;
    for (int v = 0; v < M; ++v) {
        t->offset[v] = -1;
        if (v >= L0 || t->degree[v] < 0) continue;
        long sz = (long)(t->degree[v] + 1) * (t->degree[v] + 1);
        long off = total; /* exclusive scan over all internal nodes */
        total += sz;
        if (coefPool >= 0 && off + sz > coefPool) { t->degree[v] = -1; t->demoted++; continue; }
        t->offset[v] = off;
        kept = off + sz;
    }
    t->ncoef = kept;
    free(t->coef);
    t->coef = (float*)calloc((size_t)(total > 0 ? total : 1), sizeof(float));
    /* P2M (HermiteCoefficientFunctor + shiftLeafHermiteExpansion,
     * buildDynamicRadixTree.cuh:280-313, hermitefmm.cuh:119-138): each node
     * sums its leaves' terms in leaf order.  The libm flavour evaluates each
     * term as the reference does, (1 * s0^a * s1^b) / (a! b!); the
     * deterministic flavour (the GPU's arithmetic) builds t_a = s^a / a! by
     * the recurrence t_a = (t_{a-1} * s) / a and adds fma(tx_a, ty_b, C_ab). */
    float sq = sqrtf(2.0f * h * h);
    float isq = 1.0f / sq;
    static const float inv_int[ORC_MAXDEGREE + 1] = {0.0f, 1.0f / 1, 1.0f / 2, 1.0f / 3, 1.0f / 4, 1.0f / 5,
                                                     1.0f / 6, 1.0f / 7, 1.0f / 8, 1.0f / 9, 1.0f / 10, 1.0f / 11,
                                                     1.0f / 12, 1.0f / 13, 1.0f / 14, 1.0f / 15, 1.0f / 16};
    for (int v = 0; v < L0; ++v) {
        int p = t->degree[v];
        if (p < 0) continue;
        float* C = &t->coef[t->offset[v]];
        for (int i = t->first[v]; i <= t->last[v]; ++i) {
            float s0, s1;
            if (fl == ORC_LIBM) {
                s0 = (t->leafxy[2 * i] - t->centre[2 * v]) / sq;
                s1 = (t->leafxy[2 * i + 1] - t->centre[2 * v + 1]) / sq;
            } else {
                s0 = (t->leafxy[2 * i] - t->centre[2 * v]) * isq;
                s1 = (t->leafxy[2 * i + 1] - t->centre[2 * v + 1]) * isq;
            }
            if (fl == ORC_LIBM) {
                for (int x = 0; x <= p; ++x)
                    for (int y = 0; y <= p; ++y) {
                        float term = (1.0f * (xpowi(s0, (unsigned)x, fl) * xpowi(s1, (unsigned)y, fl))) / (facf((unsigned)x) * facf((unsigned)y));
                        C[x * (p + 1) + y] += term;
                    }
            } else {
                float tx[ORC_MAXDEGREE + 1], ty[ORC_MAXDEGREE + 1];
                tx[0] = 1.0f;
                ty[0] = 1.0f;
                for (int a = 1; a <= p; ++a) {
                    tx[a] = (tx[a - 1] * s0) * inv_int[a];
                    ty[a] = (ty[a - 1] * s1) * inv_int[a];
                }
                for (int x = 0; x <= p; ++x)
                    for (int y = 0; y <= p; ++y) C[x * (p + 1) + y] = fmaf(tx[x], ty[y], C[x * (p + 1) + y]);
            }
        }
    }
    /* truncation radius per node (truncate, evaluateDynamicRadixTree.cuh:118-126) */
    for (int v = 0; v < M; ++v) {
        float nn = (float)(unsigned)t->count[v];
        t->trunc[v] = sqrtf((-2.0f * (h * h)) * xlogf(precision / nn, fl));
    }
    return t;
}

void orc_tree_export(const orc_tree* t, unsigned* keys, int* ids, int* left, int* right,
                     int* parent, int* count, int* degree, float* centre, float* box,
                     float* leafxy) {
    int n = t->n, M = n > 0 ? 2 * n - 1 : 0;
    if (keys) memcpy(keys, t->keys, sizeof(unsigned) * (size_t)n);
    if (ids) memcpy(ids, t->ids, sizeof(int) * (size_t)n);
    if (leafxy) memcpy(leafxy, t->leafxy, sizeof(float) * 2 * (size_t)n);
    if (left) memcpy(left, t->left, sizeof(int) * (size_t)M);
    if (right) memcpy(right, t->right, sizeof(int) * (size_t)M);
    if (parent) memcpy(parent, t->parent, sizeof(int) * (size_t)M);
    if (count) memcpy(count, t->count, sizeof(int) * (size_t)M);
    if (degree) memcpy(degree, t->degree, sizeof(int) * (size_t)M);
    if (centre) memcpy(centre, t->centre, sizeof(float) * 2 * (size_t)M);
    if (box) memcpy(box, t->box, sizeof(float) * 4 * (size_t)M);
}

/* evluateHermite (hermitefmm.cuh:213-237) with hermiteFunction (:35-47) */
static float hermite_eval(const orc_tree* t, int v, const float* q, int fl) {
    float sq = sqrtf(2.0f * t->h * t->h);
    float tx, ty;
    if (fl == ORC_LIBM) {  /* the reference divides */
        tx = (q[0] - t->centre[2 * v]) / sq;
        ty = (q[1] - t->centre[2 * v + 1]) / sq;
    } else {  /* the deterministic flavour multiplies by 1 / sq */
        float isq = 1.0f / sq;
        tx = (q[0] - t->centre[2 * v]) * isq;
        ty = (q[1] - t->centre[2 * v + 1]) * isq;
    }
    int p = t->degree[v];
    float hx[ORC_MAXDEGREE + 1], hy[ORC_MAXDEGREE + 1];
    float ex = xexpf(-(tx * tx), fl), ey = xexpf(-(ty * ty), fl);
    hx[0] = ex; hx[1] = (2.0f * tx) * ex;
    hy[0] = ey; hy[1] = (2.0f * ty) * ey;
    for (int k = 2; k <= p; ++k) {
        hx[k] = (2.0f * tx) * hx[k - 1] - (2.0f * (float)(k - 1)) * hx[k - 2];
        hy[k] = (2.0f * ty) * hy[k - 1] - (2.0f * (float)(k - 1)) * hy[k - 2];
    }
    if (v >= t->n - 1) return 0.0f + (1.0f * hx[0]) * hy[0]; /* leaf: coefficient 1 */
    const float* C = &t->coef[t->offset[v]];
    float w = 0.0f;
    if (fl == ORC_LIBM) {
        /* the reference's order: sum_a sum_b (C_ab h_a) h_b */
        for (int a = 0; a <= p; ++a)
            for (int b = 0; b <= p; ++b) w += (C[a * (p + 1) + b] * hx[a]) * hy[b];
        return w;
    }
    /* row-factored with fused multiply-adds: sum_a h_a (sum_b C_ab h_b) */
    for (int a = 0; a <= p; ++a) {
        float s = 0.0f;
        for (int b = 0; b <= p; ++b) s = fmaf(C[a * (p + 1) + b], hy[b], s);
        w = fmaf(hx[a], s, w);
    }
    return w;
}

static int truncated(const orc_tree* t, int v, const float* q) {
    float d2 = 0.0f;
    for (int k = 0; k < 2; ++k) {
        float cl = fminf(fmaxf(q[k], t->box[4 * v + k]), t->box[4 * v + 2 + k]);
        float d = q[k] - cl;
        d2 += d * d;
    }
    float r = t->trunc[v];
    return !(d2 < r * r);
}

/* getWeight / accumulateSubtree (evaluateDynamicRadixTree.cuh:129-242) */
float orc_tree_node_weight(const orc_tree* t, int node, const float* q, int fl) {
    if (t->degree[node] > -1) return hermite_eval(t, node, q, fl);
    int rootparent = t->parent[node];
    int v = node;
    float w = 0.0f;
    do {
        while (t->degree[v] < 0 && !truncated(t, v, q)) v = t->left[v];
        if (t->degree[v] > -1) w += hermite_eval(t, v, q, fl);
        int pidx = t->parent[v];
        while (pidx != rootparent && v == t->right[pidx]) { v = pidx; pidx = t->parent[pidx]; }
        if (pidx != rootparent) v = t->right[pidx];
    } while (t->parent[v] != rootparent);
    return w;
}

double orc_tree_direct_weight(const orc_tree* t, int node, const double* q) {
    double s = 0.0, h = t->h;
    for (int i = t->first[node]; i <= t->last[node]; ++i) {
        double dx = q[0] - t->leafxy[2 * i], dy = q[1] - t->leafxy[2 * i + 1];
        s += exp(-(dx * dx + dy * dy) / (2.0 * h * h));
    }
    return s;
}

/* insertSample (sequentialPoissonRadixTree.cuh:15-41) */
static void insert_sample(int index, float key, int* indices, float* keys, int K) {
    for (int i = 0; i < K; ++i) {
        if (key < keys[i]) {
            int ti = indices[i]; indices[i] = index; index = ti;
            float tk = keys[i]; keys[i] = key; key = tk;
        }
        if (index == -1) break;
    }
}

/* sequentialPoissonKernel (sequentialPoissonDynamicTree.cuh:56-196) with the
 * per-pixel capacity map held as the traces of the earlier rounds (a node
 * only ever appears at its own depth), which is the hash map of
 * sampleRadixTree.cuh:29-88 without its overflow.
 * Leaf size (no reference counterpart): a round descends while its node
 * holds more than M = max(K, leaf) splats and then order-samples over all of
 * the node's splats; leaf <= K is the reference's rule (M = K).  The round's
 * uniforms are M per round: uniforms[(pixel * R + r) * M + k], or Philox
 * blocks r * ceil(M / 4) + k / 4. */
int orc_tree_sample_leaf(const orc_tree* t, int W, int H, int K, int leaf, float precision, const float* uniforms,
                         uint64_t seed, uint32_t view, int x0, int x1, int fl, int* indices) {
    int R = orc_num_rounds(K);
    int M = leaf > K ? leaf : K;
    if (M > 64) return -2;
    int n = t->n;
    int status = 0;
    if (x1 > W) x1 = W;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = x0; i < x1; ++i) {
        int tnode[8][ORC_STACK];
        float tprob[8][ORC_STACK], tcap[8][ORC_STACK];
        int tlen[8];
        float keys[64];
        float u[64];
        for (int j = 0; j < H; ++j) {
            size_t pixel = (size_t)j + (size_t)H * i;
            int* out = &indices[(size_t)K * pixel];
            for (int k = 0; k < K; ++k) { out[k] = -1; keys[k] = INFINITY; }
            if (n == 0) continue;
            float q[2] = {(float)i, (float)j};
            float total = fmaxf(0.0f, orc_tree_node_weight(t, 0, q, fl));
            if (total < precision) continue;
            for (int r = 0; r < R && r < 8; ++r) {
                if (uniforms) memcpy(u, &uniforms[((size_t)pixel * R + r) * M], sizeof(float) * M);
                else orc_philox_uniforms(seed, view, (uint32_t)pixel, (uint32_t)r, M, u);
                int v = 0, d = 0;
                tnode[r][0] = 0; tprob[r][0] = 1.0f;
                while (t->count[v] > M) {
                    int a = t->left[v], b = t->right[v];
                    float w0 = fmaxf(0.0f, orc_tree_node_weight(t, a, q, fl));
                    float w1 = fmaxf(0.0f, orc_tree_node_weight(t, b, q, fl));
                    float sum = 0.0f;
                    sum += w0; sum += w1;
                    w0 = w0 / sum; w1 = w1 / sum;
                    float c0 = 1.0f, c1 = 1.0f;
                    for (int rr = r - 1; rr >= 0; --rr)
                        if (d + 1 < tlen[rr] && tnode[rr][d + 1] == a) { c0 = tcap[rr][d + 1]; break; }
                    for (int rr = r - 1; rr >= 0; --rr)
                        if (d + 1 < tlen[rr] && tnode[rr][d + 1] == b) { c1 = tcap[rr][d + 1]; break; }
                    float s0 = w0 * c0, s1 = w1 * c1;
                    ++d;
                    if (d >= ORC_STACK) { status = -1; break; }
                    if (s0 < s1) { tnode[r][d] = b; tprob[r][d] = w1; v = b; }
                    else { tnode[r][d] = a; tprob[r][d] = w0; v = a; }
                }
                if (d >= ORC_STACK) break;
                tlen[r] = d + 1;
                float prob = 1.0f;
                for (int m = d; m >= 0; --m) {
                    float cap = 1.0f;
                    for (int rr = r - 1; rr >= 0; --rr)
                        if (m < tlen[rr] && tnode[rr][m] == tnode[r][m]) { cap = tcap[rr][m]; break; }
                    tcap[r][m] = fmaxf(0.0f, cap - prob);
                    prob *= tprob[r][m];
                }
                int c = t->count[v], f0 = t->first[v];
                for (int k = 0; k < c; ++k) {
                    int leafNode = n - 1 + f0 + k;
                    float pw = fmaxf(0.0f, orc_tree_node_weight(t, leafNode, q, fl));
                    insert_sample(t->ids[f0 + k], u[k] / pw, out, keys, K);
                }
            }
        }
    }
    return status;
}

int orc_tree_sample(const orc_tree* t, int W, int H, int K, float precision, const float* uniforms,
                    uint64_t seed, uint32_t view, int x0, int x1, int fl, int* indices) {
    return orc_tree_sample_leaf(t, W, H, K, 0, precision, uniforms, seed, view, x0, x1, fl, indices);
}

/* The same estimator evaluated directly in FP64 (the CPU baseline the
 * reference lacks): node masses are sums of exp(-|q - y|^2 / (2 h^2)) over
 * the node's leaves in double, skipping subtrees whose box misses the
 * node's truncation circle (the truncation of getWeight,
 * evaluateDynamicRadixTree.cuh:118-126) but using no Hermite expansion; the
 * greedy descent, the capacities and the order-sampling keys follow
 * orc_tree_sample in double. */
static double direct_trunc64(const orc_tree* t, int node, const double* q) {
    int stack[ORC_STACK + 2];
    int sp = 0;
    double s = 0.0, i2h2 = 1.0 / (2.0 * (double)t->h * (double)t->h);
    stack[sp++] = node;
    while (sp) {
        int v = stack[--sp];
        if (v >= t->n - 1) {
            int i = v - (t->n - 1);
            double dx = q[0] - t->leafxy[2 * i], dy = q[1] - t->leafxy[2 * i + 1];
            s += exp(-(dx * dx + dy * dy) * i2h2);
            continue;
        }
        double cx = fmin(fmax(q[0], t->box[4 * v]), t->box[4 * v + 2]);
        double cy = fmin(fmax(q[1], t->box[4 * v + 1]), t->box[4 * v + 3]);
        double r = t->trunc[v];
        if ((q[0] - cx) * (q[0] - cx) + (q[1] - cy) * (q[1] - cy) >= r * r) continue;
        if (sp + 2 > ORC_STACK + 2) return s;  /* deeper than any tree built here */
        stack[sp++] = t->right[v];
        stack[sp++] = t->left[v];
    }
    return s;
}

int orc_tree_sample_fp64_leaf(const orc_tree* t, int W, int H, int K, int leaf, double precision, uint64_t seed,
                              uint32_t view, int x0, int x1, int* indices) {
    int R = orc_num_rounds(K);
    int M = leaf > K ? leaf : K;
    if (M > 64) return -2;
    int n = t->n;
    int status = 0;
    if (x1 > W) x1 = W;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = x0; i < x1; ++i) {
        int tnode[8][ORC_STACK];
        double tprob[8][ORC_STACK], tcap[8][ORC_STACK];
        int tlen[8];
        double keys[64];
        float u[64];
        for (int j = 0; j < H; ++j) {
            size_t pixel = (size_t)j + (size_t)H * i;
            int* out = &indices[(size_t)K * pixel];
            for (int k = 0; k < K; ++k) { out[k] = -1; keys[k] = INFINITY; }
            if (n == 0) continue;
            double q[2] = {(double)i, (double)j};
            if (direct_trunc64(t, 0, q) < precision) continue;
            for (int r = 0; r < R && r < 8; ++r) {
                orc_philox_uniforms(seed, view, (uint32_t)pixel, (uint32_t)r, M, u);
                int v = 0, d = 0;
                tnode[r][0] = 0; tprob[r][0] = 1.0;
                while (t->count[v] > M) {
                    int a = t->left[v], b = t->right[v];
                    double w0 = direct_trunc64(t, a, q), w1 = direct_trunc64(t, b, q);
                    double sum = w0 + w1;
                    w0 /= sum; w1 /= sum;
                    double c0 = 1.0, c1 = 1.0;
                    for (int rr = r - 1; rr >= 0; --rr)
                        if (d + 1 < tlen[rr] && tnode[rr][d + 1] == a) { c0 = tcap[rr][d + 1]; break; }
                    for (int rr = r - 1; rr >= 0; --rr)
                        if (d + 1 < tlen[rr] && tnode[rr][d + 1] == b) { c1 = tcap[rr][d + 1]; break; }
                    double s0 = w0 * c0, s1 = w1 * c1;
                    ++d;
                    if (d >= ORC_STACK) { status = -1; break; }
                    if (s0 < s1) { tnode[r][d] = b; tprob[r][d] = w1; v = b; }
                    else { tnode[r][d] = a; tprob[r][d] = w0; v = a; }
                }
                if (d >= ORC_STACK) break;
                tlen[r] = d + 1;
                double prob = 1.0;
                for (int m = d; m >= 0; --m) {
                    double cap = 1.0;
                    for (int rr = r - 1; rr >= 0; --rr)
                        if (m < tlen[rr] && tnode[rr][m] == tnode[r][m]) { cap = tcap[rr][m]; break; }
                    tcap[r][m] = fmax(0.0, cap - prob);
                    prob *= tprob[r][m];
                }
                int c = t->count[v], f0 = t->first[v];
                for (int k = 0; k < c; ++k) {
                    double dx = q[0] - t->leafxy[2 * (f0 + k)], dy = q[1] - t->leafxy[2 * (f0 + k) + 1];
                    double pw = exp(-(dx * dx + dy * dy) / (2.0 * (double)t->h * (double)t->h));
                    double key = (double)u[k] / pw;
                    int index = t->ids[f0 + k];
                    for (int s = 0; s < K; ++s) {
                        if (key < keys[s]) {
                            int ti = out[s]; out[s] = index; index = ti;
                            double tk = keys[s]; keys[s] = key; key = tk;
                        }
                        if (index == -1) break;
                    }
                }
            }
        }
    }
    return status;
}

int orc_tree_sample_fp64(const orc_tree* t, int W, int H, int K, double precision, uint64_t seed, uint32_t view,
                         int x0, int x1, int* indices) {
    return orc_tree_sample_fp64_leaf(t, W, H, K, 0, precision, seed, view, x0, x1, indices);
}

/* Stochastic mode (no reference counterpart): each of the K draws of a
 * pixel descends from the root, stepping into a child with probability
 * m_child / (m_left + m_right) (masses by getWeight), until it reaches a
 * leaf; the draw's path probability q is the product of the chosen ratios.
 * Uniform for draw k at depth d: Philox counter (pixel, view,
 * 2^31 | k << 8 | d / 4, 0), component d % 4; step left iff u <= ratio.
 * A draw whose two child masses are both zero, or that is still above the
 * leaves after 64 levels (the trace depth of the deterministic sampler), and
 * every draw of a pixel whose root mass is below precision, give index -1 and
 * q = 0. */
int orc_tree_sample_stochastic(const orc_tree* t, int W, int H, int K, float precision, uint64_t seed,
                               uint32_t view, int x0, int x1, int fl, int* indices, float* probs) {
    int n = t->n;
    int status = 0;
    if (x1 > W) x1 = W;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = x0; i < x1; ++i) {
        for (int j = 0; j < H; ++j) {
            size_t pixel = (size_t)j + (size_t)H * i;
            int* out = &indices[(size_t)K * pixel];
            float* pq = &probs[(size_t)K * pixel];
            for (int k = 0; k < K; ++k) { out[k] = -1; pq[k] = 0.0f; }
            if (n == 0) continue;
            float q[2] = {(float)i, (float)j};
            if (fmaxf(0.0f, orc_tree_node_weight(t, 0, q, fl)) < precision) continue;
            for (int k = 0; k < K; ++k) {
                int v = 0, d = 0;
                float prob = 1.0f;
                uint32_t c[4];
                int ok = 1;
                while (v < n - 1) {
                    if ((d & 3) == 0) {
                        c[0] = (uint32_t)pixel; c[1] = view; c[2] = 0x80000000u | ((uint32_t)k << 8) | (uint32_t)(d >> 2); c[3] = 0;
                        philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
                    }
                    float u = (float)((c[d & 3] >> 8) + 1u) * 0x1p-24f;
                    int a = t->left[v], b = t->right[v];
                    float w0 = fmaxf(0.0f, orc_tree_node_weight(t, a, q, fl));
                    float w1 = fmaxf(0.0f, orc_tree_node_weight(t, b, q, fl));
                    float sum = 0.0f;
                    sum += w0; sum += w1;
                    if (!(sum > 0.0f)) { ok = 0; break; }
                    float r0 = w0 / sum;
                    if (u <= r0) { prob *= r0; v = a; }
                    else { prob *= w1 / sum; v = b; }
                    if (++d >= ORC_STACK && v < n - 1) { ok = 0; status = -1; break; }
                }
                if (ok) { out[k] = t->ids[v - (n - 1)]; pq[k] = prob; }
            }
        }
    }
    return status;
}

/* Candidate entries of one pixel over all rounds: the descent is
 * deterministic (masses and capacities do not depend on the uniforms), so the
 * sampled indices are the K smallest keys u/p over these entries.  Writes
 * splat ids and leaf masses p, returns the number of entries (<= R*K). */
int orc_tree_candidates(const orc_tree* t, int K, float precision, int i, int j, int fl, int* ids,
                        float* p) {
    int R = orc_num_rounds(K);
    int n = t->n, m = 0;
    if (n == 0) return 0;
    float q[2] = {(float)i, (float)j};
    if (fmaxf(0.0f, orc_tree_node_weight(t, 0, q, fl)) < precision) return 0;
    int tnode[8][ORC_STACK], tlen[8];
    float tprob[8][ORC_STACK], tcap[8][ORC_STACK];
    for (int r = 0; r < R && r < 8; ++r) {
        int v = 0, d = 0;
        tnode[r][0] = 0; tprob[r][0] = 1.0f;
        while (t->count[v] > K) {
            int a = t->left[v], b = t->right[v];
            float w0 = fmaxf(0.0f, orc_tree_node_weight(t, a, q, fl));
            float w1 = fmaxf(0.0f, orc_tree_node_weight(t, b, q, fl));
            float sum = 0.0f;
            sum += w0; sum += w1;
            w0 = w0 / sum; w1 = w1 / sum;
            float c0 = 1.0f, c1 = 1.0f;
            for (int rr = r - 1; rr >= 0; --rr)
                if (d + 1 < tlen[rr] && tnode[rr][d + 1] == a) { c0 = tcap[rr][d + 1]; break; }
            for (int rr = r - 1; rr >= 0; --rr)
                if (d + 1 < tlen[rr] && tnode[rr][d + 1] == b) { c1 = tcap[rr][d + 1]; break; }
            ++d;
            if (d >= ORC_STACK) return -1;
            if (w0 * c0 < w1 * c1) { tnode[r][d] = b; tprob[r][d] = w1; v = b; }
            else { tnode[r][d] = a; tprob[r][d] = w0; v = a; }
        }
        tlen[r] = d + 1;
        float prob = 1.0f;
        for (int mm = d; mm >= 0; --mm) {
            float cap = 1.0f;
            for (int rr = r - 1; rr >= 0; --rr)
                if (mm < tlen[rr] && tnode[rr][mm] == tnode[r][mm]) { cap = tcap[rr][mm]; break; }
            tcap[r][mm] = fmaxf(0.0f, cap - prob);
            prob *= tprob[r][mm];
        }
        for (int k = 0; k < t->count[v]; ++k) {
            int leafNode = n - 1 + t->first[v] + k;
            ids[m] = t->ids[t->first[v] + k];
            p[m] = fmaxf(0.0f, orc_tree_node_weight(t, leafNode, q, fl));
            ++m;
        }
    }
    return m;
}

int orc_sample_view(int W, int H, float f, int N, const float* pts, const float* nrm,
                    const float* sd, int K, float smoothing, float precision, float h_in,
                    const float* uniforms, uint64_t seed, uint32_t view, int flavour,
                    int* indices, float* stats) {
    float h = h_in > 0.0f ? h_in : orc_view_bandwidth(W, H, f, N, pts, nrm, sd, smoothing);
    float radius = orc_cull_radius(h, precision, flavour);
    orc_tree* t = orc_tree_build(W, H, f, N, pts, h, radius, precision, ORC_MAXDEGREE, -1, flavour);
    if (!t) return -2;
    int st = orc_tree_sample(t, W, H, K, precision, uniforms, seed, view, 0, W, flavour, indices);
    if (stats) {
        stats[0] = h;
        stats[1] = radius;
        stats[2] = (float)t->n;
        stats[3] = (float)t->ncoef;
    }
    orc_tree_free(t);
    return st;
}

/* scatterKernel (pixelGatherCuda.cu:7-36): each sample takes its splat's
 * channels; samples with index -1 stay 0 (the reference zero-fills the output
 * and skips them). */
void orc_pixel_scatter(int B, int W, int H, int K, const int* idx, int N, int C, const float* values,
                       float* out) {
    size_t per_view = (size_t)W * H * K;
    for (int b = 0; b < B; ++b)
        for (size_t t = 0; t < per_view; ++t) {
            size_t s = t + per_view * (size_t)b;
            int id = idx[s];
            for (int c = 0; c < C; ++c)
                out[s * (size_t)C + c] = (id >= 0 && id < N) ? values[((size_t)id + (size_t)N * b) * C + c] : 0.0f;
        }
}

/* gatherKernel (pixelGatherCuda.cu:78-110): each sample's channels added to
 * its splat; the reference adds with atomics in no fixed order, here in
 * sample order (the order the deterministic GPU mode reproduces). */
void orc_pixel_gather(int B, int W, int H, int K, const int* idx, int N, int C, const float* values,
                      float* out) {
    size_t per_view = (size_t)W * H * K;
    for (size_t i = 0; i < (size_t)B * N * C; ++i) out[i] = 0.0f;
    for (int b = 0; b < B; ++b)
        for (size_t t = 0; t < per_view; ++t) {
            size_t s = t + per_view * (size_t)b;
            int id = idx[s];
            if (id < 0 || id >= N) continue;
            for (int c = 0; c < C; ++c) out[((size_t)id + (size_t)N * b) * C + c] += values[s * (size_t)C + c];
        }
}

/* nearestsamples.nearest (nearestSamplesCuda.cu:355-454): the surface
 * sample of a pixel is its largest-weight sample (first on ties,
 * :375-386); the pixel's other valid samples are candidates for it.  The
 * reference merges them under a lock (order dependent); this restatement
 * keeps, per splat, the M distinct candidates of smallest distance, ties by
 * index. */
static float orc_pdist(const float* pts, int a, int b) {
    float dx = pts[3 * a] - pts[3 * b], dy = pts[3 * a + 1] - pts[3 * b + 1], dz = pts[3 * a + 2] - pts[3 * b + 2];
    return sqrtf(dx * dx + dy * dy + dz * dz);
}

void orc_nearest_samples(int B, int W, int H, int K, const int* idx, const float* w, int N, const float* pts, int M,
                         int* out) {
    float* bd = (float*)malloc(sizeof(float) * (size_t)N * M);
    for (size_t i = 0; i < (size_t)N * M; ++i) out[i] = -1;
    int* cnt = (int*)calloc((size_t)N, sizeof(int));
    size_t P = (size_t)B * W * H;
    for (size_t pix = 0; pix < P; ++pix) {
        const int* id = idx + pix * K;
        const float* wt = w + pix * K;
        int s = id[0];
        float sw = wt[0];
        for (int k = 1; k < K; ++k)
            if (wt[k] > sw) { sw = wt[k]; s = id[k]; }
        if (s < 0 || s >= N) continue;
        for (int k = 0; k < K; ++k) {
            int c = id[k];
            if (c < 0 || c >= N || c == s) continue;
            int* li = out + (size_t)s * M;
            float* ld = bd + (size_t)s * M;
            int m = cnt[s], dup = 0;
            for (int q = 0; q < m; ++q) dup |= li[q] == c;
            if (dup) continue;
            float d = orc_pdist(pts, s, c);
            if (m == M && !(d < ld[M - 1] || (d == ld[M - 1] && c < li[M - 1]))) continue;
            int q = m < M ? m++ : M - 1;
            while (q > 0 && (d < ld[q - 1] || (d == ld[q - 1] && c < li[q - 1]))) {
                ld[q] = ld[q - 1];
                li[q] = li[q - 1];
                --q;
            }
            ld[q] = d;
            li[q] = c;
            cnt[s] = m;
        }
    }
    free(cnt);
    free(bd);
}
