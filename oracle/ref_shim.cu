// Reference shim: a host-only C-ABI library compiled from the REFERENCE's own
// headers, included in place from the reference checkout (never copied).
//
// Test infrastructure only.  It pins the CPU oracle (oracle/uds_oracle.c)
// against the reference's own arithmetic: every `__host__ __device__` function
// of the splatting path is called as written (EWA weight and gradient,
// signed distances / arg-sort / blending / blending gradient, Lambert and SH
// shading and their gradients, camera-space transform and its gradient, the
// Hermite series, the error bound, box helpers).  The reference's
// `__device__`-only tree and sampler helpers (expandBits / mortonND,
// determineRange / findSplit, hash-map capacities, nextLeaf, insertSample,
// getWeight / accumulateSubtree / truncate) are made host-callable by
// re-declaring `__device__` as `__host__ __device__` before the headers are
// included.  Where the reference only exists as a kernel body or a thrust call
// (culling, bandwidth reduction, leaf init, bottom-up fan-in, P2M driver,
// sampling kernel body) this file restates the loop around the reference's
// own helper functions, in the sequential order a single thread would run it.
//
// Built by oracle/Makefile into oracle/_ref/libudsref.so (git-ignored); it is
// only used to generate the golden fixtures under tests/golden/.
#include <cuda_runtime.h>
#include <curand_kernel.h>
#include <thrust/device_vector.h>
#include <thrust/transform.h>
#include <thrust/sort.h>
#include <thrust/sequence.h>
#include <thrust/unique.h>
#include <thrust/fill.h>
#include <thrust/copy.h>
#include <thrust/execution_policy.h>
#include <thrust/functional.h>

// CCCL 3 removed these adaptable-function bases; the reference's functors
// derive from them.  Empty stand-ins are enough for host use.
namespace thrust {
template <typename A, typename R> struct unary_function { typedef A argument_type; typedef R result_type; };
template <typename A, typename B, typename R> struct binary_function {
    typedef A first_argument_type; typedef B second_argument_type; typedef R result_type; };
}

// Make the reference's __device__-only helpers callable from host code.
#undef __device__
#define __device__ __location__(host) __location__(device)

#include "ewaSplattingGrad.cuh"
#include "alphacompositingGrad.cuh"
#include "diffuseShading.cuh"
#include "diffuseShadingGrad.cuh"
#include "transformationGrad.cuh"
#include "buildDynamicRadixTree.cuh"
#include "sequentialPoissonDynamicTree.cuh"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

// 64-bit Morton key wrapper: the reference's commonUpperBits(size_t, size_t)
// returns 0 outside device code, so determineRange / findSplit are
// instantiated with this key type and reach the count-leading-zeros below
// through argument-dependent lookup.
namespace refkey {
struct Key64 {
    unsigned long long v;
};
inline bool operator==(const Key64& a, const Key64& b) { return a.v == b.v; }
inline int commonUpperBits(const Key64& a, const Key64& b) {
    unsigned long long x = a.v ^ b.v;
    if (x == 0) return 64;
    int n = 0;
    while (!(x & 0x8000000000000000ull)) { x <<= 1; ++n; }
    return n;
}
}  // namespace refkey

typedef float real;

extern "C" {

// ---------------------------------------------------------------- projection
void ref_to_screenspace(int n, float W, float H, float f, const float* pts, float* out) {
    for (int i = 0; i < n; ++i) {
        const ConstVector3<real> p(&pts[3 * i]);
        Vector2<real> s = toScreenspace<real>(W, H, f, p);
        out[2 * i] = s[0];
        out[2 * i + 1] = s[1];
    }
}

// --------------------------------------------------------------------- EWA
// Per (pixel, splat) pair: clamped weight (evaluateEWAWeight) and the
// unclamped Gaussian (evaluteGaussian) that gates the gradient.
void ref_ewa_pairs(int n, const float* pix, float W, float H, float f, const float* pts,
                   const float* nrm, const float* sd, float smoothing, float* w, float* raw) {
    for (int i = 0; i < n; ++i) {
        const ConstVector2<real> pixel(&pix[2 * i]);
        const ConstVector3<real> p(&pts[3 * i]);
        const ConstVector3<real> nn(&nrm[3 * i]);
        const ConstVector2<real> s(&sd[2 * i]);
        w[i] = evaluateEWAWeight<real>(pixel, W, H, f, p, nn, s, smoothing);
        Vector2<real> sp = toScreenspace<real>(W, H, f, p);
        Matrix22<real> invJk = buildInverseJacobian<real>(W, H, f, sp, p, nn);
        Matrix22<real> Vk = buildCovariance<real>(invJk, s, smoothing);
        raw[i] = evaluteGaussian<real>(pixel, sp, invJk, Vk);
    }
}

void ref_ewa_grad_pairs(int n, const float* pix, float W, float H, float f, const float* pts,
                        const float* nrm, const float* sd, float smoothing, float* gp, float* gn,
                        float* gs) {
    for (int i = 0; i < n; ++i) {
        const ConstVector2<real> pixel(&pix[2 * i]);
        const ConstVector3<real> p(&pts[3 * i]);
        const ConstVector3<real> nn(&nrm[3 * i]);
        const ConstVector2<real> s(&sd[2 * i]);
        Vector3<real> a, b;
        Vector2<real> c;
        gradEWAWeight<real>(a, b, c, pixel, W, H, f, p, nn, s, smoothing);
        for (int k = 0; k < 3; ++k) { gp[3 * i + k] = a[k]; gn[3 * i + k] = b[k]; }
        gs[2 * i] = c[0];
        gs[2 * i + 1] = c[1];
    }
}

// splatting.forward (splattingCuda.cu ewaKernel body, host order)
void ref_splat_forward(int B, int W, int H, int K, float f, const int* idx, const float* pts,
                       const float* nrm, const float* sd, int sdBatch, int N, float smoothing,
                       float* weights) {
    for (int b = 0; b < B; ++b)
        for (int i = 0; i < W; ++i)
            for (int j = 0; j < H; ++j) {
                float pb[2] = {(float)i, (float)j};
                const ConstVector2<real> pixel(pb);
                for (int s = 0; s < K; ++s) {
                    size_t off = (size_t)s + (size_t)K * ((size_t)j + (size_t)H * ((size_t)i + (size_t)W * b));
                    int index = idx[off];
                    if (index < 0) { weights[off] = 0.0f; continue; }
                    size_t po = 3 * ((size_t)index + (size_t)N * b);
                    size_t so = sdBatch > 1 ? 2 * ((size_t)index + (size_t)N * b) : 2 * (size_t)index;
                    const ConstVector3<real> p(&pts[po]);
                    const ConstVector3<real> nn(&nrm[po]);
                    const ConstVector2<real> sdv(&sd[so]);
                    weights[off] = evaluateEWAWeight(pixel, (float)W, (float)H, f, p, nn, sdv, smoothing);
                }
            }
}

// splatting.backward (gradEwaKernel body, sequential accumulation)
void ref_splat_backward(int B, int W, int H, int K, float f, const float* gin, const int* idx,
                        const float* pts, const float* nrm, const float* sd, int sdBatch, int N,
                        float smoothing, float* gpts, float* gnrm, float* gsd) {
    for (int b = 0; b < B; ++b)
        for (int i = 0; i < W; ++i)
            for (int j = 0; j < H; ++j) {
                float pb[2] = {(float)i, (float)j};
                const ConstVector2<real> pixel(pb);
                for (int s = 0; s < K; ++s) {
                    size_t off = (size_t)s + (size_t)K * ((size_t)j + (size_t)H * ((size_t)i + (size_t)W * b));
                    int index = idx[off];
                    if (index < 0) continue;
                    size_t po = 3 * ((size_t)index + (size_t)N * b);
                    size_t so = sdBatch > 1 ? 2 * ((size_t)index + (size_t)N * b) : 2 * (size_t)index;
                    const ConstVector3<real> p(&pts[po]);
                    const ConstVector3<real> nn(&nrm[po]);
                    const ConstVector2<real> sdv(&sd[so]);
                    float Wf = (float)W, Hf = (float)H;
                    Vector2<real> sp = toScreenspace(Wf, Hf, f, p);
                    Matrix22<real> invJk = buildInverseJacobian<real>(Wf, Hf, f, sp, p, nn);
                    Matrix22<real> Vk = buildCovariance<real>(invJk, sdv, smoothing);
                    real weight = evaluteGaussian<real>(pixel, sp, invJk, Vk);
                    if (weight <= 1.0) {
                        Vector3<real> a, c;
                        Vector2<real> d;
                        gradEWAWeight<real>(a, c, d, pixel, Wf, Hf, f, p, nn, sdv, smoothing);
                        float g = gin[off];
                        for (int k = 0; k < 3; ++k) { gpts[po + k] += a[k] * g; gnrm[po + k] += c[k] * g; }
                        gsd[so] += d[0] * g;
                        gsd[so + 1] += d[1] * g;
                    }
                }
            }
}

// ------------------------------------------------------ depth compositing
void ref_filter_forward(int B, int W, int H, int K, const int* idx, const float* w, float f,
                        int ptsBatch, int N, const float* pts, const float* nrm, float* out) {
    std::vector<int> sorted(K);
    for (int b = 0; b < B; ++b)
        for (int x = 0; x < W; ++x)
            for (int y = 0; y < H; ++y) {
                float pb[2] = {(float)x, (float)y};
                const ConstVector2<real> pixel(pb);
                for (int i = 0; i < K; ++i) sorted[i] = i;
                size_t e = (size_t)K * ((size_t)y + (size_t)H * ((size_t)x + (size_t)W * b));
                size_t po = ptsBatch > 1 ? 3 * (size_t)N * b : 0;
                signedDistances(&out[e], pixel, (float)W, (float)H, f, (unsigned)K, &idx[e], &pts[po], &nrm[po]);
                argSort(sorted.data(), &out[e], (unsigned)K);
                blending(&out[e], sorted.data(), &w[e], (unsigned)K);
            }
}

void ref_filter_backward(int B, int W, int H, int K, const int* idx, const float* w,
                         const float* gin, float f, int ptsBatch, int N, const float* pts,
                         const float* nrm, float* out) {
    std::vector<int> sorted(K);
    for (int b = 0; b < B; ++b)
        for (int x = 0; x < W; ++x)
            for (int y = 0; y < H; ++y) {
                float pb[2] = {(float)x, (float)y};
                const ConstVector2<real> pixel(pb);
                for (int i = 0; i < K; ++i) sorted[i] = i;
                size_t e = (size_t)K * ((size_t)y + (size_t)H * ((size_t)x + (size_t)W * b));
                size_t po = ptsBatch > 1 ? 3 * (size_t)N * b : 0;
                signedDistances(&out[e], pixel, (float)W, (float)H, f, (unsigned)K, &idx[e], &pts[po], &nrm[po]);
                argSort(sorted.data(), &out[e], (unsigned)K);
                gradBlending(&out[e], sorted.data(), &w[e], &gin[e], (unsigned)K);
            }
}

// ----------------------------------------------------------------- shading
void ref_shade_forward(int P, int L, int B, const float* dirs, const float* I, int IBatch,
                       const float* nrm, const float* dif, float* out) {
    int perView = P / B;
    for (int p = 0; p < P; ++p) {
        int b = p / perView;
        const ConstVector3<real> n(&nrm[3 * (size_t)p]);
        const ConstVector3<real> d(&dif[3 * (size_t)p]);
        Vector3<real> r = shading(&dirs[3 * (size_t)L * b], &I[IBatch > 1 ? 3 * (size_t)L * b : 0], (unsigned)L, n, d);
        for (int k = 0; k < 3; ++k) out[3 * (size_t)p + k] = r[k];
    }
}

// gradShading with the atomics replaced by sequential sums (same terms).
void ref_shade_backward(int P, int L, int B, const float* gin, const float* dirs, const float* I,
                        int IBatch, const float* nrm, const float* dif, float* gdirs, float* gI,
                        float* gn, float* gd) {
    int perView = P / B;
    for (int p = 0; p < P; ++p) {
        int b = p / perView;
        const ConstVector3<real> g(&gin[3 * (size_t)p]);
        const ConstVector3<real> n(&nrm[3 * (size_t)p]);
        const ConstVector3<real> d(&dif[3 * (size_t)p]);
        const float* D = &dirs[3 * (size_t)L * b];
        const float* C = &I[IBatch > 1 ? 3 * (size_t)L * b : 0];
        float* GD = &gdirs[3 * (size_t)L * b];
        float* GC = &gI[IBatch > 1 ? 3 * (size_t)L * b : 0];
        PointerVector3<real> gno(&gn[3 * (size_t)p]);
        PointerVector3<real> gdo(&gd[3 * (size_t)p]);
        for (int l = 0; l < L; ++l) {
            const ConstVector3<real> dir(&D[3 * l]);
            const ConstVector3<real> col(&C[3 * l]);
            Matrix33<real> a, bb, c, e;
            real cs = gradLambert(a, bb, c, e, dir, col, n, d);
            if (cs > 0) {
                Vector3<real> pgd = g * a;
                Vector3<real> pgc = g * bb;
                for (int k = 0; k < 3; ++k) { GD[3 * l + k] += pgd[k]; GC[3 * l + k] += pgc[k]; }
                gno += g * c;
                gdo += g * e;
            }
        }
    }
}

void ref_shade_sh_forward(int P, int B, const float* coeffs, int cBatch, const float* nrm,
                          const float* dif, float* out) {
    int perView = P / B;
    for (int p = 0; p < P; ++p) {
        int b = p / perView;
        const ConstVector3<real> n(&nrm[3 * (size_t)p]);
        for (int i = 0; i < 3; ++i) {
            const float* c = &coeffs[cBatch > 1 ? 9 * (i + 3 * b) : 9 * i];
            out[3 * (size_t)p + i] = dif[3 * (size_t)p + i] * shadingSh(c, n) / M_PI;
        }
    }
}

void ref_shade_sh_backward(int P, int B, const float* gin, const float* coeffs, int cBatch,
                           const float* nrm, const float* dif, float* gc, float* gn, float* gd) {
    int perView = P / B;
    for (int p = 0; p < P; ++p) {
        int b = p / perView;
        const ConstVector3<real> n(&nrm[3 * (size_t)p]);
        for (int i = 0; i < 3; ++i) {
            size_t co = cBatch > 1 ? 9 * (i + 3 * b) : 9 * i;
            const float* c = &coeffs[co];
            real irr = shadingSh(c, n);
            real gsh[9];
            Vector3<real> gnv;
            gradShadingSh(gsh, gnv, c, n);
            float g = gin[3 * (size_t)p + i];
            float dd = dif[3 * (size_t)p + i];
            gd[3 * (size_t)p + i] = g * irr / M_PI;
            gn[3 * (size_t)p + i] = g * dd * gnv[i] / M_PI;
            for (int j = 0; j < 9; ++j) gc[co + j] += g * dd * gsh[j] / M_PI;
        }
    }
}

// --------------------------------------------------------------- transform
void ref_transform_forward(int affineMode, int B, const float* M, int vBatch, int N,
                           const float* v, float* out) {
    for (int b = 0; b < B; ++b) {
        const ConstMatrix44<real> T(&M[16 * b]);
        for (int x = 0; x < N; ++x) {
            const ConstVector3<real> vv(&v[vBatch > 1 ? 3 * ((size_t)x + (size_t)N * b) : 3 * (size_t)x]);
            Vector3<real> r = affineMode ? toCameraspace<real, affine>(T, vv) : toCameraspace<real, linear>(T, vv);
            for (int k = 0; k < 3; ++k) out[3 * ((size_t)x + (size_t)N * b) + k] = r[k];
        }
    }
}

void ref_transform_backward(int affineMode, int B, const float* gin, const float* M, int vBatch,
                            int N, const float* v, float* gM, float* gv) {
    for (int b = 0; b < B; ++b) {
        const ConstMatrix44<real> T(&M[16 * b]);
        for (int x = 0; x < N; ++x) {
            size_t vo = vBatch > 1 ? 3 * ((size_t)x + (size_t)N * b) : 3 * (size_t)x;
            const ConstVector3<real> vv(&v[vo]);
            const ConstVector3<real> g(&gin[3 * ((size_t)x + (size_t)N * b)]);
            Tensor443<real> gT;
            Matrix33<real> gV;
            if (affineMode) gradCameraspace<real, affine>(gT, gV, T, vv);
            else gradCameraspace<real, linear>(gT, gV, T, vv);
            Matrix44<real> cm = g * gT;
            Vector3<real> cv = g * gV;
            for (int i = 0; i < 16; ++i) gM[16 * b + i] += cm[i];
            for (int k = 0; k < 3; ++k) gv[vo + k] += cv[k];
        }
    }
}

// ------------------------------------------------------------- FGT pieces
void ref_hermite_function(float t, int ph, float* out) { hermiteFunction<real>(out, t, (unsigned)ph); }

float ref_hermite_error(float r, float nr, float ph) { return hermiteError<real>(r, nr, ph); }

float ref_evaluate_hermite(const float* xp, const float* xh, const float* coeffs, int ph, float h) {
    return evluateHermite<real, MAXDEGREE>(xp, xh, coeffs, (unsigned)ph, h);
}

void ref_shift_leaf(float* coeffs, const float* node, const float* leaf, float c, int ph, float h) {
    shiftLeafHermiteExpansion<real>(coeffs, node, leaf, c, (unsigned)ph, h);
}

unsigned ref_expand_bits(unsigned v) { return expandBits(v); }

// MortonTransformFunctor::operator() for each id.
void ref_morton(int n, const float* bounds, float W, float H, float f, const float* pts,
                const unsigned* ids, unsigned* keys) {
    MortonTransformFunctor<real> op(bounds, W, H, f, pts);
    for (int i = 0; i < n; ++i) keys[i] = op(ids[i]);
}

// Karras hierarchy (HierarchyFunctor body) over unique 64-bit keys.
void ref_karras(int n, const unsigned long long* keys, int* left, int* right, int* parent) {
    std::vector<refkey::Key64> k(n);
    for (int i = 0; i < n; ++i) k[i].v = keys[i];
    for (int i = 0; i < 2 * n - 1; ++i) parent[i] = -1;
    for (int idx = 0; idx < n - 1; ++idx) {
        uint2 ij = determineRange<refkey::Key64>(k.data(), (unsigned)n, (unsigned)idx);
        int gamma = findSplit<refkey::Key64>(k.data(), ij.x, ij.y);
        int l = gamma, r = gamma + 1;
        if ((int)std::min(ij.x, ij.y) == gamma) l += n - 1;
        if ((int)std::max(ij.x, ij.y) == gamma + 1) r += n - 1;
        left[idx] = l;
        right[idx] = r;
        parent[l] = idx;
        parent[r] = idx;
    }
}

// ----------------------------------------------------------- full sampler
// One view of sampling.sample on the host.  Reference helpers do the
// arithmetic; this driver supplies the thrust steps (reduction, copy_if,
// stable sort, scans) and the per-thread loops in sequential order.  Two
// deliberate departures, shared with the oracle and the CUDA path:
//  * node expansion centres are indexed [2*child] (the reference reads
//    [child], a race on partially built nodes);
//  * the sampler evaluates masses with getWeight (the live kernel calls
//    getWeightTaylor whose per-cell map is never filled).
// h and the cull radius are inputs so that integer outputs can be compared
// bit for bit given the same bandwidth.  `uniforms` holds R*K values per
// pixel (round-major), consumed in nextLeaf order.  Returns the number of
// hash-map overflows observed (0 in normal operation).
int ref_sample_view(int W, int H, float f, int N, const float* pts, float h, float radius,
                    int K, float precision, const float* uniforms, int* indices,
                    int* outNumVisible, unsigned* outKeys, unsigned* outIds, int* outLeft,
                    int* outRight, int* outDegree, float* outCentre) {
    float bounds[4] = {-radius, (float)W + radius, -radius, (float)H + radius};
    // culling (CullingFunctor)
    std::vector<unsigned> ids;
    for (int i = 0; i < N; ++i) {
        const ConstVector3<real> p(&pts[3 * (size_t)i]);
        Vector2<real> s = toScreenspace<real>((float)W, (float)H, f, p);
        bool vis = (p[2] <= 0.0);
        for (int a = 0; a < 2; ++a) {
            vis &= (bounds[2 * a] <= s[a]);
            vis &= (bounds[2 * a + 1] >= s[a]);
        }
        if (vis) ids.push_back((unsigned)i);
    }
    int n = (int)ids.size();
    *outNumVisible = n;
    size_t P = (size_t)W * H;
    for (size_t i = 0; i < P * K; ++i) indices[i] = -1;
    if (n == 0) return 0;
    // Morton keys + stable sort by key
    std::vector<unsigned> keys(n);
    ref_morton(n, bounds, (float)W, (float)H, f, pts, ids.data(), keys.data());
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return keys[a] < keys[b]; });
    std::vector<unsigned> skeys(n), sids(n);
    for (int i = 0; i < n; ++i) { skeys[i] = keys[order[i]]; sids[i] = ids[order[i]]; }
    std::vector<unsigned long long> k64(n);
    Morton64Functor m64;
    for (int i = 0; i < n; ++i) k64[i] = m64(skeys[i], (unsigned)i);
    int M = 2 * n - 1;
    std::vector<DynamicNode<real>> nodes(M);
    std::vector<AlignedBox<real, 2>> boxes(M);
    std::vector<real> centres(2 * M);
    // leaves (LeafNodeFunctor)
    for (int i = 0; i < n; ++i) {
        DynamicNode<real>& L = nodes[n - 1 + i];
        L.left = -1; L.right = -1; L.index = (int)sids[i]; L.sourceCount = 1; L.degree = 0;
        const ConstVector3<real> p(&pts[3 * (size_t)sids[i]]);
        Vector2<real> s = toScreenspace<real>((float)W, (float)H, f, p);
        for (int a = 0; a < 2; ++a) {
            boxes[n - 1 + i].lower[a] = s[a];
            boxes[n - 1 + i].upper[a] = s[a];
            centres[2 * (n - 1 + i) + a] = s[a];
        }
    }
    // hierarchy
    std::vector<int> left(M, -1), right(M, -1), parent(M, -1);
    if (n > 1) ref_karras(n, k64.data(), left.data(), right.data(), parent.data());
    for (int i = 0; i < M; ++i) {
        nodes[i].parent = parent[i];
        if (i < n - 1) { nodes[i].left = left[i]; nodes[i].right = right[i]; nodes[i].index = -1; }
    }
    // bottom-up fan-in in leaf order (second arrival merges)
    std::vector<int> lock(M, 0);
    unsigned depth = 1;
    for (int leaf = 0; leaf < n && n > 1; ++leaf) {
        int nodeIdx = n - 1 + leaf;
        unsigned d = 1;
        bool done = false;
        do {
            nodeIdx = nodes[nodeIdx].parent;
            if (lock[nodeIdx] == 0) { lock[nodeIdx] = 1; done = true; break; }
            DynamicNode<real>& node = nodes[nodeIdx];
            DynamicNode<real>& Lc = nodes[node.left];
            DynamicNode<real>& Rc = nodes[node.right];
            mergeBoxes<real, 2>(boxes[nodeIdx], boxes[node.left], boxes[node.right]);
            unsigned lc = Lc.sourceCount, rc = Rc.sourceCount, nc = lc + rc;
            for (int a = 0; a < 2; ++a)
                centres[2 * nodeIdx + a] = (lc * centres[2 * node.left + a] + rc * centres[2 * node.right + a]) / nc;
            node.sourceCount = nc;
            real maxNorm = maxNormFromBbox<real, 2>(boxes[nodeIdx], &centres[2 * nodeIdx]);
            real r = maxNorm / h;
            node.radius = r;
            int d0 = std::max(std::max(Lc.degree, Rc.degree), 0);
            unsigned degree = (unsigned)d0;
            while (degree <= MAXDEGREE && hermiteError<real>(r, nc, degree) > precision && r < 1.0) degree += 1;
            node.degree = -1;
            if (r < 1.0 && degree <= MAXDEGREE) node.degree = degree;
            d += 1;
        } while (nodes[nodeIdx].parent != -1);
        if (!done) depth = d;
    }
    if (n == 1) { nodes[0].parent = -1; }
    // offsets + P2M (HermiteCoefficientFunctor, sequential)
    int total = 0;
    for (int i = 0; i < M; ++i) {
        int sz = nodes[i].degree > -1 ? (nodes[i].degree + 1) * (nodes[i].degree + 1) : 0;
        nodes[i].offset = total;
        total += sz;
    }
    std::vector<real> coeffs(total > 0 ? total : 1, 0.0f);
    for (int i = 0; i < n; ++i) {
        int leafIdx = n - 1 + i;
        coeffs[nodes[leafIdx].offset] = 1.0f;
        int nodeIdx = leafIdx;
        while (nodes[nodeIdx].parent != -1) {
            nodeIdx = nodes[nodeIdx].parent;
            if (nodes[nodeIdx].degree >= 0)
                shiftLeafHermiteExpansion(&coeffs[nodes[nodeIdx].offset], &centres[2 * nodeIdx],
                                          &centres[2 * leafIdx], 1.0f, (unsigned)nodes[nodeIdx].degree, h);
        }
    }
    for (int i = 0; i < n; ++i) { outKeys[i] = skeys[i]; outIds[i] = sids[i]; }
    for (int i = 0; i < M; ++i) {
        outLeft[i] = nodes[i].left; outRight[i] = nodes[i].right; outDegree[i] = nodes[i].degree;
        outCentre[2 * i] = centres[2 * i]; outCentre[2 * i + 1] = centres[2 * i + 1];
    }
    DynamicTreeDevPtrs<real, 2> tree = {nodes.data(), boxes.data(), centres.data(), coeffs.data()};
    // sequentialPoissonKernel body, R rounds, per pixel
    unsigned R = 0;
    while ((double)R < std::sqrt((double)K)) ++R;
    unsigned mapSize = (unsigned)K * depth;
    int overflows = 0;
    std::vector<NodeState<real>> map(mapSize);
    std::vector<float> keysBuf(K);
    for (int i = 0; i < W; ++i)
        for (int j = 0; j < H; ++j) {
            size_t pixel = (size_t)j + (size_t)H * i;
            for (auto& e : map) e = NodeState<real>();
            for (int k = 0; k < K; ++k) keysBuf[k] = INFINITY;
            int* localIndices = &indices[(size_t)K * pixel];
            real query[2] = {(real)i, (real)j};
            for (unsigned round = 0; round < R; ++round) {
                const float* u = &uniforms[((size_t)pixel * R + round) * K];
                int nodeIdx = 0;
                real tot = fmaxf(real(0), getWeight<real, 2>(&tree, nodeIdx, query, precision, h));
                if (tot < precision) break;
                NodeTrace<real> trace[STACKSIZE];
                unsigned traceIdx = 1;
                trace[0].index = 0;
                trace[0].probability = 1.0f;
                real weights[2];
                while ((unsigned)nodes[nodeIdx].sourceCount > (unsigned)K) {
                    const DynamicNode<real>& node = nodes[nodeIdx];
                    weights[0] = fmaxf(real(0), getWeight<real, 2>(&tree, node.left, query, precision, h));
                    weights[1] = fmaxf(real(0), getWeight<real, 2>(&tree, node.right, query, precision, h));
                    normalize<real, 2>(weights);
                    real s0 = weights[0] * getCapacity((unsigned)node.left, map.data(), mapSize);
                    real s1 = weights[1] * getCapacity((unsigned)node.right, map.data(), mapSize);
                    if (s0 < s1) { trace[traceIdx].index = node.right; trace[traceIdx].probability = weights[1]; nodeIdx = node.right; }
                    else { trace[traceIdx].index = node.left; trace[traceIdx].probability = weights[0]; nodeIdx = node.left; }
                    traceIdx++;
                    if (traceIdx >= STACKSIZE) return -1;
                }
                real probability = 1.0f;
                for (unsigned m = traceIdx; m > 0; m--) {
                    // count a wrap-around overwrite in the fixed-size map
                    unsigned key = trace[m - 1].index, mi = hash(key, mapSize);
                    bool found = false;
                    for (unsigned t = 0; t < mapSize; ++t) {
                        if (map[mi].index == key || map[mi].used == 0) { found = true; break; }
                        mi = (mi + 1) % mapSize;
                    }
                    if (!found) overflows++;
                    real capacity = fmaxf(0.0f, getCapacity(trace[m - 1].index, map.data(), mapSize) - probability);
                    setCapacity(trace[m - 1].index, capacity, map.data(), mapSize);
                    probability *= trace[m - 1].probability;
                }
                unsigned leafCount = nodes[nodeIdx].sourceCount;
                unsigned subtreeParent = nodes[nodeIdx].parent;
                unsigned leafIdx = nodeIdx;
                for (unsigned k = 0; k < leafCount; k++) {
                    leafIdx = nextLeaf<real, 2>(nodes.data(), subtreeParent, leafIdx);
                    const DynamicNode<real>& leaf = nodes[leafIdx];
                    real prob = fmaxf(real(0), getWeight<real, 2>(&tree, leafIdx, query, precision, h));
                    real x = u[k];
                    insertSample(leaf.index, x / prob, localIndices, keysBuf.data(), (unsigned)K);
                }
            }
        }
    return overflows;
}

int ref_stacksize(void) { return STACKSIZE; }

}  // extern "C"
