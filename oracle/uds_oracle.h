/* CPU oracle for the Poisson-sampled EWA splatting path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
 * legs of bench.py call into this library, and only to check or to time the
 * CUDA path against it; the product never links or loads it.
 *
 * Every entry point restates one reference operation; the comment beside each
 * names the reference file:line it follows (paths inside the reference
 * project).  Layouts are the reference's: splat arrays (1|B, N, c) row-major
 * float32, pixel arrays (B, W, H, ...) with pixel offset j + H*i for x = i,
 * y = j.
 *
 * Parity status: the per-sample arithmetic (EWA weight, compositing,
 * shading, transform, Hermite series, Morton keys, Karras topology, sampler
 * loop) is pinned against the reference's own functions compiled on the host
 * (oracle/ref_shim.cu) through the fixtures in tests/golden/.
 */
#ifndef UDS_ORACLE_H
#define UDS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Arithmetic flavour of the sampler path.
 *  ORC_DET : the deterministic formulation the CUDA path computes
 *            (own exp/log from Cody-Waite reduction + Taylor polynomial,
 *            integer powers by repeated products, Hermite series summed
 *            row-factored with fused multiply-adds; every other operation in
 *            the reference's order).  CUDA results must equal this bit for
 *            bit.
 *  ORC_LIBM: the reference's formulation (libm expf/logf/powf, unfused
 *            products), used to pin the oracle against the reference shim. */
enum { ORC_DET = 0, ORC_LIBM = 1 };

float orc_det_expf(float x);
float orc_det_logf(float x);
void orc_philox_uniforms(uint64_t seed, uint32_t view, uint32_t pixel, uint32_t round, int K,
                         float* out);

/* transform.cpp:33-86, transformCuda.cu:11-117 */
void orc_transform_forward(int affine, int B, const float* M, int vB, int N, const float* v,
                           float* out);
void orc_transform_backward(int affine, int B, const float* gin, const float* M, int vB, int N,
                            const float* v, float* gM, float* gv);

/* splatting.cpp:43-129, splattingCuda.cu:18-233, ewaSplatting.cuh:8-91 */
void orc_to_screenspace(int n, float W, float H, float f, const float* pts, float* out);
float orc_ewa_weight(const float* pixel, float W, float H, float f, const float* p,
                     const float* nrm, const float* sd, float smoothing, float* unclamped);
void orc_ewa_grad(const float* pixel, float W, float H, float f, const float* p, const float* nrm,
                  const float* sd, float smoothing, double* gp, double* gn, double* gs);
void orc_splat_forward(int B, int W, int H, int K, float f, const int* idx, const float* pts,
                       const float* nrm, const float* sd, int sdB, int N, float smoothing,
                       float* w);
void orc_splat_backward(int B, int W, int H, int K, float f, const float* gin, const int* idx,
                        const float* pts, const float* nrm, const float* sd, int sdB, int N,
                        float smoothing, float* gp, float* gn, float* gs);

/* zSorting.cpp:24-43, zSortingCuda.cu:11-243, alphacompositing*.cuh */
void orc_filter_forward(int B, int W, int H, int K, const int* idx, const float* w, float f,
                        int pB, int N, const float* pts, const float* nrm, float* out,
                        int* order);
void orc_filter_backward(int B, int W, int H, int K, const int* idx, const float* w,
                         const float* gin, float f, int pB, int N, const float* pts,
                         const float* nrm, float* out);

/* interpolation.cpp:31-95, interpolationCuda.cu:5-167 */
void orc_interp_forward(int B, int W, int H, int K, const int* idx, const float* w, int aB, int N,
                        int C, const float* attr, float* out);
void orc_interp_backward(int B, int W, int H, int K, const float* gin, const int* idx,
                         const float* w, int aB, int N, int C, const float* attr, float* gw,
                         float* ga);

/* EWA weight -> compositing -> interpolation for one view and fixed indices,
 * every operation in double (central-difference reference; sd (N,2), attr (N,C)) */
void orc_chain64_forward(int W, int H, int K, double f, const int* idx, int N, const double* pts,
                         const double* nrm, const double* sd, double smoothing, int C, const double* attr,
                         double* img);

/* pixelgather (pixelGatherCuda.cu:7-152): scatter (B,N,C) -> (B,W,H,K,C);
 * gather (B,W,H,K,C) -> (B,N,C), each splat's samples summed in sample order */
void orc_pixel_scatter(int B, int W, int H, int K, const int* idx, int N, int C, const float* values,
                       float* out);
void orc_pixel_gather(int B, int W, int H, int K, const int* idx, int N, int C, const float* values,
                      float* out);

/* nearestsamples.nearest: per splat, the M nearest distinct candidates in
 * (distance, index) order, -1 padded; out (N x M) */
void orc_nearest_samples(int B, int W, int H, int K, const int* idx, const float* w, int N, const float* pts, int M,
                         int* out);

/* shading.cpp:51-199, shadingCuda.cu, diffuseShading*.cuh */
void orc_shade_forward(int B, int P, int L, const float* dirs, const float* I, int IB,
                       const float* nrm, const float* dif, float* out);
void orc_shade_backward(int B, int P, int L, const float* gin, const float* dirs, const float* I,
                        int IB, const float* nrm, const float* dif, float* gdirs, float* gI,
                        float* gn, float* gd);
void orc_shade_sh_forward(int B, int P, const float* coef, int cB, const float* nrm,
                          const float* dif, float* out);
void orc_shade_sh_backward(int B, int P, const float* gin, const float* coef, int cB,
                           const float* nrm, const float* dif, float* gc, float* gn, float* gd);

/* ---- FMM sampler (sampling.cpp:48-94, samplingCuda.cu:197-321) ---- */

/* Isotropic bandwidth h of one view (samplingCuda.cu:106-195, 233-248). */
float orc_view_bandwidth(int W, int H, float f, int N, const float* pts, const float* nrm,
                         const float* sd, float smoothing);
/* Cull radius (samplingCuda.cu:251-252). */
float orc_cull_radius(float h, float precision, int flavour);

typedef struct orc_tree orc_tree;

/* Build the view's tree: cull, Morton keys, stable sort, Karras hierarchy,
 * bottom-up boxes / centres / degrees, coefficient offsets, P2M.
 * coefPool < 0 means unlimited.  Returns NULL on allocation failure. */
orc_tree* orc_tree_build(int W, int H, float f, int N, const float* pts, float h, float radius,
                         float precision, int maxDegree, long coefPool, int flavour);
void orc_tree_free(orc_tree* t);
int orc_tree_size(const orc_tree* t); /* visible splats (leaves) */
long orc_tree_num_coefs(const orc_tree* t);
/* Copies of the tree arrays (any pointer may be NULL). Node arrays have
 * 2n-1 entries, leaf arrays n. */
void orc_tree_export(const orc_tree* t, unsigned* keys, int* ids, int* left, int* right,
                     int* parent, int* count, int* degree, float* centre, float* box,
                     float* leafxy);
/* getWeight (evaluateDynamicRadixTree.cuh:184-242): mass of node at query. */
float orc_tree_node_weight(const orc_tree* t, int node, const float* query, int flavour);
/* Exact FP64 Gauss sum over the leaves of node. */
double orc_tree_direct_weight(const orc_tree* t, int node, const double* query);

/* sequentialPoissonKernel (sequentialPoissonDynamicTree.cuh:56-196) over all
 * pixels of the view.  uniforms: W*H*R*K (pixel-major, then round, then
 * candidate) or NULL to draw Philox uniforms from `seed` for `view`.
 * Pixel rows [x0, x1) only (x1 <= W) so that bounded samples can be timed;
 * indices is the full W*H*K array.  Returns 0, or -1 on trace overflow. */
int orc_tree_sample(const orc_tree* t, int W, int H, int K, float precision, const float* uniforms,
                    uint64_t seed, uint32_t view, int x0, int x1, int flavour, int* indices);
/* the same with leaf buckets: a round stops at the first node holding at
 * most max(K, leaf) splats (leaf <= K: orc_tree_sample); -2 if that is > 64 */
int orc_tree_sample_leaf(const orc_tree* t, int W, int H, int K, int leaf, float precision, const float* uniforms,
                         uint64_t seed, uint32_t view, int x0, int x1, int fl, int* indices);
/* the same estimator with direct FP64 Gauss sums for the node masses (no
 * Hermite expansion; the truncation circles are kept) and FP64 descent
 * arithmetic: the CPU baseline of the whole view */
int orc_tree_sample_fp64(const orc_tree* t, int W, int H, int K, double precision, uint64_t seed, uint32_t view,
                         int x0, int x1, int* indices);
int orc_tree_sample_fp64_leaf(const orc_tree* t, int W, int H, int K, int leaf, double precision, uint64_t seed,
                              uint32_t view, int x0, int x1, int* indices);

/* Stochastic mode: K independent mass-proportional descents per pixel;
 * indices (W*H*K) and path probabilities probs (W*H*K). */
int orc_tree_sample_stochastic(const orc_tree* t, int W, int H, int K, float precision, uint64_t seed,
                               uint32_t view, int x0, int x1, int flavour, int* indices, float* probs);

/* Candidate entries (splat id, leaf mass) of pixel (i, j) over all rounds;
 * returns their number (<= ceil(sqrt(K)) * K). */
int orc_tree_candidates(const orc_tree* t, int K, float precision, int i, int j, int flavour, int* ids,
                        float* p);

/* Whole-view convenience: h (if h <= 0), radius, build, sample.  Writes
 * stats[4] = {h, radius, n_visible, n_coefs}. */
int orc_sample_view(int W, int H, float f, int N, const float* pts, const float* nrm,
                    const float* sd, int K, float smoothing, float precision, float h_in,
                    const float* uniforms, uint64_t seed, uint32_t view, int flavour,
                    int* indices, float* stats);

int orc_num_rounds(int K);
/* pieces exposed for the pinning tests */
void orc_karras_from_keys(int n, const unsigned* keys, int* left, int* right);
unsigned orc_expand_bits(unsigned v);
void orc_hermite_function(float t, int ph, int flavour, float* out);
float orc_hermite_error(float r, float nr, int ph, int flavour);
int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
