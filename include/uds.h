/* uds.h - C ABI of the GB300 splatting library (libuds.so).
 *
 * One entry point per operation of the reference's torch extensions
 * (cudaExtensions.{transform,sampling,splatting,filtering,interpolation,
 * shading}); each comment names the reference host wrapper it replaces.
 *
 * Conventions shared by every entry point:
 *  - all pointers are CUDA device pointers to contiguous float32 / int32
 *    arrays in the reference's layouts: splat arrays (1|B, N, c), pixel arrays
 *    (B, W, H, ...) with pixel offset j + H*i for x = i, y = j;
 *  - `stream` is a cudaStream_t (NULL = legacy default stream); work is only
 *    enqueued, nothing synchronises with the host;
 *  - outputs are written completely (gradient outputs are zeroed first), so
 *    callers may pass uninitialised memory;
 *  - scratch memory is caller-owned: query its size with the matching
 *    *_workspace_size function and pass a device buffer of at least that many
 *    bytes (16-byte aligned).  Nothing here calls cudaMalloc, so every call is
 *    safe inside CUDA graph capture;
 *  - the return value is a uds_status; uds_status_string() names it.
 */
#ifndef UDS_H
#define UDS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    UDS_OK = 0,
    UDS_ERR_ARGUMENT = 1,   /* bad size, NULL pointer, unsupported K, ... */
    UDS_ERR_WORKSPACE = 2,  /* workspace smaller than the query returned */
    UDS_ERR_LAUNCH = 3,     /* a kernel launch failed (cudaGetLastError) */
    UDS_ERR_CUDA = 4        /* another CUDA runtime error */
} uds_status;

const char* uds_status_string(int status);
/* Last CUDA error text seen by a failing call on this host thread. */
const char* uds_last_error(void);
int uds_version(void);
/* Number of kernels this library has enqueued since it was loaded. */
unsigned long long uds_launch_count(void);

/* Per-view record written by uds_sample (32 bytes). */
typedef struct {
    float h;          /* isotropic FGT bandwidth in pixels (samplingCuda.cu:233-248) */
    float radius;     /* cull radius (samplingCuda.cu:251-252) */
    int32_t n_visible;/* splats that survived culling = tree leaves */
    int32_t n_coefs;  /* Hermite coefficients stored for internal nodes */
    int32_t demoted;  /* nodes whose expansion did not fit the coefficient pool */
    int32_t overflow; /* pixels whose descent exceeded the 64-entry trace */
    int32_t reserved[2];
} uds_view_stats;

/* Sampling parameters (sampling.cpp:48-94 plus the uniforms interface). */
typedef struct {
    int32_t B, N, W, H, K;   /* views, splats per view, image size, samples per pixel */
    float focal;             /* focal length in pixels */
    float smoothing;         /* added to the screen-space covariance */
    float precision;         /* FGT truncation precision */
    int32_t max_degree;      /* cap of the adaptive Hermite degree (<= 16) */
    int32_t std_batch;       /* leading dim of stdDevs: 1 or B */
    int64_t coef_pool;       /* coefficient pool size in floats, < 2^26 (<=0: default
                                64 per splat, at least 2^20, at most 2^26 - 1) */
    uint64_t seed;           /* Philox key when `uniforms` is NULL */
    const uint64_t* seed_dev;/* optional device pointer: when set, the key is
                                read from it at kernel run time instead of
                                `seed`, so a captured CUDA graph draws new
                                numbers after the caller updates it */
    int32_t tile_x;          /* descent warp tile width in pixels along y:
                                4, 8, 16 or 32 (0 = 8); results do not depend
                                on it, only speed (see the autotuner) */
    int32_t fixed_degree;    /* 0: the reference's adaptive-degree expansions
                                (P2M per node over its leaves).  4, 6 or 8:
                                fixed-degree mode (no counterpart in the
                                reference): every internal node stores a
                                degree-P expansion built by the M2M shift from
                                its children's, evaluated where the adaptive
                                error bound holds at a degree <= P; needs
                                (N-1)(P+1)^2 floats of coefficient pool */
    int32_t leaf_size;       /* Poisson descent only.  <= K (0: default): the
                                reference's single-splat leaves, the descent
                                stops at the first node holding <= K splats.
                                K < L <= 64 (no counterpart in the reference):
                                leaf buckets of L splats, the maximal subtrees
                                with <= L leaves; a round stops at the first
                                node holding <= L splats and order-samples
                                over all of them with their exact Gaussians.
                                A uniforms tensor is then (B,W,H,R,max(K,L)) */
    int32_t spread;          /* Poisson descent with K <= 8: how the child
                                masses below the expansion frontier are shared
                                out: 0 every lane evaluates its own, 1 spread
                                over the warp's lanes.  Results are identical;
                                only the speed differs (the autotuner picks) */
} uds_sample_params;

/* ---- transform (transform.cpp:33-86: affineForward/Backward,
 *      linearForward/Backward).  M (B,4,4), v (vB,N,3) -> out (B,N,3). ---- */
int uds_transform_forward(int affine, int B, const float* M, int vB, int N, const float* v,
                          float* out, void* stream);
/* gM (B,4,4) and gv (vB,N,3) are overwritten. */
int uds_transform_backward(int affine, int B, const float* grad, const float* M, int vB, int N,
                           const float* v, float* gM, float* gv, void* stream);

/* ---- world2Camera (utils.py:11-49, tensor operations in the reference):
 *      positions (B, 3) and quaternions (B, 4) as (x, y, z, w) to row-major
 *      view matrices (B, 4, 4) = [R | t; 0 0 0 1], bit-identical to the
 *      reference's operation sequence; the backward maps d/dM to d/dt, d/dq. ---- */
int uds_view_matrix_forward(int B, const float* positions, const float* quaternions, float* matrices,
                            void* stream);
int uds_view_matrix_backward(int B, const float* grad, const float* quaternions, float* grad_positions,
                             float* grad_quaternions, void* stream);

/* ---- BackfaceCulling (render.py:193-205, a tensor expression in the
 *      reference): splats whose camera-space normal has z > 0 get the
 *      camera-space normal and, when normals is given, the world normal
 *      negated.  cam_normals, flipped_cam (B,N,3); normals (nB,N,3), nB in
 *      {1, B}, flipped_normals (B,N,3) (both may be NULL).  Backward: the
 *      flips of the two incoming gradients (either may be NULL); grad_normals
 *      (nB,N,3), summed over the views in view order when nB == 1. ---- */
int uds_backface_forward(int B, int N, const float* cam_normals, int nB, const float* normals, float* flipped_cam,
                         float* flipped_normals, void* stream);
int uds_backface_backward(int B, int N, const float* cam_normals, const float* grad_flipped_cam, int nB,
                          const float* grad_flipped_normals, float* grad_cam, float* grad_normals, void* stream);

/* ---- sampling.sample (sampling.cpp:48-94): points, normals (B,N,3)
 *      camera space, stdDevs (std_batch,N,2) -> indices (B,W,H,K) int32,
 *      -1 where no sample.  uniforms: optional (B,W,H,R,M) float32 in (0,1],
 *      R = ceil(sqrt(K)), M = max(K, leaf_size); NULL draws Philox4x32-10
 *      uniforms from seed.
 *      h_override: optional device float[B]; entries > 0 replace the
 *      computed bandwidth.  stats: device uds_view_stats[B] (may be NULL). ---- */
size_t uds_sample_workspace_size(const uds_sample_params* prm);
int uds_sample(const uds_sample_params* prm, const float* points, const float* normals,
               const float* std_devs, const float* uniforms, const float* h_override,
               int32_t* indices, uds_view_stats* stats, void* workspace, size_t workspace_bytes,
               void* stream);

/* Geometry of one view of an uneven batch. */
typedef struct {
    int32_t W, H;   /* image size */
    float focal;    /* focal length in pixels */
    int32_t reserved;
} uds_view_desc;

/* ---- sampling.sample for B views of different sizes in one call (no
 *      counterpart in the reference, whose host loop runs one view at a time,
 *      samplingCuda.cu:216-289): every view's tree built (side streams), then
 *      one descent launch over all views' pixels for K <= 8 and B <= 32 (one
 *      launch per view otherwise).  views: host array of B descriptors (prm's
 *      W, H and focal are ignored); indices packed view after view, view b's
 *      (W_b,H_b,K) block first; Philox uniforms from seed with counter view b
 *      (no uniforms tensor).  Workspace: uds_sample_workspace_size(prm). ---- */
int uds_sample_views(const uds_sample_params* prm, const uds_view_desc* views, const float* points,
                     const float* normals, const float* std_devs, const float* h_override, int32_t* indices,
                     uds_view_stats* stats, void* workspace, size_t workspace_bytes, void* stream);

/* Stochastic sampling mode (no counterpart in the reference, whose sampler is
 * the deterministic Poisson descent above): each of the K draws of a pixel
 * descends from the root into a child with probability proportional to its
 * FGT mass and stops at a leaf.  indices (B,W,H,K) int32 as uds_sample;
 * probs (B,W,H,K) float32 receives each draw's path probability q (the
 * product of the ratios it took, ~ leaf mass / root mass), 0 where the draw
 * is -1.  Uniforms are Philox4x32-10 keyed by prm->seed, counter
 * (pixel, view, 2^31 | k<<8 | depth/4, 0).  Same workspace as uds_sample. */
int uds_sample_stochastic(const uds_sample_params* prm, const float* points, const float* normals,
                          const float* std_devs, const float* h_override, int32_t* indices, float* probs,
                          uds_view_stats* stats, void* workspace, size_t workspace_bytes, void* stream);

/* Learned-proposal sampling (no counterpart in the reference): K weighted
 * draws per pixel.  With mlp_params (uds_mlp_param_count() floats) each draw
 * descends by the network's branch probabilities q (16 features per node,
 * evaluated level by level on the tensor cores) and gets the importance
 * weight (leaf Gaussian / root FGT mass) / q_path, an unbiased estimator for
 * any q > 0.  Pixels whose effective sample size (sum w)^2 / sum w^2 is below
 * ess_tau * K are redrawn by the stochastic sampler (their weights then use
 * its exact path probabilities); fallback (B,W,H) uint8 and n_fallback[B]
 * report them (either may be NULL).  With mlp_params NULL every pixel uses
 * the stochastic sampler.  indices (B,W,H,K) int32 (-1: none), weights
 * (B,W,H,K) float32.  Workspace: uds_proposal_workspace_size.  With
 * mlp_params the call synchronises with the stream every 8 tree levels to
 * stop once every draw has reached a leaf. */
size_t uds_proposal_workspace_size(const uds_sample_params* prm);
int uds_sample_proposal(const uds_sample_params* prm, const float* points, const float* normals,
                        const float* std_devs, const float* h_override, const float* mlp_params, float ess_tau,
                        int32_t* indices, float* weights, uint8_t* fallback, int32_t* n_fallback,
                        uds_view_stats* stats, void* workspace, size_t workspace_bytes, void* stream);
/* Training rows for the proposal network from the tree already built by
 * uds_tree_build in `workspace`: stochastic descents with exact FGT masses
 * from every stride-th pixel (both directions), `draws` per pixel; each
 * visited internal node appends (16 features, m_left / (m_left + m_right)) to
 * X (cap x 16) and target (cap), and, when keys is not NULL, the row's key
 * (pixel << 16 | draw << 8 | depth) to keys (cap): rows are appended in no
 * fixed order, sorting by key gives a fixed one.  *count (device int, preset
 * to 0) receives the number of rows produced (it may exceed cap; rows past
 * cap are dropped). */
int uds_proposal_dataset(const uds_sample_params* prm, int stride, int draws, float* X, float* target,
                         int64_t* keys, int32_t* count, int cap, const void* workspace, size_t workspace_bytes,
                         void* stream);

/* Debug view of one tree (for tests): builds view `view` and copies the
 * first n_visible entries of each array (host-sized by the caller from
 * stats).  Any output pointer may be NULL.  Arrays: keys/ids (n), node arrays
 * (2n-1): left, right, parent, count, degree; centre (2n-1,2); box (2n-1,4). */
int uds_tree_build(const uds_sample_params* prm, int view, const float* points,
                   const float* normals, const float* std_devs, const float* h_override,
                   uds_view_stats* stats, uint32_t* keys, int32_t* ids, int32_t* left,
                   int32_t* right, int32_t* parent, int32_t* count, int32_t* degree,
                   float* centre, float* box, void* workspace, size_t workspace_bytes,
                   void* stream);
/* The per-pixel descent alone (the last stage of uds_sample) on the tree of
 * `view` already built in `workspace` by uds_tree_build; `indices` (W,H,K)
 * for that view, not preset (pixels without samples are left untouched, so
 * fill it with -1 first).  Used to time the dominant kernel on its own. */
int uds_sample_descent(const uds_sample_params* prm, int view, const float* uniforms,
                       int32_t* indices, void* workspace, size_t workspace_bytes, void* stream);
/* FGT node masses (getWeight) of an already built tree (same workspace,
 * after uds_tree_build): m queries (node id, x, y) -> out[m]. */
int uds_fgt_eval(const uds_sample_params* prm, int m, const int32_t* nodes, const float* query_xy,
                 float* out, const void* workspace, size_t workspace_bytes, void* stream);

/* ---- pixelgather.scatter / gather (pixelGather.cpp:10-24,
 *      pixelGatherCuda.cu:7-152).  scatter: out (B,W,H,K,C) = values (B,N,C)
 *      at each sample's splat, 0 for index -1.  gather: out (B,N,C) = sum of
 *      values (B,W,H,K,C) over the samples of each splat; deterministic = 0
 *      adds with atomics (unordered, as the reference), deterministic = 1 sums
 *      each splat's samples in sample order (bit-reproducible; workspace
 *      uds_pixel_gather_workspace_size bytes, unused otherwise). ---- */
int uds_pixel_scatter(int B, int W, int H, int K, const int32_t* indices, int N, int C, const float* values,
                      float* out, void* stream);
size_t uds_pixel_gather_workspace_size(int B, int W, int H, int K, int N);
int uds_pixel_gather(int B, int W, int H, int K, const int32_t* indices, int N, int C, const float* values,
                     float* out, int deterministic, void* workspace, size_t workspace_bytes, void* stream);

/* ---- nearestsamples.nearest (nearestSamples.cpp:31-75,
 *      nearestSamplesCuda.cu:355-564): for every splat s, the num_nearest
 *      (<= 32) nearest splats among the other samples of the pixels whose
 *      surface sample (largest weight, first on ties) is s; distances between
 *      points (1,N,3); nearest (1,N,num_nearest) int32 ordered by (distance,
 *      index), -1 padded (the reference's lock-order-dependent merge and its
 *      infinite-distance padding are replaced by this order-free
 *      definition).  indices, weights (B,W,H,K). ---- */
size_t uds_nearest_workspace_size(int B, int W, int H, int K, int N);
int uds_nearest_samples(int B, int W, int H, int K, const int32_t* indices, const float* weights, int N,
                        const float* points, int num_nearest, int32_t* nearest, void* workspace,
                        size_t workspace_bytes, void* stream);

/* ---- NearestSamplesRegularizer.forward (splatting/regularizier.py:119-175)
 *      over the nearest lists of uds_nearest_samples: nearest (N,M) int32
 *      (-1 padded; index 0 is masked like the reference's `nearest > 0`),
 *      points / normals (1,N,3).  losses[0] = normal loss, losses[1] = plane
 *      loss, summed over splats (mean != 0: divided by N); grad_points /
 *      grad_normals (N,3) = their gradients w.r.t. the splat's own point
 *      (plane loss) and normal (normal loss), the neighbour weights and the
 *      filtered normals held constant as in the reference.  Deterministic.
 *      Workspace: uds_nearest_regularizer_workspace_size(N) bytes. ---- */
size_t uds_nearest_regularizer_workspace_size(int N);
int uds_nearest_regularizer(int N, int M, const int32_t* nearest, const float* points, const float* normals,
                            float sigma, int mean, float* losses, float* grad_points, float* grad_normals,
                            void* workspace, size_t workspace_bytes, void* stream);

/* ---- training-step tail (optimization_geometry.py:190-219), fused.
 *      uds_image_loss: kind 0 = L1, 1 = L2 (losses.py:5-31); *loss =
 *      scale * sum over the n elements, grad = d(*loss)/dx (scale = 1 for
 *      reduction 'sum', 1/n for 'mean').
 *      uds_adam_splats: one Adam step (torch.optim.Adam defaults: no weight
 *      decay) on the per-splat tensors points (N,3), normals (N,3), colors
 *      (N,C), std_devs (N,2) (any may be NULL with its gradient), moments
 *      packed in m and v (N*(3+3+C+2) floats each, zeroed before step 1), then
 *      with project != 0 the reference's constraints: normals renormalised
 *      (x / (|x| + 1e-4)) and std_devs clamped to [sd_lo, sd_hi]. ---- */
int uds_image_loss(int kind, size_t n, const float* x, const float* y, float scale, float* loss, float* grad,
                   void* stream);
int uds_adam_splats(int N, float* points, const float* g_points, float* normals, const float* g_normals,
                    float* colors, const float* g_colors, int C, float* std_devs, const float* g_std_devs, float* m,
                    float* v, int step, float lr, float beta1, float beta2, float eps, float sd_lo, float sd_hi,
                    int project, void* stream);

/* ---- proposal network (no counterpart in the reference).  Tensor-core
 *      kernels (tcgen05, accumulators in tensor memory). ---- */
/* Layout check of the tensor-core path (debug): C (128 x N, fp32) =
 * A (128 x K, bf16) * B (N x K, bf16)^T, 16 <= N <= 64, 16 <= K <= 128, both
 * multiples of 16; swap selects the reading of the two descriptor distances;
 * *err (device int, preset to 0) becomes 1 if the product did not complete. */
int uds_mma_probe(int N, int K, const uint16_t* A, const uint16_t* B, float* C, int swap, int* err,
                  void* stream);

/* Proposal network 16 -> 64 -> 64 -> 64 -> 2 (ReLU), parameters fp32 in one
 * array of uds_mlp_param_count() floats: W1 (64x16), b1, W2 (64x64), b2,
 * W3 (64x64), b3, W4 (16x64, rows 2..15 zero), b4 (16).  Computed in bf16
 * with fp32 accumulation.  uds_mlp_forward: X (R x 16) -> logits (R x 2). */
int uds_mlp_param_count(void);
int uds_mlp_forward(int R, const float* X, const float* params, float* logits, int* err, void* stream);
/* Same, the row count read on the device from *R_dev (at most R_max rows). */
int uds_mlp_forward_dev(int R_max, const int* R_dev, const float* X, const float* params, float* logits, int* err,
                        void* stream);
/* Same, the rows given as bf16 in the network's operand layout: row r is in
 * 128-row tile r/128 (4096 bytes at X_tiles + 4096*(r/128); element (r%128,
 * k) at byte (r%128/8)*256 + (k/8)*128 + (r%8)*16 + (k%8)*2), the buffer
 * holding ceil(R_max/128) tiles, 16-byte aligned.  Tiles are streamed by bulk
 * copies. */
int uds_mlp_forward_tiles(int R_max, const int* R_dev, const void* X_tiles, const float* params, float* logits,
                          int* err, void* stream);
/* Training: adds the gradient of the mean cross-entropy between
 * softmax(logits) and (target, 1 - target) over the R rows to grad (fp32,
 * uds_mlp_param_count() entries, zeroed by the caller) and the mean loss to
 * *loss (device float).  Each block's partial sums go to the workspace
 * (uds_mlp_grad_workspace_size(R) bytes) and are added in block order, so the
 * result is the same on every run.  uds_mlp_adam: one Adam step
 * (bias-corrected, step >= 1) on params with moments m1, m2; consumes
 * (zeroes) grad. */
size_t uds_mlp_grad_workspace_size(int R);
int uds_mlp_grad(int R, const float* X, const float* target, const float* params, float* grad, float* loss,
                 int* err, void* workspace, size_t workspace_bytes, void* stream);
int uds_mlp_adam(float* params, float* grad, float* m1, float* m2, int step, float lr, float beta1, float beta2,
                 float eps, void* stream);

/* ---- splatting.forward / backward (splatting.cpp:43-129).  points,
 *      normals (B,N,3) camera space; std_devs (std_batch,N,2); weights and
 *      grad (B,W,H,K).  Workspace: per-splat Gaussian constants, gradient
 *      statistics and a flag per (view, splat) pair, uds_splat_workspace_size(B, N)
 *      bytes.  Only pairs that some pixel samples are evaluated; the others
 *      get zero gradients, as in the reference. ---- */
size_t uds_splat_workspace_size(int B, int N);
int uds_splat_forward(int B, int W, int H, int K, float focal, const int32_t* indices,
                      const float* points, const float* normals, int std_batch, int N,
                      const float* std_devs, float smoothing, float* weights, void* workspace,
                      size_t workspace_bytes, void* stream);
int uds_splat_backward(int B, int W, int H, int K, float focal, const float* grad,
                       const int32_t* indices, const float* points, const float* normals,
                       int std_batch, int N, const float* std_devs, float smoothing,
                       float* grad_points, float* grad_normals, float* grad_std_devs,
                       void* workspace, size_t workspace_bytes, void* stream);

/* ---- The shading pass of Splatting.forward (render.py:268-376, the chain
 *      splattingCuda.cu:18-66 -> zSortingCuda.cu:11-62 ->
 *      interpolationCuda.cu:5-46) fused per pixel: EWA weights, depth
 *      compositing and interpolation of per-splat attributes (aB,N,C), aB in
 *      {1, B}, in one kernel after the per-splat constants.  Writes the EWA
 *      weights and depth weights (B,W,H,K) and the image (B,W,H,C),
 *      bit-identical to uds_splat_forward + uds_filter_forward (points as
 *      (B,N,3)) + uds_interp_forward.  Workspace: uds_splat_workspace_size.
 *      The backward takes the gradient of the image and, optionally (NULL:
 *      none), of the depth weights and of the EWA weights, and the EWA weights
 *      of the forward; it gives the EWA kernel's raw point / normal / std-dev
 *      gradients (as uds_splat_backward) and the attribute gradient (aB,N,C),
 *      the chain's results up to the order of atomic additions. ---- */
int uds_render_fused_forward(int B, int W, int H, int K, float focal, const int32_t* indices, const float* points,
                             const float* normals, int std_batch, int N, const float* std_devs, float smoothing,
                             int aB, int C, const float* attribute, float* weights, float* depth_weights,
                             float* image, void* workspace, size_t workspace_bytes, void* stream);
int uds_render_fused_backward(int B, int W, int H, int K, float focal, const float* grad_image,
                              const float* grad_depth_weights, const float* grad_weights, const int32_t* indices,
                              const float* weights, const float* points, const float* normals, int std_batch, int N,
                              const float* std_devs, float smoothing, int aB, int C, const float* attribute,
                              float* grad_points, float* grad_normals, float* grad_std_devs, float* grad_attribute,
                              void* workspace, size_t workspace_bytes, void* stream);

/* splatting.forward without a workspace, for callers that cannot allocate
 * device memory (a plugin slot that only passes the op's inputs and outputs,
 * a language binding without a device allocator, a real-time loop that must
 * not allocate after start-up).  No counterpart in the reference.  Same
 * arguments and results as uds_splat_forward minus the workspace; the scratch
 * is a fixed 8 MiB array inside the library, so B*N must not exceed 262144
 * (larger calls return UDS_ERR_ARGUMENT).  Every call looks the array's
 * device address up on the current device, so a device reset between calls
 * is harmless; the first call on a device may load the library's device code
 * (make it before any stream capture); calls that overlap on the GPU share
 * the array and race. */
int uds_splat_forward_static(int B, int W, int H, int K, float focal, const int32_t* indices,
                             const float* points, const float* normals, int std_batch, int N,
                             const float* std_devs, float smoothing, float* weights, void* stream);

/* ---- filtering.forward / backward (zSorting.cpp:24-43); points/normals
 *      (pB,N,3), pB = 1 or B. ---- */
int uds_filter_forward(int B, int W, int H, int K, const int32_t* indices, const float* weights,
                       float focal, int pB, int N, const float* points, const float* normals,
                       float* out, void* stream);
int uds_filter_backward(int B, int W, int H, int K, const int32_t* indices, const float* weights,
                        const float* grad, float focal, int pB, int N, const float* points,
                        const float* normals, float* grad_weights, void* stream);

/* ---- interpolation.forward / backward (interpolation.cpp:31-95);
 *      attribute (aB,N,C). ---- */
int uds_interp_forward(int B, int W, int H, int K, const int32_t* indices, const float* weights,
                       int aB, int N, int C, const float* attribute, float* out, void* stream);
int uds_interp_backward(int B, int W, int H, int K, const float* grad, const int32_t* indices,
                        const float* weights, int aB, int N, int C, const float* attribute,
                        float* grad_weights, float* grad_attribute, void* stream);

/* ---- shading.forward / backward / forwardSh / backwardSh
 *      (shading.cpp:51-199).  Pixels P = W*H per view. ---- */
int uds_shade_forward(int B, int P, int L, const float* dirs, const float* intensities, int IB,
                      const float* normals, const float* diffuse, float* out, void* stream);
int uds_shade_backward(int B, int P, int L, const float* grad, const float* dirs,
                       const float* intensities, int IB, const float* normals,
                       const float* diffuse, float* grad_dirs, float* grad_intensities,
                       float* grad_normals, float* grad_diffuse, void* stream);
int uds_shade_sh_forward(int B, int P, const float* coeffs, int cB, const float* normals,
                         const float* diffuse, float* out, void* stream);
int uds_shade_sh_backward(int B, int P, const float* grad, const float* coeffs, int cB,
                          const float* normals, const float* diffuse, float* grad_coeffs,
                          float* grad_normals, float* grad_diffuse, void* stream);

/* ---- Lambert of the forward shading mode, fused (shading.py:12-29
 *      Lambert.forward: ambient * diffuse + sum_l I_l clamp(<dir_l, n>, 0, 1)
 *      diffuse / pi, a chain of broadcasting tensor operations in the
 *      reference).  normals (B, N, 3), diffuse (dB, N, 3), dirs (B, L, 3),
 *      intensities (IB, L, 3), ambient (aB, 3); dB, IB, aB in {1, B};
 *      L <= 4.  The backward sums the gradients of broadcast operands. ---- */
int uds_lambert_forward(int B, int N, int L, const float* ambient, int aB, const float* dirs,
                        const float* intensities, int IB, const float* normals,
                        const float* diffuse, int dB, float* out, void* stream);
int uds_lambert_backward(int B, int N, int L, const float* grad, const float* ambient, int aB,
                         const float* dirs, const float* intensities, int IB, const float* normals,
                         const float* diffuse, int dB, float* grad_ambient, float* grad_dirs,
                         float* grad_intensities, float* grad_normals, float* grad_diffuse,
                         void* stream);

#ifdef __cplusplus
}
#endif
#endif
