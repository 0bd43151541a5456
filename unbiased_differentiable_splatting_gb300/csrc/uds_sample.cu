// sampling.sample (sampling.cpp:48-94, samplingCuda.cu:197-321) on one GPU:
// per view, the FMM tree over the projected splat centres and the per-pixel
// sequential-Poisson descent that draws K splat indices.
//
// Pipeline per view (all on the caller's stream, no host synchronisation;
// view-dependent sizes are read on the device):
//   1 k_bandwidth / k_view_setup  isotropic bandwidth h (mean over splats,
//                                 fixed point) and the cull radius
//   2 k_cull_morton               screen point, visibility, 30-bit Morton key;
//                                 culled splats get a key above every
//                                 visible one so a single sort compacts
//   3 radix sort                  LSD, 4 x 8-bit passes, stable, hand-written
//   4 k_leaves / k_karras         Karras (2012) radix tree over 64-bit keys
//                                 (key << 32 | rank)
//   5 k_bottomup                  atomic fan-in: boxes, count-weighted
//                                 centres, adaptive Hermite degree,
//                                 truncation radius
//   6 node sizes -> scan -> k_assign   coefficient offsets in a fixed pool
//   7 k_p2m                       Hermite moments, one warp per node, each
//                                 coefficient summed over the node's leaves in
//                                 Morton order (deterministic, no atomics)
//   8 k_sample                    per pixel: ceil(sqrt(K)) rounds of greedy
//                                 capacity descent + order sampling on u/p
//
// Every float operation on this path is spelled with an exact-rounding
// intrinsic (or is an IEEE-exact library op: sqrt, division, fma), so the
// Morton keys, the tree, the FGT masses and the sampled indices equal the CPU
// oracle's bit for bit given the same inputs and uniforms.
#include <mutex>

#include <cuda_bf16.h>

#include "uds_ewa.cuh"
#include "uds_radix.cuh"
#include "uds_tc.cuh"

namespace uds {

constexpr unsigned kCulledKey = 0x40000000u;  // above every 30-bit Morton key
constexpr int kScanThreads = 256, kScanItems = 4, kScanTile = kScanThreads * kScanItems;

struct ViewState {            // per-view device scalars (lives in the workspace)
    unsigned long long hsum;  // fixed-point sum of per-splat bandwidths (2^-32 units)
    unsigned long long hcount;
    float h, radius, lo_x, hi_x, lo_y, hi_y, sq;  // sq = sqrt(2 h^2)
    int n;                    // visible splats
    unsigned coef_used;
    float isq;                // 1 / sq (the series' scaled offsets multiply by it)
    int pad[4];
};

// ----------------------------------------------------------- workspace
struct Ws {
    ViewState* vs;
    uds_view_stats* stats;
    uint32_t *keysA, *idsA, *keysB, *idsB;
    uint32_t* hist;
    uint32_t* scanTmp;
    uint32_t* sizes;
    uint32_t* offsets;
    unsigned* fanin;
    float2* leaf_xy;
    int* leaf_id;
    int4* lnk;
    int* par;
    float4* box;
    float4* cen;
    float* coef;
    size_t coef_cap;
    size_t bytes;
};

static size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

// Default coefficient pool: 64 floats per splat, at least 2^20, at most the
// 2^26 - 1 that the 26-bit offsets of the node metadata can address (nodes
// past the pool are demoted to subtree walks, as the oracle does).
static int64_t default_pool(int64_t N) {
    int64_t p = N * 64 > (1 << 20) ? N * 64 : (1 << 20);
    return p < (1ll << 26) ? p : (1ll << 26) - 1;
}

static Ws layout(const uds_sample_params* p, char* base) {
    Ws w{};
    size_t N = (size_t)(p->N > 0 ? p->N : 1);
    size_t M = 2 * N;
    size_t nb = cdiv(N, kSortTile);
    size_t sb = cdiv(N, kScanTile);
    int64_t pool = p->coef_pool > 0 ? p->coef_pool : default_pool((int64_t)N);
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += a256(bytes); return base ? base + o : nullptr; };
    w.vs = (ViewState*)take(sizeof(ViewState));
    w.stats = (uds_view_stats*)take(sizeof(uds_view_stats) * (size_t)(p->B > 0 ? p->B : 1));
    w.keysA = (uint32_t*)take(4 * N);
    w.idsA = (uint32_t*)take(4 * N);
    w.keysB = (uint32_t*)take(4 * N);
    w.idsB = (uint32_t*)take(4 * N);
    w.hist = (uint32_t*)take(4 * 256 * nb);
    w.scanTmp = (uint32_t*)take(4 * (sb + 1));
    w.sizes = (uint32_t*)take(4 * N);
    w.offsets = (uint32_t*)take(4 * N);
    w.fanin = (unsigned*)take(4 * N);
    w.leaf_xy = (float2*)take(8 * N);
    w.leaf_id = (int*)take(4 * N);
    w.lnk = (int4*)take(16 * M);
    w.par = (int*)take(4 * M);
    w.box = (float4*)take(16 * M);
    w.cen = (float4*)take(16 * M);
    w.coef = (float*)take(4 * (size_t)pool);
    w.coef_cap = (size_t)pool;
    w.bytes = off;
    return w;
}

// --------------------------------------------------------- 1 bandwidth
// IsotropicEigenFunctor (samplingCuda.cu:133-162) with the same float /
// double promotions.
__device__ __forceinline__ float splat_bandwidth(float W, float H, float f, const float* p,
                                                 const float* n, const float* sd, float sm) {
    EwaFrame F;
    ewa_frame(W, H, f, p, n, sd, sm, F);
    const float* V = F.V;
    float det = fsub(fmul(V[0], V[3]), fmul(V[1], V[2]));
    float inv = div_via_double(1.0f, det);
    float i0 = fmul(V[3], inv), i1 = fmul(-V[1], inv), i2 = fmul(-V[2], inv), i3 = fmul(V[0], inv);
    float tr = fadd(i0, i3);
    float tt = fmul(tr, tr);
    float root, l1, l2;
    if (fabsf(tr) >= 0x1p-100f && fabsf(tt) >= 0x1p-100f) {
        // 0.25 tt and 0.5 tr are exact in float as in double, so each
        // double operation below has float operands
        root = fsqrt(sub_via_double(fmul(0.25f, tt), fsub(fmul(i0, i3), fmul(i1, i2))));
        l1 = add_via_double(fmul(0.5f, tr), root);
        l2 = sub_via_double(fmul(0.5f, tr), root);
    } else {  // tiny (or NaN) trace: the reference's double sequence
        float idet = fsub(fmul(i0, i3), fmul(i1, i2));
        root = fsqrt((float)dsub(dmul(0.25, (double)tt), (double)idet));
        l1 = (float)dadd(dmul(0.5, (double)tr), (double)root);
        l2 = (float)dsub(dmul(0.5, (double)tr), (double)root);
    }
    float lk = fminf(l1, l2);
    // (float)fmin(1.0, 1.0 / (double)sqrt(lk)): the min commutes with the
    // monotone rounding, and fminf returns 1 for a NaN quotient as fmin does
    return fminf(1.0f, div_via_double(1.0f, fsqrt(lk)));
}

__global__ void k_bandwidth(int N, float W, float H, float f, const float* __restrict__ pts,
                            const float* __restrict__ nrm, const float* __restrict__ sd, float sm,
                            ViewState* vs) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long s = 0, c = 0;
    if (x < N) {
        float p[3] = {pts[3 * (size_t)x], pts[3 * (size_t)x + 1], pts[3 * (size_t)x + 2]};
        float n[3] = {nrm[3 * (size_t)x], nrm[3 * (size_t)x + 1], nrm[3 * (size_t)x + 2]};
        float d[2] = {sd[2 * (size_t)x], sd[2 * (size_t)x + 1]};
        float hk = splat_bandwidth(W, H, f, p, n, d, sm);
        if (isfinite(hk)) {
            s = (unsigned long long)__float2ll_rn(fmul(hk, 4294967296.0f));  // exact: hk <= 1
            c = 1;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    if ((threadIdx.x & 31) == 0 && c) {
        atomicAdd(&vs->hsum, s);
        atomicAdd(&vs->hcount, c);
    }
}

// h (or its override), the cull radius and bounds (samplingCuda.cu:244-258)
__global__ void k_view_setup(const float* h_override, int view, float W, float H, float precision,
                             ViewState* vs, uds_view_stats* stats) {
    float h;
    if (h_override && h_override[view] > 0.0f) h = h_override[view];
    else if (vs->hcount == 0) h = __int_as_float(0x7fc00000);
    else h = (float)ddiv(ddiv(__ull2double_rn(vs->hsum), 4294967296.0), __ull2double_rn(vs->hcount));
    float norm = (float)dmul(2.0 * kPi, (double)fsqrt(h));
    double a = -(double)det_logf(precision);
    double b = (double)det_logf(norm);
    float r = (float)dmul(dmul(1.4142135623730951, (double)h), __dsqrt_rn(dsub(a, b)));
    vs->h = h;
    vs->radius = r;
    vs->lo_x = -r;
    vs->hi_x = fadd(W, r);
    vs->lo_y = -r;
    vs->hi_y = fadd(H, r);
    vs->sq = fsqrt(fmul(fmul(2.0f, h), h));
    vs->isq = fdiv(1.0f, vs->sq);
    vs->n = 0;
    vs->coef_used = 0;
    stats[view].h = h;
    stats[view].radius = r;
    stats[view].n_visible = 0;
    stats[view].n_coefs = 0;
    stats[view].demoted = 0;
    stats[view].overflow = 0;
}

// ------------------------------------------------------- 2 cull + Morton
__device__ __forceinline__ unsigned expand_bits(unsigned v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}
__device__ __forceinline__ unsigned morton_coord(float s, float lo, float hi) {
    float src = fdiv(fsub(s, lo), fsub(hi, lo));
    float c = fminf(fmaxf(fmul(src, 1024.0f), 0.0f), 1023.0f);
    return (unsigned)c;
}

__global__ void k_cull_morton(int N, float W, float H, float f, const float* __restrict__ pts,
                              ViewState* vs, uint32_t* __restrict__ keys, uint32_t* __restrict__ ids) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    bool vis = false;
    if (x < N) {
        float p[3] = {pts[3 * (size_t)x], pts[3 * (size_t)x + 1], pts[3 * (size_t)x + 2]};
        float s[2];
        screen_point(W, H, f, p, s);
        float lx = vs->lo_x, hx = vs->hi_x, ly = vs->lo_y, hy = vs->hi_y;
        vis = (p[2] <= 0.0f) && (lx <= s[0]) && (hx >= s[0]) && (ly <= s[1]) && (hy >= s[1]);
        unsigned key = kCulledKey;
        if (vis) key = 2u * expand_bits(morton_coord(s[0], lx, hx)) + expand_bits(morton_coord(s[1], ly, hy));
        keys[x] = key;
        ids[x] = (uint32_t)x;
    }
    unsigned ball = __ballot_sync(0xffffffffu, vis);
    if ((threadIdx.x & 31) == 0 && ball) atomicAdd(&vs->n, __popc(ball));
}

// ---------------------------------------------------------- 3 radix sort
// Exclusive scan of hist (digit-major, 256 * nb entries) in one block.
__global__ void k_radix_scan(uint32_t* hist, int total) {
    __shared__ uint32_t part[1024];
    int t = threadIdx.x;
    int per = (total + blockDim.x - 1) / blockDim.x;
    int lo = t * per, hi = min(total, lo + per);
    uint32_t s = 0;
    for (int i = lo; i < hi; ++i) s += hist[i];
    part[t] = s;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
        uint32_t v = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = t > 0 ? part[t - 1] : 0;
    for (int i = lo; i < hi; ++i) {
        uint32_t v = hist[i];
        hist[i] = run;
        run += v;
    }
}

// ------------------------------------------------ generic exclusive scan
// Length: vs->n - minus when vs is given, else M0.
__global__ void k_scan_reduce(const uint32_t* __restrict__ in, const ViewState* vs, int minus, int M0,
                              uint32_t* __restrict__ part) {
    __shared__ uint32_t red[kScanThreads / 32];
    int M = vs ? vs->n - minus : M0;
    size_t base = (size_t)blockIdx.x * kScanTile;
    uint32_t s = 0;
    for (int r = 0; r < kScanItems; ++r) {
        size_t i = base + (size_t)r * kScanThreads + threadIdx.x;
        if ((long long)i < M) s += in[i];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < kScanThreads / 32; ++w) t += red[w];
        part[blockIdx.x] = t;
    }
}

__global__ void k_scan_top(uint32_t* part, int nb) {
    __shared__ uint32_t buf[1024];
    int t = threadIdx.x;
    int per = (nb + blockDim.x - 1) / blockDim.x;
    int lo = t * per, hi = min(nb, lo + per);
    uint32_t s = 0;
    for (int i = lo; i < hi; ++i) s += part[i];
    buf[t] = s;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
        uint32_t v = t >= o ? buf[t - o] : 0;
        __syncthreads();
        buf[t] += v;
        __syncthreads();
    }
    uint32_t run = t > 0 ? buf[t - 1] : 0;
    for (int i = lo; i < hi; ++i) {
        uint32_t v = part[i];
        part[i] = run;
        run += v;
    }
    if (t == blockDim.x - 1) part[nb] = buf[t];  // total
}

// in and out may be the same array (each thread reads its items first).
__global__ void k_scan_down(const uint32_t* in, const ViewState* vs, int minus, int M0, const uint32_t* part,
                            uint32_t* out) {
    __shared__ uint32_t wsum[kScanThreads / 32];
    int M = vs ? vs->n - minus : M0;
    size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems], local = 0;
#pragma unroll
    for (int r = 0; r < kScanItems; ++r) {
        size_t i = base + r;
        v[r] = (long long)i < M ? in[i] : 0u;
        local += v[r];
    }
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = local;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    uint32_t woff = 0;
    for (int w = 0; w < warp; ++w) woff += wsum[w];
    uint32_t run = part[blockIdx.x] + woff + incl - local;
#pragma unroll
    for (int r = 0; r < kScanItems; ++r) {
        size_t i = base + r;
        if ((long long)i < M) out[i] = run;
        run += v[r];
    }
}

// ---------------------------------------------------- 4 leaves + Karras
__device__ __forceinline__ float trunc_radius(float h, float precision, int count) {
    return fsqrt(fmul(fmul(-2.0f, fmul(h, h)), det_logf(fdiv(precision, (float)(unsigned)count))));
}

__global__ void k_leaves(int N, float W, float H, float f, const float* __restrict__ pts,
                         const ViewState* vs, float precision, const uint32_t* __restrict__ ids,
                         float2* __restrict__ leaf_xy, int* __restrict__ leaf_id, int4* __restrict__ lnk,
                         int* __restrict__ par, float4* __restrict__ box, float4* __restrict__ cen) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int n = vs->n;
    if (i >= n) return;
    int id = (int)ids[i];
    float p[3] = {pts[3 * (size_t)id], pts[3 * (size_t)id + 1], pts[3 * (size_t)id + 2]};
    float s[2];
    screen_point(W, H, f, p, s);
    int v = n - 1 + i;
    leaf_xy[i] = make_float2(s[0], s[1]);
    leaf_id[i] = id;
    lnk[v] = make_int4(-1, -1, i, 1);
    par[v] = -1;
    box[v] = make_float4(s[0], s[1], s[0], s[1]);
    cen[v] = make_float4(s[0], s[1], trunc_radius(vs->h, precision, 1), make_meta(0, 0));
}

__device__ __forceinline__ int cpref(const uint32_t* keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    unsigned long long a = ((unsigned long long)keys[i] << 32) | (unsigned)i;
    unsigned long long b = ((unsigned long long)keys[j] << 32) | (unsigned)j;
    return __clzll(a ^ b);
}

// determineRange / findSplit (buildRadixTree.cuh:76-167), Karras (2012)
__global__ void k_karras(const ViewState* vs, const uint32_t* __restrict__ keys, int4* __restrict__ lnk,
                         int* __restrict__ par) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    int n = vs->n;
    if (idx >= n - 1) return;
    int lo, hi;
    if (idx == 0) {
        lo = 0; hi = n - 1;
        par[0] = -1;
    } else {
        int dL = cpref(keys, n, idx, idx - 1), dR = cpref(keys, n, idx, idx + 1);
        int d = (dR > dL) ? 1 : -1;
        int dmin = min(dL, dR);
        int lmax = 2;
        while (cpref(keys, n, idx, idx + d * lmax) > dmin) lmax <<= 1;
        int l = 0;
        for (int t = lmax >> 1; t > 0; t >>= 1)
            if (cpref(keys, n, idx, idx + (l + t) * d) > dmin) l += t;
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
    if (lo == split) lc += n - 1;
    if (hi == split + 1) rc += n - 1;
    lnk[idx] = make_int4(lc, rc, lo, hi - lo + 1);
    par[lc] = idx;
    par[rc] = idx;
}

// ------------------------------------------------------------ 5 bottom-up
// hermiteError (hermitefmm.cuh:184-195) with integer powers as products
__device__ __forceinline__ float hermite_error(float r, float nr, unsigned ph) {
    if (r >= 1.0f) return r;
    float om = fsub(1.0f, r);
    float a = fdiv(nr, fmul(om, om));
    float rp = ipowf(r, ph);
    float b = fdiv(rp, fsqrt(facf(ph)));
    float c = fmul(b, b);
    float d = fmul(fmul(2.0f, fsub(1.0f, rp)), b);
    return fmul(a, fadd(c, d));
}

// InternalNodeFunctor (buildDynamicRadixTree.cuh:155-221): the second thread
// to reach a node merges it.  Child centres are read at [child] (the
// reference indexes expansionPoints[child] instead of [2*child]).
__global__ void k_bottomup(const ViewState* vs, float precision, int max_degree,
                           const int4* __restrict__ lnk, const int* __restrict__ par, float4* box,
                           float4* cen, unsigned* fanin) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int n = vs->n;
    if (i >= n || n < 2) return;
    float h = vs->h;
    int v = n - 1 + i;
    while (true) {
        int p = par[v];
        if (p < 0) break;
        __threadfence();
        unsigned old = atomicAdd(&fanin[p], 1u);
        if (old == 0) return;
        __threadfence();
        int4 L = lnk[p];
        int a = L.x, b = L.y;
        float4 ba = __ldcg(&box[a]), bb = __ldcg(&box[b]);
        float4 ca = __ldcg(&cen[a]), cb = __ldcg(&cen[b]);
        float na = (float)(unsigned)lnk[a].w, nb = (float)(unsigned)lnk[b].w, nc = (float)(unsigned)L.w;
        float4 bx = make_float4(fminf(ba.x, bb.x), fminf(ba.y, bb.y), fmaxf(ba.z, bb.z), fmaxf(ba.w, bb.w));
        float cx = fdiv(fadd(fmul(na, ca.x), fmul(nb, cb.x)), nc);
        float cy = fdiv(fadd(fmul(na, ca.y), fmul(nb, cb.y)), nc);
        float mn = fmaxf(0.0f, fmaxf(fsub(cx, bx.x), fsub(bx.z, cx)));
        mn = fmaxf(mn, fmaxf(fsub(cy, bx.y), fsub(bx.w, cy)));
        float r = fdiv(mn, h);
        int d0 = max(meta_degree(ca.w), meta_degree(cb.w));
        unsigned deg = (unsigned)max(d0, 0);
        while (deg <= (unsigned)max_degree && hermite_error(r, nc, deg) > precision && r < 1.0f) deg += 1;
        int degree = (r < 1.0f && deg <= (unsigned)max_degree) ? (int)deg : -1;
        __stcg(&box[p], bx);
        __stcg(&cen[p], make_float4(cx, cy, trunc_radius(h, precision, L.w), make_meta(0, degree)));
        v = p;
    }
}

// ------------------------------------------- 5b fixed-degree M2M pass
// Fixed-degree mode (no reference counterpart): every internal node stores a
// degree-P Hermite expansion at offset v * (P+1)^2, obtained from its
// children's by the M2M shift instead of summing over its leaves:
//   M_ab(c) = sum_{a' <= a, b' <= b} M_a'b'(c_child) t_{a-a'}(dx) t_{b-b'}(dy),
// t_k(d) = d^k / k!, (dx, dy) = (c_child - c) / sqrt(2 h^2); a leaf child is
// the single moment M_00 = 1 at its own position.  Exact for the truncated
// moments (the moments of the union are polynomial in the shift), so the
// expansions equal the per-leaf sums up to rounding at O(P^3) per node.  The
// node is evaluated through its expansion (degree P) when the adaptive error
// bound holds at some degree <= P (k_bottomup run with max_degree = P), else
// walked (degree -1); the coefficients exist either way for the parent's
// shift.  Same second-arrival fan-in as k_bottomup.
__global__ void k_fixed_assign(ViewState* vs, float4* cen, int P) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    int n = vs->n;
    if (v == 0) vs->coef_used = (unsigned)((n > 1 ? n - 1 : 0) * (P + 1) * (P + 1));
    if (v >= n - 1) return;
    float4 c = cen[v];
    c.w = make_meta(v * (P + 1) * (P + 1), meta_degree(c.w) >= 0 ? P : -1);
    cen[v] = c;
}

template <int P>
__global__ void k_m2m(const ViewState* vs, const int4* __restrict__ lnk, const int* __restrict__ par,
                      const float4* __restrict__ cen, float* coef, unsigned* fanin) {
    constexpr int P1 = P + 1, P2 = P1 * P1;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int n = vs->n;
    if (i >= n || n < 2) return;
    float sq = vs->sq;
    int v = n - 1 + i;
    while (true) {
        int p = par[v];
        if (p < 0) break;
        __threadfence();
        if (atomicAdd(&fanin[p], 1u) == 0) return;
        __threadfence();
        int4 L = lnk[p];
        float4 cp = cen[p];
        float acc[P1][P1];
#pragma unroll
        for (int a = 0; a < P1; ++a)
#pragma unroll
            for (int b = 0; b < P1; ++b) acc[a][b] = 0.0f;
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            int c = side ? L.y : L.x;
            float4 cc = cen[c];
            float dx = (cc.x - cp.x) / sq, dy = (cc.y - cp.y) / sq;
            float tx[P1], ty[P1];
            tx[0] = 1.0f;
            ty[0] = 1.0f;
#pragma unroll
            for (int k = 1; k < P1; ++k) {
                tx[k] = tx[k - 1] * dx / (float)k;
                ty[k] = ty[k - 1] * dy / (float)k;
            }
            if (c >= n - 1) {
#pragma unroll
                for (int a = 0; a < P1; ++a)
#pragma unroll
                    for (int b = 0; b < P1; ++b) acc[a][b] = fmaf(tx[a], ty[b], acc[a][b]);
            } else {
                const float* C = coef + (size_t)c * P2;
                float D[P1][P1];  // shift along y first
#pragma unroll
                for (int a = 0; a < P1; ++a)
#pragma unroll
                    for (int b = 0; b < P1; ++b) {
                        float sum = 0.0f;
#pragma unroll
                        for (int bb = 0; bb <= b; ++bb) sum = fmaf(__ldcg(C + a * P1 + bb), ty[b - bb], sum);
                        D[a][b] = sum;
                    }
#pragma unroll
                for (int a = 0; a < P1; ++a)
#pragma unroll
                    for (int b = 0; b < P1; ++b) {
                        float sum = acc[a][b];
#pragma unroll
                        for (int aa = 0; aa <= a; ++aa) sum = fmaf(D[aa][b], tx[a - aa], sum);
                        acc[a][b] = sum;
                    }
            }
        }
        float* out = coef + (size_t)p * P2;
#pragma unroll
        for (int a = 0; a < P1; ++a)
#pragma unroll
            for (int b = 0; b < P1; ++b) __stcg(out + a * P1 + b, acc[a][b]);
        v = p;
    }
}

// ------------------------------------------------ 6 coefficient offsets
__global__ void k_node_sizes(const ViewState* vs, const float4* __restrict__ cen, uint32_t* __restrict__ sizes) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= vs->n - 1) return;
    int d = meta_degree(cen[v].w);
    sizes[v] = d >= 0 ? (uint32_t)((d + 1) * (d + 1)) : 0u;
}

__global__ void k_assign(ViewState* vs, float4* cen, const uint32_t* __restrict__ sizes,
                         const uint32_t* __restrict__ offsets, size_t cap, uds_view_stats* st) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    int n = vs->n;
    if (v >= n - 1) return;
    uint32_t sz = sizes[v];
    if (sz == 0) return;
    float4 c = cen[v];
    int d = meta_degree(c.w);
    uint32_t off = offsets[v];
    if ((size_t)off + sz > cap) {
        c.w = make_meta(0, -1);
        atomicAdd(&st->demoted, 1);
    } else {
        c.w = make_meta((int)off, d);
        atomicMax(&vs->coef_used, off + sz);
    }
    cen[v] = c;
}

// ----------------------------------------------------------------- 7 P2M
// shiftLeafHermiteExpansion (hermitefmm.cuh:119-138) summed per node over
// its leaves in Morton order: C_ab = sum_i t_a(s0_i) t_b(s1_i) with
// t_a(s) = s^a / a!, s = (leaf - centre) * (1 / sqrt(2 h^2)).  A warp builds
// one node at a time.  For a chunk of 32 leaves each lane builds one leaf's
// t-tables in shared memory (t_a = (t_{a-1} s) * (1 / a)); each lane then
// owns a block of BR rows x BC columns of C (the block shape depends on the
// degree, so that the blocks of a (p+1)^2 table fit 32 lanes) and adds
// fma(t_a(s0), t_b(s1), C_ab) leaf by leaf: every coefficient is summed in
// leaf order exactly as the oracle's deterministic flavour does, and one
// shared-memory read feeds BR or BC multiply-adds.  A warp takes 32
// consecutive nodes (one coalesced read of their records and links) and
// builds their expansions one after another: one node per warp left the
// kernel waiting on two dependent memory round trips per few hundred
// multiply-adds.
constexpr int kP2MWarps = 4;
// 1 / a, rounded once at compile time (the oracle uses the same constants)
__constant__ float kInvInt[kMaxDegree + 1] = {0.0f, 1.0f / 1, 1.0f / 2, 1.0f / 3, 1.0f / 4, 1.0f / 5, 1.0f / 6,
                                              1.0f / 7, 1.0f / 8, 1.0f / 9, 1.0f / 10, 1.0f / 11, 1.0f / 12,
                                              1.0f / 13, 1.0f / 14, 1.0f / 15, 1.0f / 16};
constexpr int kTStride = kMaxDegree + 1;  // odd: conflict-free row writes
// rows x columns per lane for p + 1 = 1 .. 17 coefficients per side
__constant__ unsigned char kP2MBlock[kMaxDegree + 2][2] = {
    {1, 1}, {1, 1}, {1, 1}, {1, 1}, {1, 1}, {1, 1}, {1, 2}, {1, 2}, {1, 2},
    {1, 3}, {2, 2}, {2, 3}, {2, 3}, {2, 4}, {2, 4}, {2, 4}, {2, 4}, {3, 4}};

template <int BR, int BC>
__device__ __forceinline__ void p2m_block(const float* tx, const float* ty, int cnt, const int* ra, const int* cb,
                                          float (&acc)[3][4]) {
    for (int j = 0; j < cnt; ++j) {
        float xv[BR], yv[BC];
#pragma unroll
        for (int i = 0; i < BR; ++i) xv[i] = tx[j * kTStride + ra[i]];
#pragma unroll
        for (int k = 0; k < BC; ++k) yv[k] = ty[j * kTStride + cb[k]];
#pragma unroll
        for (int i = 0; i < BR; ++i)
#pragma unroll
            for (int k = 0; k < BC; ++k) acc[i][k] = __fmaf_rn(xv[i], yv[k], acc[i][k]);
    }
}

__global__ void __launch_bounds__(32 * kP2MWarps) k_p2m(const ViewState* vs, const int4* __restrict__ lnk,
                                                        const float4* __restrict__ cen,
                                                        const float2* __restrict__ leaf_xy,
                                                        float* __restrict__ coef) {
    __shared__ float s_tx[kP2MWarps][32 * kTStride];
    __shared__ float s_ty[kP2MWarps][32 * kTStride];
    const unsigned full = 0xffffffffu;
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int n = vs->n;
    float isq = vs->isq;
    // 32 consecutive internal nodes per warp: lane l loads node v0 + l's
    // record and links (one coalesced read), then the warp builds the nodes'
    // expansions one after another
    int v0 = (int)((((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32);
    if (v0 >= n - 1) return;  // uniform over the warp
    int vl = v0 + lane;
    bool inner = vl < n - 1;
    float4 cl = inner ? cen[vl] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    int4 Ll = inner ? lnk[vl] : make_int4(0, 0, 0, 0);
    unsigned todo = __ballot_sync(full, inner && meta_degree(cl.w) >= 0);
    float* tx = s_tx[warp];
    float* ty = s_ty[warp];
    while (todo) {
        int k = __ffs(todo) - 1;
        todo &= todo - 1;
        float4 c;
        c.x = __shfl_sync(full, cl.x, k);
        c.y = __shfl_sync(full, cl.y, k);
        c.w = __shfl_sync(full, cl.w, k);
        int first = __shfl_sync(full, Ll.z, k), count = __shfl_sync(full, Ll.w, k);
        int p = meta_degree(c.w);
        int off = meta_offset(c.w);
        int P1 = p + 1;
        int BR = kP2MBlock[P1][0], BC = kP2MBlock[P1][1];
        int nC = (P1 + BC - 1) / BC, nR = (P1 + BR - 1) / BR;
        int gr = lane / nC, gc = lane % nC;
        bool owner = gr < nR;
        // this lane's rows and columns; reads past the table repeat its last
        // row / column (their sums are not written)
        int ra[3], cb[4];
#pragma unroll
        for (int i = 0; i < 3; ++i) ra[i] = min(gr * BR + i, p);
#pragma unroll
        for (int q = 0; q < 4; ++q) cb[q] = min(gc * BC + q, p);
        float acc[3][4];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][q] = 0.0f;
        int end = first + count;
        for (int i0 = first; i0 < end; i0 += 32) {
            int cnt = min(32, end - i0);
            if (lane < cnt) {
                float2 q = leaf_xy[i0 + lane];
                float s0 = fmul(fsub(q.x, c.x), isq);
                float s1 = fmul(fsub(q.y, c.y), isq);
                float ax = 1.0f, ay = 1.0f;
                tx[lane * kTStride] = 1.0f;
                ty[lane * kTStride] = 1.0f;
                for (int a = 1; a <= p; ++a) {
                    ax = fmul(fmul(ax, s0), kInvInt[a]);
                    ay = fmul(fmul(ay, s1), kInvInt[a]);
                    tx[lane * kTStride + a] = ax;
                    ty[lane * kTStride + a] = ay;
                }
            }
            __syncwarp();
            if (owner) {
                switch (BR * 8 + BC) {  // uniform over the warp
                    case 9: p2m_block<1, 1>(tx, ty, cnt, ra, cb, acc); break;
                    case 10: p2m_block<1, 2>(tx, ty, cnt, ra, cb, acc); break;
                    case 11: p2m_block<1, 3>(tx, ty, cnt, ra, cb, acc); break;
                    case 18: p2m_block<2, 2>(tx, ty, cnt, ra, cb, acc); break;
                    case 19: p2m_block<2, 3>(tx, ty, cnt, ra, cb, acc); break;
                    case 20: p2m_block<2, 4>(tx, ty, cnt, ra, cb, acc); break;
                    default: p2m_block<3, 4>(tx, ty, cnt, ra, cb, acc); break;
                }
            }
            __syncwarp();
        }
        if (owner) {
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    int a = gr * BR + i, b = gc * BC + q;
                    if (i < BR && q < BC && a <= p && b <= p) coef[off + a * P1 + b] = acc[i][q];
                }
        }
    }
}

// -------------------------------------------------------- FGT evaluation
template <typename P>
__device__ __forceinline__ const P* shifted(const P* p, size_t bytes) {
    return reinterpret_cast<const P*>(reinterpret_cast<const char*>(p) + bytes);
}

struct Tree {
    const int4* lnk;
    const int* par;
    const float4* box;
    const float4* cen;
    const float* coef;
    const float2* leaf_xy;
    const int* leaf_id;
    int n;
    float sq;
    float isq;
};

// evluateHermite with hermiteFunction (hermitefmm.cuh:35-47, 213-237): the
// Hermite functions follow the reference's recursion; the series is summed
// row-factored, sum_a h_a(tx) (sum_b C_ab h_b(ty)), with fused multiply-adds
// (the CPU oracle's deterministic flavour sums the same way).
// A leaf's expansion is its own Gaussian: degree 0, coefficient 1.  Callers
// that know they hold a leaf use this directly, which keeps the series'
// loops out of their code.
__device__ __forceinline__ float leaf_mass(const Tree& T, float4 c, float qx, float qy) {
    float tx = fmul(fsub(qx, c.x), T.isq);
    float ty = fmul(fsub(qy, c.y), T.isq);
    float ex = det_expf(-fmul(tx, tx));
    float ey = det_expf(-fmul(ty, ty));
    return fadd(0.0f, fmul(fmul(1.0f, ex), ey));
}

__device__ __forceinline__ float hermite_eval(const Tree& T, int v, float4 c, float qx, float qy) {
    if (v >= T.n - 1) return leaf_mass(T, c, qx, qy);
    float tx = fmul(fsub(qx, c.x), T.isq);
    float ty = fmul(fsub(qy, c.y), T.isq);
    float ex = det_expf(-fmul(tx, tx));
    float ey = det_expf(-fmul(ty, ty));
    int p = meta_degree(c.w);
    const float* C = T.coef + meta_offset(c.w);
    float hy[kMaxDegree + 1];
    float ty2 = fmul(2.0f, ty);
    hy[0] = ey;
    hy[1] = fmul(ty2, ey);
#pragma unroll
    for (int k = 2; k <= kMaxDegree; ++k)
        if (k <= p) hy[k] = fsub(fmul(ty2, hy[k - 1]), fmul(fmul(2.0f, (float)(k - 1)), hy[k - 2]));
    float tx2 = fmul(2.0f, tx);
    float hxm2 = 0.0f, hxm1 = 0.0f;
    float w = 0.0f;
    const int P1 = p + 1;
    int a = 0;
    // Rows four at a time: the four row sums are independent chains, so they
    // are interleaved; each chain and the outer sum keep their order.
    for (; a + 4 <= P1; a += 4) {
        float h[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            int aa = a + q;
            float hx = aa == 0 ? ex
                               : (aa == 1 ? fmul(tx2, ex)
                                          : fsub(fmul(tx2, hxm1), fmul(fmul(2.0f, (float)(aa - 1)), hxm2)));
            h[q] = hx;
            hxm2 = hxm1;
            hxm1 = hx;
        }
        const float* C0 = C + a * P1;
        float r0 = 0.0f, r1 = 0.0f, r2 = 0.0f, r3 = 0.0f;
#pragma unroll
        for (int b = 0; b <= kMaxDegree; ++b) {
            if (b <= p) {
                r0 = __fmaf_rn(C0[b], hy[b], r0);
                r1 = __fmaf_rn(C0[P1 + b], hy[b], r1);
                r2 = __fmaf_rn(C0[2 * P1 + b], hy[b], r2);
                r3 = __fmaf_rn(C0[3 * P1 + b], hy[b], r3);
            }
        }
        w = __fmaf_rn(h[0], r0, w);
        w = __fmaf_rn(h[1], r1, w);
        w = __fmaf_rn(h[2], r2, w);
        w = __fmaf_rn(h[3], r3, w);
    }
    for (; a <= p; ++a) {
        float hx = a == 0 ? ex
                          : (a == 1 ? fmul(tx2, ex) : fsub(fmul(tx2, hxm1), fmul(fmul(2.0f, (float)(a - 1)), hxm2)));
        const float* Ca = C + a * P1;
        float r = 0.0f;
#pragma unroll
        for (int b = 0; b <= kMaxDegree; ++b)
            if (b <= p) r = __fmaf_rn(Ca[b], hy[b], r);
        w = __fmaf_rn(hx, r, w);
        hxm2 = hxm1;
        hxm1 = hx;
    }
    return w;
}

__device__ __forceinline__ bool truncated_box(float4 b, float r, float qx, float qy) {
    float clx = fminf(fmaxf(qx, b.x), b.z), cly = fminf(fmaxf(qy, b.y), b.w);
    float dx = fsub(qx, clx), dy = fsub(qy, cly);
    float d2 = fadd(fadd(0.0f, fmul(dx, dx)), fmul(dy, dy));
    return !(d2 < fmul(r, r));
}

__device__ __forceinline__ bool truncated(const Tree& T, int v, float r, float qx, float qy) {
    return truncated_box(T.box[v], r, qx, qy);
}

// getWeight / accumulateSubtree (evaluateDynamicRadixTree.cuh:129-242):
// stackless depth-first walk summing, in visiting order, the expansions of
// the nodes that carry one and skipping subtrees whose box misses the
// truncation circle.  A walk visits each node at most twice, so the step
// budget 4n + 64 only guards against a malformed tree.
__device__ float node_weight(const Tree& T, int v, float qx, float qy) {
    float4 c = T.cen[v];
    if (meta_degree(c.w) >= 0) return hermite_eval(T, v, c, qx, qy);
    int rootparent = T.par[v];
    float w = 0.0f;
    int budget = 4 * T.n + 64;
    do {
        c = T.cen[v];
        while (meta_degree(c.w) < 0 && !truncated(T, v, c.z, qx, qy)) {
            int l = T.lnk[v].x;
            if (l < 0 || --budget < 0) return w;
            v = l;
            c = T.cen[v];
        }
        if (meta_degree(c.w) >= 0) w = fadd(w, hermite_eval(T, v, c, qx, qy));
        int p = T.par[v];
        while (p != rootparent && v == T.lnk[p].y) {
            if (--budget < 0) return w;
            v = p;
            p = T.par[p];
        }
        if (p != rootparent) v = T.lnk[p].y;
    } while (T.par[v] != rootparent && --budget >= 0);
    return w;
}

__device__ __noinline__ float node_weight_out_of_line(Tree T, int v, float qx, float qy) {
    return node_weight(T, v, qx, qy);
}

// --------------------------------------------------------------- 8 sampler
// Per-pixel mass cache.  getWeight(v) of a node without expansion that the
// truncation circle reaches is the running sum, in depth-first order, of the
// expansions below it; one walk from the root therefore yields getWeight of
// every node it opens if each opened node keeps its own running sum, fed the
// same values in the same order (so the sums are bit-identical to separate
// walks).  The opened nodes and the frontier nodes whose expansion the walk
// evaluated are stored in pre-order, one 8-byte record each: the mass and
// the entries of the two children.  A child entry is -1 when the child's box
// misses the truncation circle (it has no expansion, so its getWeight is
// exactly 0) and -2 below an expansion (not walked: its children's masses
// are evaluated when needed).  The descent reads one record per child and
// level.
constexpr int kTable = 160;
constexpr int kNotWalked = -2;

__device__ __forceinline__ int2 mass_rec(float mass, int left, int right) {
    return make_int2(__float_as_int(mass), (int)(((unsigned)left & 0xffffu) | ((unsigned)right << 16)));
}
__device__ __forceinline__ float rec_mass(int2 r) { return __int_as_float(r.x); }
__device__ __forceinline__ int rec_left(int2 r) { return (int)(short)(r.y & 0xffff); }
__device__ __forceinline__ int rec_right(int2 r) { return r.y >> 16; }
// the record of a node the cache does not hold
__device__ __forceinline__ int2 no_record() { return mass_rec(0.0f, kNotWalked, kNotWalked); }

struct MassCache {
    int2 rec[kTable];
    int m;
    bool ok;
};

// Warp-cooperative walk.  The 32 pixels of a warp (an 8 x 4 tile) walk the
// union of their trees in lock-step.  At a node, every lane inside tests its
// own truncation circle; lanes that open the node continue into its children,
// the others leave that subtree.  Restricted to one lane, the union walk
// visits exactly that lane's nodes in its own depth-first order, so the
// running sums are unchanged; but expansion coefficients are now loaded once
// per warp and the Hermite loops run with warp-uniform bounds.
//
// Each iteration enters one node (its centre, box and links in one round
// trip to memory); the stack in shared memory holds the opened ancestors
// (lanes that opened each, its right child), and whether an ancestor's right
// subtree is under way is one bit of a register.  After a node that is not
// descended into, finished ancestors are closed in the same iteration.
//
// The running sums of a lane's opened ancestors live in shared memory,
// acc[depth][lane]: every lane inside a node has opened the same ancestors,
// so the update loop over them has one trip count per warp and touches one
// bank per lane; each sum is written to the lane's cache once, when its node
// is closed.  The stack holds kWalkDepth levels (the trees built here are
// about 20-30 deep; a smaller block leaves more of the SM's L1 to the
// per-lane caches).  A lane whose walk would go deeper gives up its cache
// (the descent then evaluates masses directly) and takes its total from a
// direct subtree walk.
constexpr int kWalkDepth = 40;
struct WalkStack {
    unsigned mask[kWalkDepth];  // lanes that opened the ancestor at this depth
    int right[kWalkDepth];      // its right child
    float acc[kWalkDepth][32];
};

__device__ void warp_root_walk(const Tree& T, float qx, float qy, bool live, MassCache& mc, float& total,
                               WalkStack& ws) {
    const unsigned full = 0xffffffffu;
    const int lane = (threadIdx.x + blockDim.x * threadIdx.y) & 31;
    mc.m = 0;
    mc.ok = true;
    total = 0.0f;
    unsigned liveMask = __ballot_sync(full, live);
    float4 c = T.cen[0];
    if (meta_degree(c.w) >= 0) {
        if (live) total = hermite_eval(T, 0, c, qx, qy);
        return;
    }
    if (!liveMask) return;
    // per opened ancestor (same index in every lane inside): its entry, its
    // left child's entry and where its right child's entry would start
    int ostack[kWalkDepth], lstack[kWalkDepth], rstack[kWalkDepth];
    int osp = 0;
    int sp = -1;                    // deepest opened ancestor of v
    unsigned long long onright = 0; // bit k: ancestor k's right subtree is under way
    int v = 0;                      // node entered next, and the lanes inside it
    unsigned in = liveMask;
    bool deep = false;  // a subtree was not walked: total is incomplete
    int budget = 4 * T.n + 64;
    while (true) {
        if (--budget < 0) { mc.ok = false; deep = true; break; }
        bool mine = (in >> lane) & 1u;
        c = T.cen[v];
        float4 bx = T.box[v];
        int4 Lv = T.lnk[v];
        bool descend = false;
        if (meta_degree(c.w) >= 0) {
            if (mine) {
                float val = hermite_eval(T, v, c, qx, qy);
                total = fadd(total, val);
                if (mc.ok) {
                    for (int q = 0; q < osp; ++q) ws.acc[q][lane] = fadd(ws.acc[q][lane], val);
                    if (mc.m < kTable) {
                        mc.rec[mc.m] = mass_rec(val, kNotWalked, kNotWalked);
                        ++mc.m;
                    } else {
                        mc.ok = false;
                    }
                }
            }
        } else {
            bool op = mine && !truncated_box(bx, c.z, qx, qy);
            unsigned opened = __ballot_sync(full, op);
            // v sits at depth sp + 1; its children would be at sp + 2
            if (opened && sp + 2 >= kWalkDepth) {
                if (op) {  // this lane's subtree below v is not walked
                    mc.ok = false;
                    deep = true;
                }
            } else if (opened) {
                if (op && mc.ok) {
                    if (mc.m < kTable && osp < kWalkDepth) {
                        ws.acc[osp][lane] = 0.0f;
                        ostack[osp++] = mc.m++;
                    } else {
                        mc.ok = false;
                    }
                }
                ++sp;
                onright &= ~(1ull << sp);
                if (lane == 0) {
                    ws.mask[sp] = opened;
                    ws.right[sp] = Lv.y;
                }
                v = Lv.x;
                in = opened;
                descend = true;
            }
        }
        __syncwarp();
        if (descend) continue;
        // climb: close ancestors whose right subtree is done; at the first
        // one whose left subtree is done, continue with its right child
        bool more = false;
        while (sp >= 0) {
            unsigned pin = ws.mask[sp];
            bool pm = (pin >> lane) & 1u;
            if (!((onright >> sp) & 1ull)) {
                // the left child, if recorded, directly follows its parent
                if (pm && mc.ok) {
                    int q = ostack[osp - 1];
                    lstack[osp - 1] = mc.m > q + 1 ? q + 1 : -1;
                    rstack[osp - 1] = mc.m;
                }
                onright |= 1ull << sp;
                v = ws.right[sp];
                in = pin;
                more = true;
                break;
            }
            if (pm && mc.ok) {
                int q = ostack[--osp];
                int rs = rstack[osp];
                mc.rec[q] = mass_rec(ws.acc[osp][lane], lstack[osp], mc.m > rs ? rs : -1);
            }
            --sp;
        }
        if (!more) break;
        __syncwarp();  // the stack slots read above may be rewritten next
    }
    // the same running sum in the same order, by a direct walk (rare: out of
    // line)
    if (deep && live) total = node_weight_out_of_line(T, 0, qx, qy);
}

// Child masses (w0, w1) = getWeight of the children (a, b) for every lane
// of the warp with `need` (all lanes call this together); the value of each
// is the same node_weight call whichever lane makes it, so both forms below
// give identical masses, only the speed differs (the autotuner picks one per
// view shape; uds_sample_params.spread).
// SPREAD false: every needing lane evaluates its own two children, left then
//   right; neighbouring pixels at the same node evaluate the same child side
//   by side (equal trip counts, one coefficient stream).
// SPREAD true: the 2c evaluations of the c needing lanes are spread over the
//   warp's 32 lanes, first the left children of the needing lanes (in lane
//   order), then their right children, so a lane waits for one series
//   instead of two while c <= 16.  `owner`: 32 ints of the warp's shared
//   memory.
template <bool SPREAD>
__device__ __forceinline__ void warp_child_masses(const Tree& T, bool need, int a, int b, float qx, float qy,
                                                  float& w0, float& w1, int* owner) {
    if (!SPREAD) {
        if (need) {
#pragma unroll 1
            for (int ch = 0; ch < 2; ++ch) {
                float x = fmaxf(0.0f, node_weight(T, ch ? b : a, qx, qy));
                if (ch) w1 = x; else w0 = x;
            }
        }
        return;
    }
    const unsigned full = 0xffffffffu;
    unsigned nm = __ballot_sync(full, need);
    if (!nm) return;
    const int lane = (threadIdx.x + blockDim.x * threadIdx.y) & 31;
    int c = __popc(nm), c2 = 2 * c;
    int rank = __popc(nm & ((1u << lane) - 1u));
    if (need) owner[rank] = lane;
    __syncwarp();
#pragma unroll 1
    for (int e0 = 0; e0 < c2; e0 += 32) {
        int e = e0 + lane;
        bool right = e >= c;
        int o = e < c2 ? owner[right ? e - c : e] : lane;
        float oqx = __shfl_sync(full, qx, o), oqy = __shfl_sync(full, qy, o);
        int oa = __shfl_sync(full, a, o), ob = __shfl_sync(full, b, o);
        float x = 0.0f;
        if (e < c2) x = fmaxf(0.0f, node_weight(T, right ? ob : oa, oqx, oqy));
        int s0 = rank - e0, s1 = c + rank - e0;  // lanes holding this lane's children in this pass
        float x0 = __shfl_sync(full, x, s0 & 31), x1 = __shfl_sync(full, x, s1 & 31);
        if (need && s0 >= 0 && s0 < 32) w0 = x0;
        if (need && s1 >= 0 && s1 < 32) w1 = x1;
    }
    __syncwarp();  // owner is rewritten by the next call
}

// Views of different sizes in one descent launch: blocks [first[v],
// first[v+1]) of the one-dimensional grid cover view v, bx[v] blocks along
// y per block row; its indices start at entry ioff[v] of the packed output.
constexpr int kMaxUneven = 32;
struct UnevenViews {
    int nv;
    int first[kMaxUneven + 1];
    int bx[kMaxUneven];
    int W[kMaxUneven], H[kMaxUneven];
    long long ioff[kMaxUneven];
};

template <int R, int KM, bool UNEVEN, bool SPREAD>
__global__ void __launch_bounds__(128, 4) k_sample(Tree T, const ViewState* vs, int W, int H, int K,
                                                int M, float precision, const float* __restrict__ uniforms,
                                                uint64_t seed, const uint64_t* __restrict__ seed_ptr,
                                                uint32_t view, int* __restrict__ indices, uds_view_stats* st,
                                                size_t vstride, size_t ustride, size_t istride, UnevenViews uv) {
    // block tile_x (y) x 128 / tile_x (x).  blockIdx.z selects the
    // view: its tree lives vstride bytes after the previous view's, its
    // uniforms ustride floats and its indices istride entries further on.
    // With UNEVEN the view and the block's place in it come from uv
    // (blockIdx.x only; no uniforms tensor).
    if (seed_ptr) seed = *seed_ptr;
    unsigned bxi = blockIdx.x, byi = blockIdx.y, vz = blockIdx.z;
    if (UNEVEN) {
        int b = 0;
        while (b + 1 < uv.nv && uv.first[b + 1] <= (int)blockIdx.x) ++b;
        int local = (int)blockIdx.x - uv.first[b];
        bxi = (unsigned)(local % uv.bx[b]);
        byi = (unsigned)(local / uv.bx[b]);
        vz = (unsigned)b;
        W = uv.W[b];
        H = uv.H[b];
        indices += uv.ioff[b];
    }
    if (vz) {
        size_t off = (size_t)vz * vstride;
        T.lnk = shifted(T.lnk, off);
        T.par = shifted(T.par, off);
        T.box = shifted(T.box, off);
        T.cen = shifted(T.cen, off);
        T.coef = shifted(T.coef, off);
        T.leaf_xy = shifted(T.leaf_xy, off);
        T.leaf_id = shifted(T.leaf_id, off);
        vs = shifted(vs, off);
        view += vz;
        if (!UNEVEN) {
            indices += (size_t)vz * istride;
            if (uniforms) uniforms += (size_t)vz * ustride;
        }
        st += vz;
    }
    __shared__ WalkStack s_walk[4];
    const unsigned full = 0xffffffffu;
    int j = bxi * blockDim.x + threadIdx.x;
    int i = byi * blockDim.y + threadIdx.y;
    int tid = threadIdx.x + blockDim.x * threadIdx.y;
    int warp = tid >> 5, lane = tid & 31;
    bool live = (i < W && j < H);
    T.n = vs->n;
    T.sq = vs->sq;
    T.isq = vs->isq;
    if (T.n == 0) return;  // indices were preset to -1 (uniform over the grid)
    size_t pixel = (size_t)j + (size_t)H * i;
    float qx = (float)i, qy = (float)j;
    MassCache mc;
    float total;
    warp_root_walk(T, qx, qy, live, mc, total, s_walk[warp]);
    int* ws_owner = s_walk[warp].right;  // free once the walk is done
    total = fmaxf(0.0f, total);
    bool act = live && !(total < precision);
    if (!__any_sync(full, act)) return;
    // K-sized arrays stay in registers for K <= 16 (loops fully unrolled)
    constexpr int UK = KM <= 16 ? KM : 1;
    int ids[KM];
    float keys[KM];
#pragma unroll UK
    for (int k = 0; k < KM; ++k) { ids[k] = -1; keys[k] = __int_as_float(0x7f800000); }
    // each round's path is kept as its choice bits (bit m: right child taken
    // at depth m) and its length, in registers: two rounds meet the same node
    // at depth m iff their first m choices agree (node ids are unique)
    unsigned long long pb[R];
    float tc[R][kTrace];
    float tp[kTrace];
    int tl[R];
#pragma unroll
    for (int rr = 0; rr < R; ++rr) { pb[rr] = 0ull; tl[rr] = 0; }
    // child masses of the node met at each depth by the latest round; slots
    // [0, cvn) are valid (depths are reached in order, so no clearing needed)
    int cv[kTrace];
    float cw0[kTrace], cw1[kTrace];
    int cvn = 0;
    bool overflow = false;
    for (int r = 0; r < R; ++r) {
        int v = 0, d = 0;
        const int2 no_rec = no_record();
        int2 rc = (mc.ok && mc.m > 0) ? mc.rec[0] : no_rec;  // cache record of v
        unsigned long long cur = 0ull;                        // this round's choice bits so far
        tp[0] = 1.0f;
        int4 L = T.lnk[0];
        bool going = act && L.w > M;
        while (__any_sync(full, going)) {
            int a = L.x, b = L.y;
            float w0 = 0.0f, w1 = 0.0f;
            int2 ra = no_rec, rb = no_rec;  // the children's records
            bool need = false;
            if (going) {
                int ia = rec_left(rc), ib = rec_right(rc);
                if (ia != kNotWalked) {
                    if (ia >= 0) { ra = mc.rec[ia]; w0 = fmaxf(0.0f, rec_mass(ra)); }
                    if (ib >= 0) { rb = mc.rec[ib]; w1 = fmaxf(0.0f, rec_mass(rb)); }
                } else if (d < cvn && cv[d] == v) {
                    w0 = cw0[d];
                    w1 = cw1[d];
                } else {
                    need = true;
                }
            }
            // every lane that needs its node's child masses gets them in the
            // same pass, whatever node it is at (below the expansion frontier
            // a child is one expansion, so the divergence is only in the
            // series' trip counts); one call site keeps the walk inlined once,
            // small enough for the instruction cache
            warp_child_masses<SPREAD>(T, need, a, b, qx, qy, w0, w1, ws_owner);
            if (going) {
                // (re)write unconditionally: a hit stores the same masses, and
                // a store does not wait on the per-thread memory like a load
                cv[d] = v;
                cw0[d] = w0;
                cw1[d] = w1;
                if (d >= cvn) cvn = d + 1;
                float sum = fadd(fadd(0.0f, w0), w1);
                w0 = fdiv(w0, sum);
                w1 = fdiv(w1, sum);
                // capacities of a and b: from the latest earlier round whose
                // path passed through v (same first d choices) into that child
                float c0 = 1.0f, c1 = 1.0f;
                bool f0 = false, f1 = false;
                unsigned long long pre = (1ull << d) - 1ull;
#pragma unroll
                for (int rr = R - 1; rr >= 0; --rr) {
                    if (rr < r && d + 1 < tl[rr] && ((pb[rr] ^ cur) & pre) == 0ull) {
                        bool right = (pb[rr] >> d) & 1ull;
                        if (!right && !f0) { c0 = tc[rr][d + 1]; f0 = true; }
                        if (right && !f1) { c1 = tc[rr][d + 1]; f1 = true; }
                    }
                }
                float s0 = fmul(w0, c0), s1 = fmul(w1, c1);
                ++d;
                if (d >= kTrace) {
                    overflow = true;
                    going = false;
                    act = false;
                } else {
                    if (s0 < s1) { cur |= 1ull << (d - 1); tp[d] = w1; v = b; rc = rb; }
                    else { tp[d] = w0; v = a; rc = ra; }
                    L = T.lnk[v];
                    going = L.w > M;
                }
            }
        }
        if (!act) continue;
#pragma unroll
        for (int rr = 0; rr < R; ++rr)
            if (rr == r) { pb[rr] = cur; tl[rr] = d + 1; }
        float prob = 1.0f;
        for (int m = d; m >= 0; --m) {
            float cap = 1.0f;
            bool found = false;
            unsigned long long pre = (1ull << m) - 1ull;
#pragma unroll
            for (int rr = R - 1; rr >= 0; --rr)
                if (rr < r && !found && m < tl[rr] && ((pb[rr] ^ cur) & pre) == 0ull) { cap = tc[rr][m]; found = true; }
            tc[r][m] = fmaxf(0.0f, fsub(cap, prob));
            prob = fmul(prob, tp[m]);
        }
        // order sampling over the subtree's leaves (insertSample,
        // sequentialPoissonRadixTree.cuh:15-41); a leaf's mass is its own
        // Gaussian (degree 0, coefficient 1).  The subtree holds at most M
        // leaves: K, or the leaf size when that is larger.
        int f0 = L.z, cnt = L.w;
        // the round's uniforms, drawn as the leaves use them (after the
        // descent, so they hold no registers there): Philox block
        // (pixel, view, r * ceil(M / 4) + k / 4), or the caller's tensor
        const float* up = uniforms ? uniforms + ((size_t)pixel * R + r) * M : nullptr;
        const int G = (M + 3) >> 2;
        uint32_t c4[4];
#pragma unroll 1
        for (int k0 = 0; k0 < cnt; k0 += 4) {
            if (!up) {
                c4[0] = (uint32_t)pixel; c4[1] = view; c4[2] = (uint32_t)(r * G + (k0 >> 2)); c4[3] = 0u;
                philox4x32_10(c4, (uint32_t)seed, (uint32_t)(seed >> 32));
            }
#pragma unroll
            for (int k4 = 0; k4 < 4; ++k4) {
                int k = k0 + k4;
                if (k < cnt) {
                    float uk = up ? up[k] : bits_to_uniform(c4[k4]);
                    int leafNode = T.n - 1 + f0 + k;
                    float pw = fmaxf(0.0f, leaf_mass(T, T.cen[leafNode], qx, qy));
                    float key = fdiv(uk, pw);
                    int index = T.leaf_id[f0 + k];
                    bool done = false;
#pragma unroll UK
                    for (int q = 0; q < KM; ++q) {
                        if (!done && q < K) {
                            if (key < keys[q]) {
                                int ti = ids[q]; ids[q] = index; index = ti;
                                float tk = keys[q]; keys[q] = key; key = tk;
                            }
                            if (index == -1) done = true;
                        }
                    }
                }
            }
        }
    }
    if (overflow) atomicAdd(&st->overflow, 1);
    if (!live) return;
    int* out = indices + (size_t)K * pixel;
#pragma unroll UK
    for (int k = 0; k < KM; ++k)
        if (k < K) out[k] = ids[k];
}

// Stochastic mode (no reference counterpart).  Each of the K draws of a
// pixel descends from the root into a child with probability
// m_child / (m_left + m_right), masses by getWeight, and records the product
// q of the ratios it took: the probability of having drawn that leaf, which
// importance-weighted estimators divide by.  Draw k at depth d uses Philox
// counter (pixel, view, 2^31 | k << 8 | d / 4, 0), component d % 4, and steps
// left iff u <= m_left / (m_left + m_right).  The draws of one pixel share
// their upper paths, so the child masses of the last path are kept per depth
// (node ids are unique, so a hit is exact).  A draw that meets two zero
// masses, or is still above the leaves after kTrace levels, stays -1 / 0.
__global__ void __launch_bounds__(128, 4) k_stochastic(Tree T, const ViewState* vs, int W, int H, int K,
                                                       float precision, uint64_t seed,
                                                       const uint64_t* __restrict__ seed_ptr, uint32_t view,
                                                       int* __restrict__ indices, float* __restrict__ probs,
                                                       uds_view_stats* st, const unsigned char* __restrict__ mask,
                                                       float* __restrict__ weights) {
    // same warp layout and per-pixel mass cache as k_sample: one warp walks
    // its 32 pixels' trees together, then every lane draws its K paths; the
    // masses come from the cache, the per-depth cache of earlier draws, or a
    // direct evaluation by each lane that needs them (all bit-identical to
    // separate getWeight calls)
    if (seed_ptr) seed = *seed_ptr;
    __shared__ WalkStack s_walk[4];
    const unsigned full = 0xffffffffu;
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y * blockDim.y + threadIdx.y;
    int tid = threadIdx.x + blockDim.x * threadIdx.y;
    int warp = tid >> 5;
    size_t pixel = (size_t)j + (size_t)H * i;
    bool live = (i < W && j < H) && (!mask || mask[pixel]);
    T.n = vs->n;
    T.sq = vs->sq;
    T.isq = vs->isq;
    int n = T.n;
    if (n == 0) return;
    float qx = (float)i, qy = (float)j;
    MassCache mc;
    float m0;
    warp_root_walk(T, qx, qy, live, mc, m0, s_walk[warp]);
    m0 = fmaxf(0.0f, m0);
    bool act = live && !(m0 < precision);
    if (!__any_sync(full, act)) return;
    int cv[kTrace];
    float cw0[kTrace], cw1[kTrace];
    int cvn = 0;
    bool overflow = false;
    for (int k = 0; k < K; ++k) {
        int v = 0, d = 0;
        const int2 no_rec = no_record();
        int2 rc = (mc.ok && mc.m > 0) ? mc.rec[0] : no_rec;
        float prob = 1.0f;
        uint32_t c[4];
        bool ok = act;
        int4 L = T.lnk[0];
        bool going = act && v < n - 1;
        while (__any_sync(full, going)) {
            int a = L.x, b = L.y;
            float w0 = 0.0f, w1 = 0.0f;
            int2 ra = no_rec, rb = no_rec;  // the children's records
            int4 La = L, Lb = L;            // and links, loaded with them
            bool need = false;
            if (going) {
                La = T.lnk[a];
                Lb = T.lnk[b];
                int ia = rec_left(rc), ib = rec_right(rc);
                if (ia != kNotWalked) {
                    if (ia >= 0) { ra = mc.rec[ia]; w0 = fmaxf(0.0f, rec_mass(ra)); }
                    if (ib >= 0) { rb = mc.rec[ib]; w1 = fmaxf(0.0f, rec_mass(rb)); }
                } else if (d < cvn && cv[d] == v) {
                    w0 = cw0[d];
                    w1 = cw1[d];
                } else {
                    need = true;
                }
            }
            // every lane that needs its node's child masses gets them in the
            // same pass (one call site: the walk is inlined once)
            warp_child_masses<false>(T, need, a, b, qx, qy, w0, w1, s_walk[warp].right);
            if (going) {
                cv[d] = v;
                cw0[d] = w0;
                cw1[d] = w1;
                if (d >= cvn) cvn = d + 1;
                if ((d & 3) == 0) {
                    c[0] = (uint32_t)pixel; c[1] = view; c[2] = 0x80000000u | ((uint32_t)k << 8) | (uint32_t)(d >> 2);
                    c[3] = 0;
                    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
                }
                float u = bits_to_uniform(c[d & 3]);
                float sum = fadd(fadd(0.0f, w0), w1);
                if (!(sum > 0.0f)) {
                    ok = false;
                    going = false;
                } else {
                    float r0 = fdiv(w0, sum);
                    if (u <= r0) { prob = fmul(prob, r0); v = a; rc = ra; L = La; }
                    else { prob = fmul(prob, fdiv(w1, sum)); v = b; rc = rb; L = Lb; }
                    ++d;
                    if (d >= kTrace && v < n - 1) {
                        ok = false;
                        overflow = true;
                        going = false;
                    } else {
                        going = v < n - 1;
                    }
                }
            }
        }
        if (ok) {
            size_t o = (size_t)K * pixel + k;
            indices[o] = T.leaf_id[v - (n - 1)];
            probs[o] = prob;
            // importance weight of the draw: (leaf mass / root mass) / q
            if (weights) weights[o] = leaf_mass(T, T.cen[v], qx, qy) / m0 / prob;
        }
    }
    if (overflow) atomicAdd(&st->overflow, 1);
}

// ============================================================ proposal
// Learned proposal for the stochastic mode (no reference counterpart).  A
// draw descends from the root; at each internal node a small network maps
// 16 cheap features of the node's two children (offsets of the query from
// their centres, their leaf counts, box distances and sizes, all in units of
// sqrt(2) h) to the probability q of the left branch, instead of evaluating
// both children's FGT masses.  The draw's importance weight is
// p / q_path with p = (leaf Gaussian) / (root FGT mass): only the root mass
// is evaluated per pixel, and the weighted estimator stays unbiased because
// q > 0 on every branch.  The descent runs level-synchronously over all
// draws so that each level's network evaluations form one batch for the
// tensor-core kernel (uds_mlp_forward_dev).
constexpr int kFeat = 16;

__device__ __forceinline__ float feat_clamp(float x) { return fminf(fmaxf(x, -16.0f), 16.0f); }

__device__ __forceinline__ float box_distance(float4 b, float qx, float qy) {
    float dx = fmaxf(fmaxf(b.x - qx, qx - b.z), 0.0f), dy = fmaxf(fmaxf(b.y - qy, qy - b.w), 0.0f);
    return sqrtf(dx * dx + dy * dy);
}

__device__ void branch_features(const Tree& T, int v, int depth, float qx, float qy, float* f) {
    int4 L = T.lnk[v];
    float is = T.isq;
    float bd[2];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        int x = c ? L.y : L.x;
        float4 cc = T.cen[x], b = T.box[x];
        int cnt = T.lnk[x].w;
        bd[c] = box_distance(b, qx, qy) * is;
        f[6 * c + 0] = feat_clamp((qx - cc.x) * is);
        f[6 * c + 1] = feat_clamp((qy - cc.y) * is);
        f[6 * c + 2] = log2f((float)cnt) * 0.125f;
        f[6 * c + 3] = feat_clamp(bd[c]);
        f[6 * c + 4] = feat_clamp(0.5f * sqrtf((b.z - b.x) * (b.z - b.x) + (b.w - b.y) * (b.w - b.y)) * is);
        f[6 * c + 5] = x >= T.n - 1 ? 1.0f : 0.0f;
    }
    f[12] = (float)depth * (1.0f / 32.0f);
    f[13] = log2f((float)L.w) * 0.125f;
    f[14] = feat_clamp(bd[0] - bd[1]);
    f[15] = 0.0f;
}

__device__ __forceinline__ float draw_uniform(uint64_t seed, uint32_t pixel, uint32_t view, uint32_t tag, int k,
                                              int level) {
    uint32_t c[4] = {pixel, view, tag | ((uint32_t)k << 8) | (uint32_t)(level >> 2), 0u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    return bits_to_uniform(c[level & 3]);
}

// Training rows: plain stochastic descents (exact FGT masses) from every
// stride-th pixel in each direction, `draws` per pixel; each internal node
// visited gives (features, m_left / (m_left + m_right)).
__global__ void __launch_bounds__(128) k_prop_dataset(Tree T, const ViewState* vs, int W, int H, int stride,
                                                      int draws, float precision, uint64_t seed, uint32_t view,
                                                      float* __restrict__ X, float* __restrict__ target,
                                                      long long* __restrict__ keys, int* __restrict__ count,
                                                      int cap) {
    int j = (blockIdx.x * blockDim.x + threadIdx.x) * stride;
    int i = (blockIdx.y * blockDim.y + threadIdx.y) * stride;
    if (i >= W || j >= H) return;
    T.n = vs->n;
    T.sq = vs->sq;
    T.isq = vs->isq;
    int n = T.n;
    if (n < 2) return;
    float qx = (float)i, qy = (float)j;
    if (fmaxf(0.0f, node_weight(T, 0, qx, qy)) < precision) return;
    uint32_t pixel = (uint32_t)(j + H * i);
    int cn[kTrace];
    float cm0[kTrace], cm1[kTrace];
    for (int d = 0; d < kTrace; ++d) cn[d] = -1;
    for (int k = 0; k < draws; ++k) {
        int v = 0;
        for (int d = 0; v < n - 1 && d < kTrace; ++d) {
            int4 L = T.lnk[v];
            float w0, w1;
            if (cn[d] == v) {
                w0 = cm0[d];
                w1 = cm1[d];
            } else {
                w0 = fmaxf(0.0f, node_weight(T, L.x, qx, qy));
                w1 = fmaxf(0.0f, node_weight(T, L.y, qx, qy));
                cn[d] = v;
                cm0[d] = w0;
                cm1[d] = w1;
            }
            float sum = w0 + w1;
            if (!(sum > 0.0f)) break;
            float pl = w0 / sum;
            int r = atomicAdd(count, 1);
            if (r < cap) {
                float f[kFeat];
                branch_features(T, v, d, qx, qy, f);
#pragma unroll
                for (int q = 0; q < kFeat; ++q) X[(size_t)r * kFeat + q] = f[q];
                target[r] = pl;
                if (keys) keys[r] = ((long long)pixel << 16) | ((long long)k << 8) | d;
            }
            v = draw_uniform(seed, pixel, view, 0xA0000000u, k, d) <= pl ? L.x : L.y;
        }
    }
}

// Per pixel: root mass; active pixels put their K draws on the list.
__global__ void k_prop_init(Tree T, const ViewState* vs, int W, int H, int K, float precision,
                            float* __restrict__ root_mass, int* __restrict__ node_out, int* __restrict__ draw_out,
                            float* __restrict__ logq_out, int* __restrict__ count_out, int* __restrict__ indices,
                            float* __restrict__ weights) {
    // root masses by the warp-cooperative walk of k_sample (128-thread
    // blocks, warps of consecutive threads)
    __shared__ WalkStack s_walk[4];
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y * blockDim.y + threadIdx.y;
    int warp = (threadIdx.x + blockDim.x * threadIdx.y) >> 5;
    bool live = i < W && j < H;
    T.n = vs->n;
    T.sq = vs->sq;
    T.isq = vs->isq;
    size_t pixel = (size_t)j + (size_t)H * i;
    float qx = (float)i, qy = (float)j;
    float m0 = 0.0f;
    if (T.n > 0) {
        MassCache mc;
        warp_root_walk(T, qx, qy, live, mc, m0, s_walk[warp]);
        m0 = fmaxf(0.0f, m0);
    }
    if (!live) return;
    root_mass[pixel] = m0;
    if (T.n == 0 || m0 < precision) return;
    if (T.n == 1) {  // the root is the only leaf
        for (int k = 0; k < K; ++k) {
            indices[(size_t)K * pixel + k] = T.leaf_id[0];
            weights[(size_t)K * pixel + k] = leaf_mass(T, T.cen[0], qx, qy) / m0;
        }
        return;
    }
    int base = atomicAdd(count_out, K);
    for (int k = 0; k < K; ++k) {
        node_out[base + k] = 0;
        draw_out[base + k] = (int)(pixel * K + k);
        logq_out[base + k] = 0.0f;
    }
}

// Rows go straight into the network's operand layout: bf16, 128-row tiles of
// 4096 bytes, K-major core matrices (two 16-byte stores per row), so the
// network kernel can stream whole tiles with bulk copies.
__global__ void k_prop_features(Tree T, const ViewState* vs, int H, int K, int level, const int* __restrict__ count,
                                const int* __restrict__ node_in, const int* __restrict__ draw_in,
                                unsigned char* __restrict__ Xt) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= *count) return;
    T.n = vs->n;
    T.sq = vs->sq;
    T.isq = vs->isq;
    int pixel = draw_in[r] / K;
    float qx = (float)(pixel / H), qy = (float)(pixel % H);
    float f[kFeat];
    branch_features(T, node_in[r], level, qx, qy, f);
    unsigned char* tile = Xt + (size_t)(r >> 7) * (128 * kFeat * 2);
#pragma unroll
    for (int c = 0; c < kFeat; c += 8) {
        __nv_bfloat162 h[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) h[q] = __floats2bfloat162_rn(f[c + 2 * q], f[c + 2 * q + 1]);
        *reinterpret_cast<uint4*>(tile + tc::kmajor_offset(r & 127, c, kFeat)) = *reinterpret_cast<uint4*>(h);
    }
}

// Take one branch per draw with the network's q; finished draws write their
// leaf and importance weight, the others go on the next level's list.
__global__ void k_prop_step(Tree T, const ViewState* vs, int H, int K, int level, uint64_t seed,
                            const uint64_t* __restrict__ seed_ptr, uint32_t view, const int* __restrict__ count_in,
                            const int* __restrict__ node_in, const int* __restrict__ draw_in,
                            const float* __restrict__ logq_in, const float* __restrict__ logits,
                            const float* __restrict__ root_mass, int* __restrict__ count_out,
                            int* __restrict__ node_out, int* __restrict__ draw_out, float* __restrict__ logq_out,
                            int* __restrict__ indices, float* __restrict__ weights) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= *count_in) return;
    if (seed_ptr) seed = *seed_ptr;
    T.n = vs->n;
    T.sq = vs->sq;
    T.isq = vs->isq;
    int draw = draw_in[r];
    int pixel = draw / K, k = draw % K;
    int v = node_in[r];
    int4 L = T.lnk[v];
    float z0 = logits[2 * r], z1 = logits[2 * r + 1];
    float m = fmaxf(z0, z1);
    float e0 = __expf(z0 - m), e1 = __expf(z1 - m);
    float q0 = e0 / (e0 + e1);
    float u = draw_uniform(seed, (uint32_t)pixel, view, 0xC0000000u, k, level);
    bool left = u <= q0;
    float qc = left ? q0 : 1.0f - q0;
    float logq = logq_in[r] + __logf(fmaxf(qc, 1e-30f));
    int c = left ? L.x : L.y;
    if (c >= T.n - 1) {
        float qx = (float)(pixel / H), qy = (float)(pixel % H);
        float g = leaf_mass(T, T.cen[c], qx, qy);
        indices[draw] = T.leaf_id[c - (T.n - 1)];
        weights[draw] = g / root_mass[pixel] * __expf(-logq);
    } else if (level + 1 < kTrace) {
        int o = atomicAdd(count_out, 1);
        node_out[o] = c;
        draw_out[o] = draw;
        logq_out[o] = logq;
    }
}

// Effective sample size of each pixel's K weighted draws; pixels below
// tau * K are marked for the plain sampler.
__global__ void k_prop_ess(int W, int H, int K, float tau, const float* __restrict__ root_mass, float precision,
                           const float* __restrict__ weights, unsigned char* __restrict__ mask,
                           int* __restrict__ nfallback) {
    size_t pixel = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (pixel >= (size_t)W * H) return;
    unsigned char fb = 0;
    if (root_mass[pixel] >= precision) {
        float s1 = 0.0f, s2 = 0.0f;
        for (int k = 0; k < K; ++k) {
            float w = weights[(size_t)K * pixel + k];
            s1 += w;
            s2 += w * w;
        }
        fb = !(s2 > 0.0f && s1 * s1 >= tau * (float)K * s2);  // also when no draw finished
    }
    mask[pixel] = fb;
    if (fb) atomicAdd(nfallback, 1);
}

__global__ void k_prop_clear(size_t P, int K, const unsigned char* __restrict__ mask, int* __restrict__ indices,
                             float* __restrict__ weights) {
    size_t pixel = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (pixel >= P || !mask[pixel]) return;
    for (int k = 0; k < K; ++k) {
        indices[(size_t)K * pixel + k] = -1;
        weights[(size_t)K * pixel + k] = 0.0f;
    }
}

__global__ void k_finish_view(const ViewState* vs, uds_view_stats* st) {
    st->n_visible = vs->n;
    st->n_coefs = (int)vs->coef_used;
}

// Evaluate getWeight for (node, query) pairs (debug entry point).
__global__ void k_fgt_eval(Tree T, const ViewState* vs, int m, const int* __restrict__ nodes,
                           const float* __restrict__ q, float* __restrict__ out) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m) return;
    T.n = vs->n;
    T.sq = vs->sq;
    T.isq = vs->isq;
    out[t] = node_weight(T, nodes[t], q[2 * t], q[2 * t + 1]);
}

// ------------------------------------------------------------ host side
static int build_view(const uds_sample_params* p, const Ws& w, int view, const float* pts,
                      const float* nrm, const float* sd, const float* h_override, cudaStream_t s) {
    int N = p->N;
    float W = (float)p->W, H = (float)p->H, f = p->focal;
    const float* vp = pts + 3 * (size_t)N * view;
    const float* vn = nrm + 3 * (size_t)N * view;
    const float* vsd = sd + (p->std_batch > 1 ? 2 * (size_t)N * view : 0);
    cudaError_t e = cudaMemsetAsync(w.vs, 0, sizeof(ViewState), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(w.fanin, 0, 4 * (size_t)(N > 0 ? N : 1), s);
    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    int st;
    unsigned nbN = cdiv(N > 0 ? N : 1, 128);
    if (N > 0) {
        k_bandwidth<<<nbN, 128, 0, s>>>(N, W, H, f, vp, vn, vsd, p->smoothing, w.vs);
        if ((st = launch_status())) return st;
    }
    k_view_setup<<<1, 1, 0, s>>>(h_override, view, W, H, p->precision, w.vs, w.stats);
    if ((st = launch_status())) return st;
    if (N == 0) return UDS_OK;
    k_cull_morton<<<nbN, 128, 0, s>>>(N, W, H, f, vp, w.vs, w.keysA, w.idsA);
    if ((st = launch_status())) return st;
    unsigned nb = cdiv(N, kSortTile);
    uint32_t *ki = w.keysA, *vi = w.idsA, *ko = w.keysB, *vo = w.idsB;
    for (int pass = 0; pass < 4; ++pass) {
        int shift = 8 * pass;
        k_radix_hist<<<nb, kSortThreads, 0, s>>>(N, nullptr, ki, shift, w.hist);
        int nh = (int)(256 * nb);
        int launched = 3;
        if (nh <= 16 * 1024) {
            k_radix_scan<<<1, 1024, 0, s>>>(w.hist, nh);
        } else {  // many tiles: the three-phase multi-block scan
            unsigned hb = cdiv(nh, kScanTile);
            k_scan_reduce<<<hb, kScanThreads, 0, s>>>(w.hist, nullptr, 0, nh, w.scanTmp);
            k_scan_top<<<1, 1024, 0, s>>>(w.scanTmp, (int)hb);
            k_scan_down<<<hb, kScanThreads, 0, s>>>(w.hist, nullptr, 0, nh, w.scanTmp, w.hist);
            launched = 5;
        }
        k_radix_scatter<<<nb, kSortThreads, 0, s>>>(N, nullptr, ki, vi, ko, vo, shift, w.hist);
        if ((st = launch_status(launched))) return st;
        uint32_t* t = ki; ki = ko; ko = t;
        t = vi; vi = vo; vo = t;
    }
    // after an even number of passes the sorted data is back in A
    k_leaves<<<nbN, 128, 0, s>>>(N, W, H, f, vp, w.vs, p->precision, vi, w.leaf_xy, w.leaf_id, w.lnk, w.par,
                                 w.box, w.cen);
    k_karras<<<nbN, 128, 0, s>>>(w.vs, ki, w.lnk, w.par);
    if (p->fixed_degree > 0) {
        int P = p->fixed_degree;
        k_bottomup<<<nbN, 128, 0, s>>>(w.vs, p->precision, P, w.lnk, w.par, w.box, w.cen, w.fanin);
        k_fixed_assign<<<nbN, 128, 0, s>>>(w.vs, w.cen, P);
        e = cudaMemsetAsync(w.fanin, 0, 4 * (size_t)N, s);
        if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
        switch (P) {
            case 4: k_m2m<4><<<nbN, 128, 0, s>>>(w.vs, w.lnk, w.par, w.cen, w.coef, w.fanin); break;
            case 6: k_m2m<6><<<nbN, 128, 0, s>>>(w.vs, w.lnk, w.par, w.cen, w.coef, w.fanin); break;
            default: k_m2m<8><<<nbN, 128, 0, s>>>(w.vs, w.lnk, w.par, w.cen, w.coef, w.fanin); break;
        }
        k_finish_view<<<1, 1, 0, s>>>(w.vs, w.stats + view);
        return launch_status(6);
    }
    k_bottomup<<<nbN, 128, 0, s>>>(w.vs, p->precision, p->max_degree, w.lnk, w.par, w.box, w.cen, w.fanin);
    k_node_sizes<<<nbN, 128, 0, s>>>(w.vs, w.cen, w.sizes);
    if ((st = launch_status(4))) return st;
    unsigned sb = cdiv(N, kScanTile);
    k_scan_reduce<<<sb, kScanThreads, 0, s>>>(w.sizes, w.vs, 1, 0, w.scanTmp);
    k_scan_top<<<1, 1024, 0, s>>>(w.scanTmp, (int)sb);
    k_scan_down<<<sb, kScanThreads, 0, s>>>(w.sizes, w.vs, 1, 0, w.scanTmp, w.offsets);
    k_assign<<<nbN, 128, 0, s>>>(w.vs, w.cen, w.sizes, w.offsets, w.coef_cap, w.stats + view);
    k_p2m<<<cdiv((size_t)N, 32 * kP2MWarps), 32 * kP2MWarps, 0, s>>>(w.vs, w.lnk, w.cen, w.leaf_xy, w.coef);
    k_finish_view<<<1, 1, 0, s>>>(w.vs, w.stats + view);
    return launch_status(6);
}

// Leaves one order-sampling round considers: the descent stops at the first
// node holding at most max(K, leaf_size) splats.
static int candidates(const uds_sample_params* p) { return p->leaf_size > p->K ? p->leaf_size : p->K; }

static Tree tree_of(const Ws& w) {
    Tree T;
    T.lnk = w.lnk; T.par = w.par; T.box = w.box; T.cen = w.cen; T.coef = w.coef;
    T.leaf_xy = w.leaf_xy; T.leaf_id = w.leaf_id; T.n = 0; T.sq = 0.0f; T.isq = 0.0f;
    return T;
}

template <int R>
// Descent for views view .. view + nviews - 1 in one launch (grid.z = view),
// their trees vstride bytes apart in the workspace.
// Block: 128 threads, tile_x (y) by 128 / tile_x (x) pixels; each warp is a
// tile_x by 32 / tile_x pixel tile.  Every lane's walk is its own, so the
// indices do not depend on the tile shape, only the speed does.
static void launch_sample(const Tree& T, const Ws& w, const uds_sample_params* p, const float* u, int view,
                          int* idx, cudaStream_t s, int nviews = 1, size_t vstride = 0) {
    int tx = p->tile_x > 0 ? p->tile_x : 8;
    dim3 block(tx, 128 / tx);
    dim3 grid(cdiv(p->H, block.x), cdiv(p->W, block.y), nviews);
    size_t istride = (size_t)p->W * p->H * p->K;
    const int M = candidates(p);
    size_t ustride = (size_t)p->W * p->H * R * M;
    UnevenViews none{};
    if (R <= 3 && p->K <= 8) {
        constexpr int RR = R <= 3 ? R : 3;
        if (p->spread)
            k_sample<RR, 8, false, true><<<grid, block, 0, s>>>(T, w.vs, p->W, p->H, p->K, M, p->precision, u, p->seed,
                                                                p->seed_dev, (uint32_t)view, idx, w.stats + view,
                                                                vstride, ustride, istride, none);
        else
            k_sample<RR, 8, false, false><<<grid, block, 0, s>>>(T, w.vs, p->W, p->H, p->K, M, p->precision, u,
                                                                 p->seed, p->seed_dev, (uint32_t)view, idx,
                                                                 w.stats + view, vstride, ustride, istride, none);
    } else {
        k_sample<(R >= 3 ? R : 3), kMaxK, false, false><<<grid, block, 0, s>>>(
            T, w.vs, p->W, p->H, p->K, M, p->precision, u, p->seed, p->seed_dev, (uint32_t)view, idx,
            w.stats + view, vstride, ustride, istride, none);
    }
}

// Views of different sizes (K <= 8) in one launch: a one-dimensional grid of
// every view's blocks; uv built by the caller.
template <int R>
static void launch_sample_uneven(const Tree& T, const Ws& w, const uds_sample_params* p, const UnevenViews& uv,
                                 int* idx, cudaStream_t s, size_t vstride) {
    int tx = p->tile_x > 0 ? p->tile_x : 8;
    dim3 block(tx, 128 / tx);
    if (p->spread)
        k_sample<R, 8, true, true><<<uv.first[uv.nv], block, 0, s>>>(T, w.vs, 0, 0, p->K, candidates(p), p->precision,
                                                                     nullptr, p->seed, p->seed_dev, 0u, idx, w.stats,
                                                                     vstride, 0, 0, uv);
    else
        k_sample<R, 8, true, false><<<uv.first[uv.nv], block, 0, s>>>(T, w.vs, 0, 0, p->K, candidates(p),
                                                                      p->precision, nullptr, p->seed, p->seed_dev,
                                                                      0u, idx, w.stats, vstride, 0, 0, uv);
}

static int check_params(const uds_sample_params* p) {
    if (!p) return UDS_ERR_ARGUMENT;
    if (p->B <= 0 || p->N < 0 || p->W <= 0 || p->H <= 0 || p->K <= 0 || p->K > kMaxK) return UDS_ERR_ARGUMENT;
    if (p->max_degree < 0 || p->max_degree > kMaxDegree) return UDS_ERR_ARGUMENT;
    if (p->std_batch != 1 && p->std_batch != p->B) return UDS_ERR_ARGUMENT;
    if (!(p->precision > 0.0f) || !(p->focal > 0.0f)) return UDS_ERR_ARGUMENT;
    if ((size_t)p->N * 2 >= (1u << 31)) return UDS_ERR_ARGUMENT;
    if (p->tile_x != 0 && p->tile_x != 4 && p->tile_x != 8 && p->tile_x != 16 && p->tile_x != 32)
        return UDS_ERR_ARGUMENT;
    if (p->leaf_size < 0 || p->leaf_size > kMaxLeaf) return UDS_ERR_ARGUMENT;
    if (p->spread != 0 && p->spread != 1) return UDS_ERR_ARGUMENT;
    if (p->fixed_degree != 0) {
        if (p->fixed_degree != 4 && p->fixed_degree != 6 && p->fixed_degree != 8) return UDS_ERR_ARGUMENT;
        int64_t need = (int64_t)(p->N > 1 ? p->N - 1 : 0) * (p->fixed_degree + 1) * (p->fixed_degree + 1);
        int64_t cap = p->coef_pool > 0 ? p->coef_pool : default_pool(p->N);
        if (need > cap) return UDS_ERR_ARGUMENT;  // one expansion per internal node must fit the pool
    }
    int64_t pool = p->coef_pool > 0 ? p->coef_pool : default_pool(p->N);
    if (pool >= (1ll << 26)) return UDS_ERR_ARGUMENT;  // offsets are packed in 26 bits
    return UDS_OK;
}

}  // namespace uds

using namespace uds;

namespace uds {
// Side streams for building several views' trees at once (their workspace
// slots are disjoint).  Created per device on first use outside stream
// capture; a call under capture before that builds the views in order.
constexpr int kBuildStreams = 4;
struct BuildStreams {
    bool ready = false;
    std::mutex enqueue;  // one call at a time forks, builds and joins
    cudaStream_t side[kBuildStreams];
    cudaEvent_t fork, join[kBuildStreams];
};

static BuildStreams* build_streams(cudaStream_t s) {
    static std::mutex mu;
    static BuildStreams pool[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lock(mu);
    BuildStreams& b = pool[dev];
    if (b.ready) return &b;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) return nullptr;
    bool ok = cudaEventCreateWithFlags(&b.fork, cudaEventDisableTiming) == cudaSuccess;
    for (int k = 0; k < kBuildStreams && ok; ++k)
        ok = cudaStreamCreateWithFlags(&b.side[k], cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&b.join[k], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        return nullptr;
    }
    b.ready = true;
    return &b;
}
}  // namespace uds

// uds_sample keeps every view's tree resident (one slot per view) so that one
// descent launch covers all views; the other entry points use slot 0.
extern "C" size_t uds_sample_workspace_size(const uds_sample_params* prm) {
    if (check_params(prm)) return 0;
    return layout(prm, nullptr).bytes * (size_t)prm->B;
}

extern "C" int uds_sample(const uds_sample_params* prm, const float* points, const float* normals,
                          const float* std_devs, const float* uniforms, const float* h_override,
                          int32_t* indices, uds_view_stats* stats, void* workspace, size_t workspace_bytes,
                          void* stream) {
    int st = check_params(prm);
    if (st) return st;
    if (!indices || (prm->N > 0 && (!points || !normals || !std_devs))) return UDS_ERR_ARGUMENT;
    char* base = reinterpret_cast<char*>(workspace);
    Ws w = layout(prm, base);
    size_t slot = w.bytes;
    if (!workspace || workspace_bytes < slot * (size_t)prm->B) return UDS_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    size_t per_view = (size_t)prm->W * prm->H * prm->K;
    cudaError_t e = cudaMemsetAsync(indices, 0xFF, sizeof(int32_t) * per_view * prm->B, s);
    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    // every view's tree in its own slot (the per-view record stays in slot 0);
    // several views at once on side streams forked from and joined to s
    BuildStreams* bs = prm->B > 1 ? build_streams(s) : nullptr;
    int nside = bs ? (prm->B < kBuildStreams ? prm->B : kBuildStreams) : 0;
    std::unique_lock<std::mutex> hold;
    if (nside) hold = std::unique_lock<std::mutex>(bs->enqueue);
    if (nside) {
        e = cudaEventRecord(bs->fork, s);
        for (int k = 0; k < nside && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(bs->side[k], bs->fork, 0);
        if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    }
    for (int b = 0; b < prm->B; ++b) {
        Ws wb = layout(prm, base + slot * (size_t)b);
        wb.stats = w.stats;
        cudaStream_t sb = nside ? bs->side[b % nside] : s;
        if ((st = build_view(prm, wb, b, points, normals, std_devs, h_override, sb))) return st;
    }
    if (nside) {
        for (int k = 0; k < nside && e == cudaSuccess; ++k) {
            e = cudaEventRecord(bs->join[k], bs->side[k]);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(s, bs->join[k], 0);
        }
        if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    }
    if (prm->N > 0) {
        // one descent launch over all views
        Tree T = tree_of(w);
        int B = prm->B;
        switch (num_rounds(prm->K)) {
            case 1: launch_sample<1>(T, w, prm, uniforms, 0, indices, s, B, slot); break;
            case 2: launch_sample<2>(T, w, prm, uniforms, 0, indices, s, B, slot); break;
            case 3: launch_sample<3>(T, w, prm, uniforms, 0, indices, s, B, slot); break;
            case 4: launch_sample<4>(T, w, prm, uniforms, 0, indices, s, B, slot); break;
            case 5: launch_sample<5>(T, w, prm, uniforms, 0, indices, s, B, slot); break;
            case 6: launch_sample<6>(T, w, prm, uniforms, 0, indices, s, B, slot); break;
            case 7: launch_sample<7>(T, w, prm, uniforms, 0, indices, s, B, slot); break;
            default: launch_sample<8>(T, w, prm, uniforms, 0, indices, s, B, slot); break;
        }
        if ((st = launch_status())) return st;
    }
    if (stats) {
        e = cudaMemcpyAsync(stats, w.stats, sizeof(uds_view_stats) * prm->B, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    }
    return UDS_OK;
}

// Views of different sizes in one call: every view's tree in its own slot,
// then one descent launch over all views' pixels (K <= 8; larger K, or more
// than kMaxUneven views, one launch per view).  prm->W, H and focal are
// replaced by each view's; indices are packed view after view.
extern "C" int uds_sample_views(const uds_sample_params* prm, const uds_view_desc* views, const float* points,
                                const float* normals, const float* std_devs, const float* h_override,
                                int32_t* indices, uds_view_stats* stats, void* workspace, size_t workspace_bytes,
                                void* stream) {
    int st = check_params(prm);
    if (st) return st;
    if (!views || !indices || (prm->N > 0 && (!points || !normals || !std_devs))) return UDS_ERR_ARGUMENT;
    size_t total = 0;
    for (int b = 0; b < prm->B; ++b) {
        if (views[b].W <= 0 || views[b].H <= 0 || !(views[b].focal > 0.0f)) return UDS_ERR_ARGUMENT;
        total += (size_t)views[b].W * views[b].H * prm->K;
    }
    char* base = reinterpret_cast<char*>(workspace);
    Ws w = layout(prm, base);
    size_t slot = w.bytes;  // does not depend on the image size
    if (!workspace || workspace_bytes < slot * (size_t)prm->B) return UDS_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    cudaError_t e = cudaMemsetAsync(indices, 0xFF, sizeof(int32_t) * total, s);
    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    BuildStreams* bs = prm->B > 1 ? build_streams(s) : nullptr;
    int nside = bs ? (prm->B < kBuildStreams ? prm->B : kBuildStreams) : 0;
    std::unique_lock<std::mutex> hold;
    if (nside) hold = std::unique_lock<std::mutex>(bs->enqueue);
    if (nside) {
        e = cudaEventRecord(bs->fork, s);
        for (int k = 0; k < nside && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(bs->side[k], bs->fork, 0);
        if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    }
    for (int b = 0; b < prm->B; ++b) {
        uds_sample_params pv = *prm;
        pv.W = views[b].W;
        pv.H = views[b].H;
        pv.focal = views[b].focal;
        Ws wb = layout(&pv, base + slot * (size_t)b);
        wb.stats = w.stats;
        cudaStream_t sb = nside ? bs->side[b % nside] : s;
        if ((st = build_view(&pv, wb, b, points, normals, std_devs, h_override, sb))) return st;
    }
    if (nside) {
        for (int k = 0; k < nside && e == cudaSuccess; ++k) {
            e = cudaEventRecord(bs->join[k], bs->side[k]);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(s, bs->join[k], 0);
        }
        if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    }
    if (prm->N > 0) {
        Tree T = tree_of(w);
        int R = num_rounds(prm->K);
        int tx = prm->tile_x > 0 ? prm->tile_x : 8;
        if (prm->K <= 8 && prm->B <= kMaxUneven) {
            UnevenViews uv{};
            uv.nv = prm->B;
            long long off = 0;
            int blocks = 0;
            for (int b = 0; b < prm->B; ++b) {
                uv.first[b] = blocks;
                uv.bx[b] = (int)cdiv(views[b].H, tx);
                uv.W[b] = views[b].W;
                uv.H[b] = views[b].H;
                uv.ioff[b] = off;
                blocks += uv.bx[b] * (int)cdiv(views[b].W, 128 / tx);
                off += (long long)views[b].W * views[b].H * prm->K;
            }
            uv.first[prm->B] = blocks;
            switch (R) {
                case 1: launch_sample_uneven<1>(T, w, prm, uv, indices, s, slot); break;
                case 2: launch_sample_uneven<2>(T, w, prm, uv, indices, s, slot); break;
                default: launch_sample_uneven<3>(T, w, prm, uv, indices, s, slot); break;
            }
            if ((st = launch_status())) return st;
        } else {
            size_t off = 0;
            for (int b = 0; b < prm->B; ++b) {
                uds_sample_params pv = *prm;
                pv.W = views[b].W;
                pv.H = views[b].H;
                Ws wb = layout(&pv, base + slot * (size_t)b);
                wb.stats = w.stats;
                Tree Tb = tree_of(wb);
                switch (R) {
                    case 1: launch_sample<1>(Tb, wb, &pv, nullptr, b, indices + off, s); break;
                    case 2: launch_sample<2>(Tb, wb, &pv, nullptr, b, indices + off, s); break;
                    case 3: launch_sample<3>(Tb, wb, &pv, nullptr, b, indices + off, s); break;
                    case 4: launch_sample<4>(Tb, wb, &pv, nullptr, b, indices + off, s); break;
                    case 5: launch_sample<5>(Tb, wb, &pv, nullptr, b, indices + off, s); break;
                    case 6: launch_sample<6>(Tb, wb, &pv, nullptr, b, indices + off, s); break;
                    case 7: launch_sample<7>(Tb, wb, &pv, nullptr, b, indices + off, s); break;
                    default: launch_sample<8>(Tb, wb, &pv, nullptr, b, indices + off, s); break;
                }
                if ((st = launch_status())) return st;
                off += (size_t)views[b].W * views[b].H * prm->K;
            }
        }
    }
    if (stats) {
        e = cudaMemcpyAsync(stats, w.stats, sizeof(uds_view_stats) * prm->B, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    }
    return UDS_OK;
}

extern "C" int uds_sample_stochastic(const uds_sample_params* prm, const float* points, const float* normals,
                                     const float* std_devs, const float* h_override, int32_t* indices,
                                     float* probs, uds_view_stats* stats, void* workspace, size_t workspace_bytes,
                                     void* stream) {
    int st = check_params(prm);
    if (st) return st;
    if (!indices || !probs || (prm->N > 0 && (!points || !normals || !std_devs))) return UDS_ERR_ARGUMENT;
    Ws w = layout(prm, reinterpret_cast<char*>(workspace));
    if (!workspace || workspace_bytes < w.bytes) return UDS_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    size_t per_view = (size_t)prm->W * prm->H * prm->K;
    cudaError_t e = cudaMemsetAsync(indices, 0xFF, sizeof(int32_t) * per_view * prm->B, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(probs, 0, sizeof(float) * per_view * prm->B, s);
    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    Tree T = tree_of(w);
    dim3 block(8, 16);
    dim3 grid(cdiv(prm->H, block.x), cdiv(prm->W, block.y));
    for (int b = 0; b < prm->B; ++b) {
        if ((st = build_view(prm, w, b, points, normals, std_devs, h_override, s))) return st;
        if (prm->N == 0) continue;
        k_stochastic<<<grid, block, 0, s>>>(T, w.vs, prm->W, prm->H, prm->K, prm->precision, prm->seed, prm->seed_dev, (uint32_t)b,
                                            indices + per_view * b, probs + per_view * b, w.stats + b, nullptr, nullptr);
        if ((st = launch_status())) return st;
    }
    if (stats) {
        e = cudaMemcpyAsync(stats, w.stats, sizeof(uds_view_stats) * prm->B, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    }
    return UDS_OK;
}

extern "C" int uds_tree_build(const uds_sample_params* prm, int view, const float* points,
                              const float* normals, const float* std_devs, const float* h_override,
                              uds_view_stats* stats, uint32_t* keys, int32_t* ids, int32_t* left,
                              int32_t* right, int32_t* parent, int32_t* count, int32_t* degree, float* centre,
                              float* box, void* workspace, size_t workspace_bytes, void* stream);

namespace uds {
// Copy the built tree into plain per-node arrays (debug).
__global__ void k_export(const ViewState* vs, const Ws w, uint32_t* keys, int* ids, int* left, int* right,
                         int* parent, int* count, int* degree, float* centre, float* box) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    int n = vs->n;
    int M = n > 0 ? 2 * n - 1 : 0;
    if (v < n) {
        if (keys) keys[v] = w.keysA[v];
        if (ids) ids[v] = w.leaf_id[v];
    }
    if (v < M) {
        int4 L = w.lnk[v];
        float4 c = w.cen[v], b = w.box[v];
        if (left) left[v] = L.x;
        if (right) right[v] = L.y;
        if (parent) parent[v] = w.par[v];
        if (count) count[v] = L.w;
        if (degree) degree[v] = meta_degree(c.w);
        if (centre) { centre[2 * v] = c.x; centre[2 * v + 1] = c.y; }
        if (box) { box[4 * v] = b.x; box[4 * v + 1] = b.y; box[4 * v + 2] = b.z; box[4 * v + 3] = b.w; }
    }
}
}  // namespace uds

extern "C" int uds_tree_build(const uds_sample_params* prm, int view, const float* points,
                              const float* normals, const float* std_devs, const float* h_override,
                              uds_view_stats* stats, uint32_t* keys, int32_t* ids, int32_t* left,
                              int32_t* right, int32_t* parent, int32_t* count, int32_t* degree, float* centre,
                              float* box, void* workspace, size_t workspace_bytes, void* stream) {
    int st = check_params(prm);
    if (st) return st;
    if (view < 0 || view >= prm->B) return UDS_ERR_ARGUMENT;
    Ws w = layout(prm, reinterpret_cast<char*>(workspace));
    if (!workspace || workspace_bytes < w.bytes) return UDS_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    if ((st = build_view(prm, w, view, points, normals, std_devs, h_override, s))) return st;
    if (prm->N > 0) {
        k_export<<<cdiv(2 * (size_t)prm->N, 128), 128, 0, s>>>(w.vs, w, keys, ids, left, right, parent, count,
                                                               degree, centre, box);
        if ((st = launch_status())) return st;
    }
    if (stats) {
        cudaError_t e = cudaMemcpyAsync(stats, w.stats + view, sizeof(uds_view_stats), cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    }
    return UDS_OK;
}

extern "C" int uds_sample_descent(const uds_sample_params* prm, int view, const float* uniforms,
                                  int32_t* indices, void* workspace, size_t workspace_bytes, void* stream) {
    int st = check_params(prm);
    if (st) return st;
    if (view < 0 || view >= prm->B || !indices) return UDS_ERR_ARGUMENT;
    Ws w = layout(prm, reinterpret_cast<char*>(workspace));
    if (!workspace || workspace_bytes < w.bytes) return UDS_ERR_WORKSPACE;
    if (prm->N == 0) return UDS_OK;
    cudaStream_t s = as_stream(stream);
    Tree T = tree_of(w);
    switch (num_rounds(prm->K)) {
        case 1: launch_sample<1>(T, w, prm, uniforms, view, indices, s); break;
        case 2: launch_sample<2>(T, w, prm, uniforms, view, indices, s); break;
        case 3: launch_sample<3>(T, w, prm, uniforms, view, indices, s); break;
        case 4: launch_sample<4>(T, w, prm, uniforms, view, indices, s); break;
        case 5: launch_sample<5>(T, w, prm, uniforms, view, indices, s); break;
        case 6: launch_sample<6>(T, w, prm, uniforms, view, indices, s); break;
        case 7: launch_sample<7>(T, w, prm, uniforms, view, indices, s); break;
        default: launch_sample<8>(T, w, prm, uniforms, view, indices, s); break;
    }
    return launch_status();
}

extern "C" int uds_fgt_eval(const uds_sample_params* prm, int m, const int32_t* nodes, const float* query_xy,
                            float* out, const void* workspace, size_t workspace_bytes, void* stream) {
    int st = check_params(prm);
    if (st) return st;
    Ws w = layout(prm, reinterpret_cast<char*>(const_cast<void*>(workspace)));
    if (!workspace || workspace_bytes < w.bytes) return UDS_ERR_WORKSPACE;
    if (m <= 0) return UDS_OK;
    k_fgt_eval<<<cdiv(m, 128), 128, 0, as_stream(stream)>>>(tree_of(w), w.vs, m, nodes, query_xy, out);
    return launch_status();
}

extern "C" int uds_mlp_forward_tiles(int R_max, const int* R_dev, const void* X_tiles, const float* params,
                                     float* logits, int* err, void* stream);

namespace uds {
// Proposal-mode buffers after the tree slot.
struct PropWs {
    float* root_mass;
    unsigned char* mask;
    int* node[2];
    int* draw[2];
    float* logq[2];
    float* X;
    float* logits;
    int* counts;  // [0], [1]: list lengths; [2]: fallback pixels; [3]: network error flag
    size_t bytes;
};

static PropWs prop_layout(const uds_sample_params* p, char* base) {
    PropWs q{};
    size_t P = (size_t)p->W * p->H, D = P * (size_t)p->K;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += a256(bytes); return base ? base + o : nullptr; };
    q.root_mass = (float*)take(4 * P);
    q.mask = (unsigned char*)take(P);
    for (int c = 0; c < 2; ++c) {
        q.node[c] = (int*)take(4 * D);
        q.draw[c] = (int*)take(4 * D);
        q.logq[c] = (float*)take(4 * D);
    }
    // feature tiles: 128 rows of 16 bf16 per 4096 bytes
    q.X = (float*)take(cdiv(D > 0 ? D : 1, 128) * (size_t)4096);
    q.logits = (float*)take(8 * D);
    q.counts = (int*)take(16);
    q.bytes = off;
    return q;
}
}  // namespace uds

extern "C" size_t uds_proposal_workspace_size(const uds_sample_params* prm) {
    if (check_params(prm)) return 0;
    return layout(prm, nullptr).bytes + prop_layout(prm, nullptr).bytes;
}

extern "C" int uds_sample_proposal(const uds_sample_params* prm, const float* points, const float* normals,
                                   const float* std_devs, const float* h_override, const float* mlp_params,
                                   float ess_tau, int32_t* indices, float* weights, uint8_t* fallback,
                                   int32_t* n_fallback, uds_view_stats* stats, void* workspace,
                                   size_t workspace_bytes, void* stream) {
    int st = check_params(prm);
    if (st) return st;
    if (!indices || !weights || (prm->N > 0 && (!points || !normals || !std_devs))) return UDS_ERR_ARGUMENT;
    if (prm->W * (size_t)prm->H * prm->K >= (1ull << 31)) return UDS_ERR_ARGUMENT;
    char* base = reinterpret_cast<char*>(workspace);
    Ws w = layout(prm, base);
    PropWs q = prop_layout(prm, base ? base + w.bytes : nullptr);
    if (!workspace || workspace_bytes < w.bytes + q.bytes) return UDS_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    size_t P = (size_t)prm->W * prm->H, per_view = P * prm->K;
    cudaError_t e = cudaMemsetAsync(indices, 0xFF, sizeof(int32_t) * per_view * prm->B, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(weights, 0, sizeof(float) * per_view * prm->B, s);
    if (e == cudaSuccess && n_fallback) e = cudaMemsetAsync(n_fallback, 0, sizeof(int32_t) * prm->B, s);
    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    Tree T = tree_of(w);
    dim3 block(16, 8);
    dim3 grid(cdiv(prm->H, block.x), cdiv(prm->W, block.y));
    for (int b = 0; b < prm->B; ++b) {
        if ((st = build_view(prm, w, b, points, normals, std_devs, h_override, s))) return st;
        if (prm->N == 0) continue;
        int* idx = indices + per_view * b;
        float* wt = weights + per_view * b;
        const unsigned char* mask = nullptr;
        if (mlp_params) {
            e = cudaMemsetAsync(q.counts, 0, 16, s);
            if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
            k_prop_init<<<dim3(cdiv(prm->H, 8), cdiv(prm->W, 16)), dim3(8, 16), 0, s>>>(T, w.vs, prm->W, prm->H, prm->K, prm->precision, q.root_mass,
                                               q.node[0], q.draw[0], q.logq[0], q.counts, idx, wt);
            if ((st = launch_status())) return st;
            unsigned nb = cdiv(per_view, 256);
            int cur = 0;
            for (int level = 0; level < kTrace; ++level) {
                if (level % 8 == 7) {  // stop once every draw has reached its leaf
                    int left = 0;
                    e = cudaMemcpyAsync(&left, q.counts + cur, sizeof(int), cudaMemcpyDeviceToHost, s);
                    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
                    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
                    if (left == 0) break;
                }
                k_prop_features<<<nb, 256, 0, s>>>(T, w.vs, prm->H, prm->K, level, q.counts + cur, q.node[cur],
                                                   q.draw[cur], reinterpret_cast<unsigned char*>(q.X));
                if ((st = launch_status())) return st;
                if ((st = uds_mlp_forward_tiles((int)per_view, q.counts + cur, q.X, mlp_params, q.logits,
                                                q.counts + 3, stream)))
                    return st;
                e = cudaMemsetAsync(q.counts + (cur ^ 1), 0, 4, s);
                if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
                k_prop_step<<<nb, 256, 0, s>>>(T, w.vs, prm->H, prm->K, level, prm->seed, prm->seed_dev, (uint32_t)b,
                                               q.counts + cur, q.node[cur], q.draw[cur], q.logq[cur], q.logits,
                                               q.root_mass, q.counts + (cur ^ 1), q.node[cur ^ 1], q.draw[cur ^ 1],
                                               q.logq[cur ^ 1], idx, wt);
                if ((st = launch_status())) return st;
                cur ^= 1;
            }
            k_prop_ess<<<cdiv(P, 256), 256, 0, s>>>(prm->W, prm->H, prm->K, ess_tau, q.root_mass, prm->precision, wt,
                                                     q.mask, n_fallback ? n_fallback + b : q.counts + 2);
            if ((st = launch_status())) return st;
            // fallback pixels: clear the proposal's draws, then the plain sampler
            k_prop_clear<<<cdiv(P, 256), 256, 0, s>>>(P, prm->K, q.mask, idx, wt);
            if ((st = launch_status())) return st;
            mask = q.mask;
            if (fallback) {
                e = cudaMemcpyAsync(fallback + P * b, q.mask, P, cudaMemcpyDeviceToDevice, s);
                if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
            }
        }
        // the plain stochastic sampler: every pixel, or the fallback pixels
        float* probs = q.logits;  // scratch for the path probabilities
        k_stochastic<<<grid, block, 0, s>>>(T, w.vs, prm->W, prm->H, prm->K, prm->precision, prm->seed,
                                            prm->seed_dev, (uint32_t)b, idx, probs, w.stats + b, mask, wt);
        if ((st = launch_status())) return st;
    }
    if (stats) {
        e = cudaMemcpyAsync(stats, w.stats, sizeof(uds_view_stats) * prm->B, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    }
    return UDS_OK;
}

extern "C" int uds_proposal_dataset(const uds_sample_params* prm, int stride, int draws, float* X, float* target,
                                    int64_t* keys, int32_t* count, int cap, const void* workspace,
                                    size_t workspace_bytes, void* stream) {
    int st = check_params(prm);
    if (st) return st;
    if (stride < 1 || draws < 1 || draws > 255 || cap < 0 || !count || (cap > 0 && (!X || !target)))
        return UDS_ERR_ARGUMENT;
    Ws w = layout(prm, reinterpret_cast<char*>(const_cast<void*>(workspace)));
    if (!workspace || workspace_bytes < w.bytes) return UDS_ERR_WORKSPACE;
    if (prm->N == 0) return UDS_OK;
    dim3 block(16, 8);
    dim3 grid(cdiv(cdiv(prm->H, stride), block.x), cdiv(cdiv(prm->W, stride), block.y));
    k_prop_dataset<<<grid, block, 0, as_stream(stream)>>>(tree_of(w), w.vs, prm->W, prm->H, stride, draws,
                                                          prm->precision, prm->seed, 0u, X, target,
                                                          reinterpret_cast<long long*>(keys), count, cap);
    return launch_status();
}
