// Proposal network kernels on the fifth-generation tensor cores (tcgen05,
// accumulators in TMEM): a single-tile GEMM that checks the operand layout
// and descriptors against the host, the network's forward pass (inference)
// and its gradient (training).
#include "uds_common.cuh"
#include "uds_tc.cuh"

#include <cuda_bf16.h>

namespace uds {

constexpr uint32_t kWaitLimit = 1u << 24;  // mbarrier polls before giving up

// C[128 x N] = A[128 x K] * B[N x K]^T, bf16 in, fp32 out; one CTA of 128
// threads.  `swap` exchanges the two descriptor distances (the test checks
// which reading is right).  err[0] is set if the MMA never completed.
__global__ void __launch_bounds__(128) k_mma_probe(int N, int K, const uint16_t* __restrict__ A,
                                                   const uint16_t* __restrict__ B, float* __restrict__ C, int swap,
                                                   int* __restrict__ err) {
    __shared__ __align__(1024) unsigned char sA[32768];
    __shared__ __align__(1024) unsigned char sB[32768];
    __shared__ uint64_t mbar;
    __shared__ uint32_t taddr_s;
    int tid = threadIdx.x, warp = tid >> 5;
    // zero the buffers so that any byte a wrong descriptor reads is defined
    for (int i = tid; i < 32768 / 16; i += 128) {
        reinterpret_cast<uint4*>(sA)[i] = make_uint4(0, 0, 0, 0);
        reinterpret_cast<uint4*>(sB)[i] = make_uint4(0, 0, 0, 0);
    }
    __syncthreads();
    for (int i = tid; i < 128 * K; i += 128) {
        int r = i / K, k = i % K;
        *reinterpret_cast<uint16_t*>(sA + tc::kmajor_offset(r, k, K)) = A[i];
    }
    for (int i = tid; i < N * K; i += 128) {
        int r = i / K, k = i % K;
        *reinterpret_cast<uint16_t*>(sB + tc::kmajor_offset(r, k, K)) = B[i];
    }
    if (tid == 0) tc::mbar_init(&mbar, 1);
    tc::fence_async_smem();
    __syncthreads();
    if (warp == 0) {
        tc::tmem_alloc(&taddr_s, 64);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    uint32_t taddr = taddr_s;
    if (tid == 0) {
        uint32_t kchunk = 128, rgroup = (uint32_t)(K / 8) * 128;
        uint32_t lbo = swap ? rgroup : kchunk, sbo = swap ? kchunk : rgroup;
        uint32_t idesc = tc::idesc_bf16(128, N);
        for (int ks = 0; ks < K / 16; ++ks) {
            uint64_t ad = tc::smem_desc(tc::smem_u32(sA) + ks * 256, lbo, sbo);
            uint64_t bd = tc::smem_desc(tc::smem_u32(sB) + ks * 256, lbo, sbo);
            tc::mma_bf16(taddr, ad, bd, idesc, ks > 0);
        }
        tc::mma_commit(&mbar);
    }
    bool ok = tc::mbar_wait(&mbar, 0, kWaitLimit);
    if (!ok && (tid & 31) == 0) atomicExch(err, 1);
    tc::fence_after_sync();
    if (ok) {
        int row = warp * 32 + (tid & 31);
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tc::tmem_ld16(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int c = 0; c < 16; ++c) C[(size_t)row * N + c0 + c] = v[c];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, 64);
}

}  // namespace uds

using namespace uds;

extern "C" int uds_mma_probe(int N, int K, const uint16_t* A, const uint16_t* B, float* C, int swap, int* err,
                             void* stream) {
    if (N < 16 || N > 64 || N % 16 || K < 16 || K > 128 || K % 16 || !A || !B || !C || !err)
        return UDS_ERR_ARGUMENT;
    k_mma_probe<<<1, 128, 0, as_stream(stream)>>>(N, K, A, B, C, swap, err);
    return launch_status();
}

// ===================================================================== MLP
// Proposal network: 16 input features -> 64 -> 64 -> 64 (ReLU) -> 2 branch
// logits (the last layer is computed 16 wide, rows 2..15 of its weight are
// zero).  Parameters are fp32 in one flat array (PARAM layout below); the
// kernels stage them in shared memory as bf16 and run every layer as one or
// a few tcgen05 MMAs (M = 128 rows of the batch, N = 64 or 16, K = 16 each)
// with fp32 accumulators in TMEM; bias and ReLU are applied in the epilogue
// (TMEM -> registers -> bf16 -> shared memory, the next layer's A operand).
namespace uds {
namespace mlp {
constexpr int kIn = 16, kHid = 64, kOut = 16, kLogits = 2;
// flat fp32 parameter layout
constexpr int oW1 = 0, oB1 = oW1 + kHid * kIn;
constexpr int oW2 = oB1 + kHid, oB2 = oW2 + kHid * kHid;
constexpr int oW3 = oB2 + kHid, oB3 = oW3 + kHid * kHid;
constexpr int oW4 = oB3 + kHid, oB4 = oW4 + kOut * kHid;
constexpr int kParams = oB4 + kOut;
constexpr int kTile = 128;
}  // namespace mlp

// Shared memory of the forward kernel (bf16 operands in the K-major core
// layout of uds_tc.cuh).
struct MlpFwdSmem {
    __align__(1024) unsigned char w1[mlp::kHid * mlp::kIn * 2];
    __align__(1024) unsigned char w2[mlp::kHid * mlp::kHid * 2];
    __align__(1024) unsigned char w3[mlp::kHid * mlp::kHid * 2];
    __align__(1024) unsigned char w4[mlp::kOut * mlp::kHid * 2];
    __align__(1024) unsigned char x[mlp::kTile * mlp::kIn * 2];
    __align__(1024) unsigned char h[mlp::kTile * mlp::kHid * 2];
    float bias[3 * mlp::kHid + mlp::kOut];
    uint64_t mbar;
    uint32_t taddr;
};

__device__ __forceinline__ void put_bf16(unsigned char* base, uint32_t off, float v) {
    *reinterpret_cast<__nv_bfloat16*>(base + off) = __float2bfloat16_rn(v);
}

// Row r, elements k0 .. k0+7 (k0 a multiple of 8) of a K-major operand are one
// 16-byte core-matrix row: store them with one vector store.
__device__ __forceinline__ void put8_bf16(unsigned char* base, int r, int k0, int K, const float* v) {
    __nv_bfloat162 h[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
    *reinterpret_cast<uint4*>(base + tc::kmajor_offset(r, k0, K)) = *reinterpret_cast<uint4*>(h);
}

// Stage an fp32 [R x K] row-major matrix as bf16 K-major operand.
__device__ __forceinline__ void stage_matrix(unsigned char* dst, const float* src, int R, int K) {
    for (int i = threadIdx.x; i < R * K; i += blockDim.x) put_bf16(dst, tc::kmajor_offset(i / K, i % K, K), src[i]);
}

// One layer: TMEM[0..N) = A (128 x K) * B (N x K)^T, issued by thread 0 and
// waited for by all; returns false if it did not complete in time.
__device__ __forceinline__ bool mlp_layer(uint32_t taddr, const unsigned char* a, const unsigned char* b, int K,
                                          int N, uint64_t* mbar, uint32_t& phase) {
    if (threadIdx.x == 0) {
        tc::fence_after_sync();
        uint32_t lbo = 128, sbo = (uint32_t)(K / 8) * 128;
        uint32_t idesc = tc::idesc_bf16(128, N);
        for (int ks = 0; ks < K / 16; ++ks)
            tc::mma_bf16(taddr, tc::smem_desc(tc::smem_u32(a) + ks * 256, lbo, sbo),
                         tc::smem_desc(tc::smem_u32(b) + ks * 256, lbo, sbo), idesc, ks > 0);
        tc::mma_commit(mbar);
    }
    bool ok = tc::mbar_wait(mbar, phase & 1u, kWaitLimit);
    ++phase;
    tc::fence_after_sync();
    return __syncthreads_and(ok) != 0;  // uniform over the block
}

// Inference: logits (R x 2, fp32) of feature rows X (R x 16, fp32).
// Persistent CTAs of 128 threads; thread t owns row t of each 128-row tile.
__global__ void __launch_bounds__(128) k_mlp_forward(int R, const int* __restrict__ Rdev, const float* __restrict__ X,
                                                     const float* __restrict__ P, float* __restrict__ out,
                                                     int* __restrict__ err) {
    if (Rdev) R = min(R, *Rdev);  // row count produced on the device
    if ((int)blockIdx.x * mlp::kTile >= R) return;  // no tile for this CTA
    extern __shared__ __align__(1024) unsigned char s_raw[];
    MlpFwdSmem& S = *reinterpret_cast<MlpFwdSmem*>(s_raw);
    using namespace mlp;
    int tid = threadIdx.x, warp = tid >> 5;
    stage_matrix(S.w1, P + oW1, kHid, kIn);
    stage_matrix(S.w2, P + oW2, kHid, kHid);
    stage_matrix(S.w3, P + oW3, kHid, kHid);
    stage_matrix(S.w4, P + oW4, kOut, kHid);
    for (int i = tid; i < kHid; i += 128) {
        S.bias[i] = P[oB1 + i];
        S.bias[kHid + i] = P[oB2 + i];
        S.bias[2 * kHid + i] = P[oB3 + i];
    }
    if (tid < kOut) S.bias[3 * kHid + tid] = P[oB4 + tid];
    if (tid == 0) tc::mbar_init(&S.mbar, 1);
    if (warp == 0) {
        tc::tmem_alloc(&S.taddr, 64);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    uint32_t taddr = S.taddr;
    uint32_t lane_base = taddr + ((uint32_t)(warp * 32) << 16);
    uint32_t phase = 0;
    bool ok = true;
    int tiles = (R + kTile - 1) / kTile;
    for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
        int row = t * kTile + tid;
        // features -> bf16 A operand (rows past R are zero)
        {
            float xv[kIn];
            const float4* xr = reinterpret_cast<const float4*>(X + (size_t)row * kIn);
#pragma unroll
            for (int q = 0; q < kIn / 4; ++q) {
                float4 f4 = row < R ? xr[q] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                xv[4 * q] = f4.x; xv[4 * q + 1] = f4.y; xv[4 * q + 2] = f4.z; xv[4 * q + 3] = f4.w;
            }
            put8_bf16(S.x, tid, 0, kIn, xv);
            put8_bf16(S.x, tid, 8, kIn, xv + 8);
        }
        tc::fence_async_smem();
        __syncthreads();
        const unsigned char* a = S.x;
        int K = kIn;
        const unsigned char* ws[3] = {S.w1, S.w2, S.w3};
        for (int l = 0; l < 3 && ok; ++l) {
            ok = mlp_layer(taddr, a, ws[l], K, kHid, &S.mbar, phase);
            if (!ok) break;
            // epilogue: bias + ReLU, bf16 into the hidden buffer (the MMA that
            // read it has completed)
            for (int c0 = 0; c0 < kHid; c0 += 16) {
                float v[16];
                tc::tmem_ld16(lane_base + (uint32_t)c0, v);
#pragma unroll
                for (int c = 0; c < 16; ++c) v[c] = fmaxf(v[c] + S.bias[l * kHid + c0 + c], 0.0f);
                put8_bf16(S.h, tid, c0, kHid, v);
                put8_bf16(S.h, tid, c0 + 8, kHid, v + 8);
            }
            tc::fence_before_sync();
            tc::fence_async_smem();
            __syncthreads();
            a = S.h;
            K = kHid;
        }
        if (!ok) break;
        ok = mlp_layer(taddr, S.h, S.w4, kHid, kOut, &S.mbar, phase);
        if (!ok) break;
        float v[16];
        tc::tmem_ld16(lane_base, v);
        if (row < R) {
            out[(size_t)row * kLogits] = v[0] + S.bias[3 * kHid];
            out[(size_t)row * kLogits + 1] = v[1] + S.bias[3 * kHid + 1];
        }
        tc::fence_before_sync();
        __syncthreads();
    }
    if (!ok && (tid & 31) == 0) atomicExch(err, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, 64);
}

// Inference on feature rows already in the tensor-core operand layout: row r
// is in 128-row tile r / 128, whose 4096 bytes (bf16, K-major core layout)
// start at Xt + 4096 * (r / 128).  Tiles stream into shared memory by bulk
// copies (the TMA engine) completing on per-buffer mbarriers, two buffers
// deep: tile i + 1 is in flight while tile i runs its four layers.
struct MlpTileSmem {
    __align__(1024) unsigned char w1[mlp::kHid * mlp::kIn * 2];
    __align__(1024) unsigned char w2[mlp::kHid * mlp::kHid * 2];
    __align__(1024) unsigned char w3[mlp::kHid * mlp::kHid * 2];
    __align__(1024) unsigned char w4[mlp::kOut * mlp::kHid * 2];
    __align__(1024) unsigned char x[2][mlp::kTile * mlp::kIn * 2];
    __align__(1024) unsigned char h[mlp::kTile * mlp::kHid * 2];
    float bias[3 * mlp::kHid + mlp::kOut];
    uint64_t mbar;      // MMA completion
    uint64_t xbar[2];   // tile arrivals
    uint32_t taddr;
};

constexpr uint32_t kTileBytes = mlp::kTile * mlp::kIn * 2;

__global__ void __launch_bounds__(128) k_mlp_forward_tiles(int R, const int* __restrict__ Rdev,
                                                           const unsigned char* __restrict__ Xt,
                                                           const float* __restrict__ P, float* __restrict__ out,
                                                           int* __restrict__ err) {
    if (Rdev) R = min(R, *Rdev);
    if ((int)blockIdx.x * mlp::kTile >= R) return;
    extern __shared__ __align__(1024) unsigned char s_raw[];
    MlpTileSmem& S = *reinterpret_cast<MlpTileSmem*>(s_raw);
    using namespace mlp;
    int tid = threadIdx.x, warp = tid >> 5;
    int tiles = (R + kTile - 1) / kTile;
    if (tid == 0) {
        tc::mbar_init(&S.mbar, 1);
        tc::mbar_init(&S.xbar[0], 1);
        tc::mbar_init(&S.xbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // first tile on its way while the weights are staged
        tc::mbar_expect_tx(&S.xbar[0], kTileBytes);
        tc::bulk_load(S.x[0], Xt + (size_t)blockIdx.x * kTileBytes, kTileBytes, &S.xbar[0]);
    }
    stage_matrix(S.w1, P + oW1, kHid, kIn);
    stage_matrix(S.w2, P + oW2, kHid, kHid);
    stage_matrix(S.w3, P + oW3, kHid, kHid);
    stage_matrix(S.w4, P + oW4, kOut, kHid);
    for (int i = tid; i < kHid; i += 128) {
        S.bias[i] = P[oB1 + i];
        S.bias[kHid + i] = P[oB2 + i];
        S.bias[2 * kHid + i] = P[oB3 + i];
    }
    if (tid < kOut) S.bias[3 * kHid + tid] = P[oB4 + tid];
    if (warp == 0) {
        tc::tmem_alloc(&S.taddr, 64);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    tc::fence_async_smem();
    __syncthreads();
    tc::fence_after_sync();
    uint32_t taddr = S.taddr;
    uint32_t lane_base = taddr + ((uint32_t)(warp * 32) << 16);
    uint32_t phase = 0, xphase[2] = {0u, 0u};
    bool pending[2] = {true, false};  // thread 0's view of the loads in flight
    bool ok = true;
    int it = 0;
    for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x, ++it) {
        int b = it & 1;
        int tn = t + gridDim.x;
        // the other buffer was read by the previous tile's first layer, which
        // has completed: refill it with the next tile
        if (tid == 0 && tn < tiles) {
            tc::mbar_expect_tx(&S.xbar[b ^ 1], kTileBytes);
            tc::bulk_load(S.x[b ^ 1], Xt + (size_t)tn * kTileBytes, kTileBytes, &S.xbar[b ^ 1]);
            pending[b ^ 1] = true;
        }
        bool got = tc::mbar_wait(&S.xbar[b], xphase[b] & 1u, kWaitLimit);
        ++xphase[b];
        pending[b] = false;
        ok = __syncthreads_and(got) != 0;
        if (!ok) break;
        const unsigned char* a = S.x[b];
        int K = kIn;
        const unsigned char* ws[3] = {S.w1, S.w2, S.w3};
        for (int l = 0; l < 3 && ok; ++l) {
            ok = mlp_layer(taddr, a, ws[l], K, kHid, &S.mbar, phase);
            if (!ok) break;
            for (int c0 = 0; c0 < kHid; c0 += 16) {
                float v[16];
                tc::tmem_ld16(lane_base + (uint32_t)c0, v);
#pragma unroll
                for (int c = 0; c < 16; ++c) v[c] = fmaxf(v[c] + S.bias[l * kHid + c0 + c], 0.0f);
                put8_bf16(S.h, tid, c0, kHid, v);
                put8_bf16(S.h, tid, c0 + 8, kHid, v + 8);
            }
            tc::fence_before_sync();
            tc::fence_async_smem();
            __syncthreads();
            a = S.h;
            K = kHid;
        }
        if (!ok) break;
        ok = mlp_layer(taddr, S.h, S.w4, kHid, kOut, &S.mbar, phase);
        if (!ok) break;
        float v[16];
        tc::tmem_ld16(lane_base, v);
        int row = t * kTile + tid;
        if (row < R) {
            out[(size_t)row * kLogits] = v[0] + S.bias[3 * kHid];
            out[(size_t)row * kLogits + 1] = v[1] + S.bias[3 * kHid + 1];
        }
        tc::fence_before_sync();
        __syncthreads();
    }
    if (!ok && (tid & 31) == 0) atomicExch(err, 1);
    // a tile load still in flight (after an error) must land before exit
    if (tid == 0 && !ok) {
        for (int q = 0; q < 2; ++q)
            if (pending[q]) tc::mbar_wait(&S.xbar[q], xphase[q] & 1u, kWaitLimit);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, 64);
}

// ------------------------------------------------------------ training
// Gradient of the mean cross-entropy between the branch distribution
// softmax(logits) and the target (p, 1 - p) over R rows, added to G (fp32,
// kParams entries; the caller zeroes it) and the loss added to loss[0].
// Per 128-row tile: the forward pass keeps the three hidden activations in
// shared memory; the backward pass runs dH = dZ * W (B operand: W
// transposed, staged once) and the weight gradients dW += dZ^T H (operands
// written transposed, K = the tile's rows) on the tensor cores, the weight
// gradients accumulating in TMEM across the CTA's tiles, and the bias
// gradients on the CUDA cores in shared memory; each CTA writes its partial
// sums once at the end.
struct MlpGradSmem {
    __align__(1024) unsigned char w1[mlp::kHid * mlp::kIn * 2];
    __align__(1024) unsigned char w2[mlp::kHid * mlp::kHid * 2];
    __align__(1024) unsigned char w3[mlp::kHid * mlp::kHid * 2];
    __align__(1024) unsigned char w4[mlp::kOut * mlp::kHid * 2];
    __align__(1024) unsigned char w2t[mlp::kHid * mlp::kHid * 2];
    __align__(1024) unsigned char w3t[mlp::kHid * mlp::kHid * 2];
    __align__(1024) unsigned char w4t[mlp::kHid * mlp::kOut * 2];
    __align__(1024) unsigned char x[mlp::kTile * mlp::kIn * 2];
    __align__(1024) unsigned char h[3][mlp::kTile * mlp::kHid * 2];
    __align__(1024) unsigned char dz[2][mlp::kTile * mlp::kHid * 2];
    __align__(1024) unsigned char dz4[mlp::kTile * mlp::kOut * 2];
    // weight-gradient operands: dZ^T padded to 128 rows (rows 64 .. 127 stay
    // zero) and H^T (or X^T), K = the tile's 128 rows
    __align__(1024) unsigned char at[mlp::kTile * mlp::kTile * 2];
    __align__(1024) unsigned char bt[mlp::kHid * mlp::kTile * 2];
    float dz4f[mlp::kTile][2];
    float bias[3 * mlp::kHid + mlp::kOut];
    float dbias[3 * mlp::kHid + mlp::kOut];
    float wloss[4];
    uint64_t mbar;
    uint32_t taddr;
};

__device__ __forceinline__ float get_bf16(const unsigned char* base, uint32_t off) {
    return __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(base + off));
}

// 8 consecutive K elements (k0 multiple of 8) of row r of a K-major operand.
__device__ __forceinline__ void get8(const unsigned char* base, int r, int k0, int K, float (&v)[8]) {
    uint4 q = *reinterpret_cast<const uint4*>(base + tc::kmajor_offset(r, k0, K));
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&q);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float2 f = __bfloat1622float2(h[i]);
        v[2 * i] = f.x;
        v[2 * i + 1] = f.y;
    }
}

// Stage W (R x K, fp32 row-major) transposed: operand of K rows x R columns.
__device__ __forceinline__ void stage_transposed(unsigned char* dst, const float* src, int R, int K) {
    for (int i = threadIdx.x; i < R * K; i += blockDim.x) {
        int r = i / K, k = i % K;
        put_bf16(dst, tc::kmajor_offset(k, r, R), src[i]);
    }
}

// Row r of a K-major [128 x K] bf16 tile becomes column r of the K-major
// [K x 128] tile dst (a transposed operand whose K is the tile's rows).
__device__ __forceinline__ void transpose_row(unsigned char* dst, const unsigned char* src, int r, int K) {
    for (int k0 = 0; k0 < K; k0 += 8) {
        uint4 q = *reinterpret_cast<const uint4*>(src + tc::kmajor_offset(r, k0, K));
        const unsigned short* e = reinterpret_cast<const unsigned short*>(&q);
#pragma unroll
        for (int i = 0; i < 8; ++i)
            *reinterpret_cast<unsigned short*>(dst + tc::kmajor_offset(k0 + i, r, mlp::kTile)) = e[i];
    }
}

// TMEM columns [col, col + N) (+)= at (128 x 128) * bt (N x 128)^T: a weight
// gradient dW = dZ^T H summed over the tile's rows on the tensor cores (rows
// 64 .. 127 of the accumulator stay zero).  Issued by one thread.
__device__ __forceinline__ void mma_wgrad(uint32_t taddr, uint32_t col, const unsigned char* at,
                                          const unsigned char* bt, int N, bool accumulate) {
    const uint32_t lbo = 128, sbo = (uint32_t)(mlp::kTile / 8) * 128;
    uint32_t idesc = tc::idesc_bf16(128, N);
    for (int ks = 0; ks < mlp::kTile / 16; ++ks)
        tc::mma_bf16(taddr + col, tc::smem_desc(tc::smem_u32(at) + ks * 256, lbo, sbo),
                     tc::smem_desc(tc::smem_u32(bt) + ks * 256, lbo, sbo), idesc, accumulate || ks > 0);
}

// TMEM columns of k_mlp_grad: activations / input gradients, then the
// accumulators of dW4 (2 x 64 used), dW3, dW2 (64 x 64) and dW1 (64 x 16)
constexpr uint32_t kColAct = 0, kColW4 = 64, kColW3 = 128, kColW2 = 192, kColW1 = 256, kGradCols = 512;

// Each block writes its partial gradients (and loss) to its own slice of
// part (kParams + 1 floats per block, every slot written by one thread);
// k_mlp_grad_reduce then sums the slices in block order, so the gradient does
// not depend on the order in which blocks finish.
constexpr int kGradPart = mlp::kParams + 1;

__global__ void __launch_bounds__(128) k_mlp_grad(int R, const float* __restrict__ X, const float* __restrict__ target,
                                                  float scale, const float* __restrict__ P,
                                                  float* __restrict__ part, int* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char s_raw[];
    MlpGradSmem& S = *reinterpret_cast<MlpGradSmem*>(s_raw);
    using namespace mlp;
    int tid = threadIdx.x, warp = tid >> 5;
    stage_matrix(S.w1, P + oW1, kHid, kIn);
    stage_matrix(S.w2, P + oW2, kHid, kHid);
    stage_matrix(S.w3, P + oW3, kHid, kHid);
    stage_matrix(S.w4, P + oW4, kOut, kHid);
    stage_transposed(S.w2t, P + oW2, kHid, kHid);
    stage_transposed(S.w3t, P + oW3, kHid, kHid);
    stage_transposed(S.w4t, P + oW4, kOut, kHid);
    for (int i = tid; i < 3 * kHid + kOut; i += 128) {
        S.bias[i] = P[oB1 + (i < kHid ? i : i < 2 * kHid ? (oB2 - oB1) + i - kHid
                                              : i < 3 * kHid ? (oB3 - oB1) + i - 2 * kHid : (oB4 - oB1) + i - 3 * kHid)];
        S.dbias[i] = 0.0f;
    }
    // dz4 columns 2..15 stay zero; so do rows 64 .. 127 of the transposed
    // dZ operand
    for (int i = tid; i < kTile * kOut * 2 / 16; i += 128) reinterpret_cast<uint4*>(S.dz4)[i] = make_uint4(0, 0, 0, 0);
    for (int i = tid; i < kTile * kTile * 2 / 16; i += 128) reinterpret_cast<uint4*>(S.at)[i] = make_uint4(0, 0, 0, 0);
    if (tid == 0) tc::mbar_init(&S.mbar, 1);
    if (warp == 0) {
        tc::tmem_alloc(&S.taddr, kGradCols);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    tc::fence_async_smem();
    __syncthreads();
    tc::fence_after_sync();
    uint32_t taddr = S.taddr;
    uint32_t lane_base = taddr + ((uint32_t)(warp * 32) << 16);
    uint32_t phase = 0;
    bool ok = true;
    bool first = true;  // the first tile starts the weight-gradient accumulators
    float lsum = 0.0f;
    int tiles = (R + kTile - 1) / kTile;
    for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
        int row = t * kTile + tid;
        bool valid = row < R;
        {
            float xv[kIn];
            const float4* xr = reinterpret_cast<const float4*>(X + (size_t)row * kIn);
#pragma unroll
            for (int q = 0; q < kIn / 4; ++q) {
                float4 f4 = valid ? xr[q] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                xv[4 * q] = f4.x; xv[4 * q + 1] = f4.y; xv[4 * q + 2] = f4.z; xv[4 * q + 3] = f4.w;
            }
            put8_bf16(S.x, tid, 0, kIn, xv);
            put8_bf16(S.x, tid, 8, kIn, xv + 8);
        }
        tc::fence_async_smem();
        __syncthreads();
        // ---- forward
        const unsigned char* a = S.x;
        int K = kIn;
        const unsigned char* ws[3] = {S.w1, S.w2, S.w3};
        for (int l = 0; l < 3 && ok; ++l) {
            ok = mlp_layer(taddr, a, ws[l], K, kHid, &S.mbar, phase);
            if (!ok) break;
            for (int c0 = 0; c0 < kHid; c0 += 16) {
                float v[16];
                tc::tmem_ld16(lane_base + (uint32_t)c0, v);
#pragma unroll
                for (int c = 0; c < 16; ++c) v[c] = fmaxf(v[c] + S.bias[l * kHid + c0 + c], 0.0f);
                put8_bf16(S.h[l], tid, c0, kHid, v);
                put8_bf16(S.h[l], tid, c0 + 8, kHid, v + 8);
            }
            tc::fence_before_sync();
            tc::fence_async_smem();
            __syncthreads();
            a = S.h[l];
            K = kHid;
        }
        if (!ok) break;
        ok = mlp_layer(taddr, S.h[2], S.w4, kHid, kOut, &S.mbar, phase);
        if (!ok) break;
        {
            float v[16];
            tc::tmem_ld16(lane_base, v);
            float z0 = v[0] + S.bias[3 * kHid], z1 = v[1] + S.bias[3 * kHid + 1];
            float m = fmaxf(z0, z1);
            float e0 = __expf(z0 - m), e1 = __expf(z1 - m);
            float q0 = e0 / (e0 + e1);
            float p = valid ? target[row] : 0.0f;
            float d0 = valid ? (q0 - p) * scale : 0.0f;
            if (valid) {
                float lz = m + __logf(e0 + e1);
                lsum += -(p * (z0 - lz) + (1.0f - p) * (z1 - lz));
            }
            S.dz4f[tid][0] = d0;
            S.dz4f[tid][1] = -d0;
            put_bf16(S.dz4, tc::kmajor_offset(tid, 0, kOut), d0);
            put_bf16(S.dz4, tc::kmajor_offset(tid, 1, kOut), -d0);
        }
        tc::fence_before_sync();
        __syncthreads();
        // ---- backward.  Each layer stages its weight-gradient operands (dZ^T
        // and the layer input transposed), then one thread issues the input-
        // gradient GEMM dH = dZ W and the weight-gradient GEMM dW += dZ^T H
        // on the tensor cores, while the CUDA cores sum the bias gradients.
        // layer 4: dZ4^T is 16 rows (2 nonzero); rows 16 .. 63 are cleared
        transpose_row(S.at, S.dz4, tid, kOut);
        for (int i = tid; i < 48 * kTile * 2 / 16; i += 128)
            reinterpret_cast<uint4*>(S.at + 16 * kTile * 2)[i] = make_uint4(0, 0, 0, 0);
        transpose_row(S.bt, S.h[2], tid, kHid);
        tc::fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            uint32_t idesc = tc::idesc_bf16(128, kHid);
            for (int ks = 0; ks < kOut / 16; ++ks)
                tc::mma_bf16(taddr + kColAct, tc::smem_desc(tc::smem_u32(S.dz4) + ks * 256, 128, (kOut / 8) * 128),
                             tc::smem_desc(tc::smem_u32(S.w4t) + ks * 256, 128, (kOut / 8) * 128), idesc, ks > 0);
            mma_wgrad(taddr, kColW4, S.at, S.bt, kHid, !first);
            tc::mma_commit(&S.mbar);
        }
        if (tid < 2) {
            float sb = 0.0f;
            for (int r = 0; r < kTile; ++r) sb += S.dz4f[r][tid];
            S.dbias[3 * kHid + tid] += sb;
        }
        ok = tc::mbar_wait(&S.mbar, phase & 1u, kWaitLimit);
        ++phase;
        tc::fence_after_sync();
        ok = __syncthreads_and(ok) != 0;
        if (!ok) break;
        // dZ3 = dH3 * relu'(Z3) -> dz[0]
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float v[16];
            tc::tmem_ld16(lane_base + kColAct + (uint32_t)c0, v);
#pragma unroll
            for (int c = 0; c < 16; ++c) {
                float hv = get_bf16(S.h[2], tc::kmajor_offset(tid, c0 + c, kHid));
                put_bf16(S.dz[0], tc::kmajor_offset(tid, c0 + c, kHid), hv > 0.0f ? v[c] : 0.0f);
            }
        }
        tc::fence_before_sync();
        tc::fence_async_smem();
        __syncthreads();
        // layers 3 and 2
        const unsigned char* wt[2] = {S.w3t, S.w2t};
        const uint32_t wcol[2] = {kColW3, kColW2};
        for (int l = 0; l < 2 && ok; ++l) {
            const unsigned char* dzl = S.dz[l];
            const unsigned char* hprev = S.h[1 - l];  // H2 for layer 3, H1 for layer 2
            transpose_row(S.at, dzl, tid, kHid);
            transpose_row(S.bt, hprev, tid, kHid);
            tc::fence_async_smem();
            __syncthreads();
            if (tid == 0) {
                tc::fence_after_sync();
                uint32_t idesc = tc::idesc_bf16(128, kHid);
                for (int ks = 0; ks < kHid / 16; ++ks)
                    tc::mma_bf16(taddr + kColAct, tc::smem_desc(tc::smem_u32(dzl) + ks * 256, 128, 8 * 128),
                                 tc::smem_desc(tc::smem_u32(wt[l]) + ks * 256, 128, 8 * 128), idesc, ks > 0);
                mma_wgrad(taddr, wcol[l], S.at, S.bt, kHid, !first);
                tc::mma_commit(&S.mbar);
            }
            if (tid < kHid) {
                float sb = 0.0f;
                for (int r = 0; r < kTile; ++r) sb += get_bf16(dzl, tc::kmajor_offset(r, tid, kHid));
                S.dbias[(2 - l) * kHid + tid] += sb;
            }
            ok = tc::mbar_wait(&S.mbar, phase & 1u, kWaitLimit);
            ++phase;
            tc::fence_after_sync();
            ok = __syncthreads_and(ok) != 0;
            if (!ok) break;
            // dZ_{l-1} = dH * relu'(Z_{l-1}) -> the other dz buffer
            unsigned char* dzn = S.dz[1 - l];
            for (int c0 = 0; c0 < kHid; c0 += 16) {
                float v[16];
                tc::tmem_ld16(lane_base + kColAct + (uint32_t)c0, v);
#pragma unroll
                for (int c = 0; c < 16; ++c) {
                    float hv = get_bf16(hprev, tc::kmajor_offset(tid, c0 + c, kHid));
                    put_bf16(dzn, tc::kmajor_offset(tid, c0 + c, kHid), hv > 0.0f ? v[c] : 0.0f);
                }
            }
            tc::fence_before_sync();
            tc::fence_async_smem();
            __syncthreads();
        }
        if (!ok) break;
        // layer 1: dW1 += dZ1^T X (dZ1 is in dz[0] after two swaps), db1
        {
            const unsigned char* dz1 = S.dz[0];
            transpose_row(S.at, dz1, tid, kHid);
            transpose_row(S.bt, S.x, tid, kIn);
            tc::fence_async_smem();
            __syncthreads();
            if (tid == 0) {
                tc::fence_after_sync();
                mma_wgrad(taddr, kColW1, S.at, S.bt, kIn, !first);
                tc::mma_commit(&S.mbar);
            }
            if (tid < kHid) {
                float sb = 0.0f;
                for (int r = 0; r < kTile; ++r) sb += get_bf16(dz1, tc::kmajor_offset(r, tid, kHid));
                S.dbias[tid] += sb;
            }
            ok = tc::mbar_wait(&S.mbar, phase & 1u, kWaitLimit);
            ++phase;
            tc::fence_after_sync();
            ok = __syncthreads_and(ok) != 0;
        }
        first = false;
    }
    if (!ok && (tid & 31) == 0) atomicExch(err, 1);
    // this block's partial sums: one writer per slot, no atomics.  Thread t
    // reads TMEM lane t: row t of each weight-gradient accumulator (rows
    // 64 .. 127 are the zero padding)
    float* G = part + (size_t)blockIdx.x * kGradPart;
    if (ok) {
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float v4[16], v3[16], v2[16];
            tc::tmem_ld16(lane_base + kColW4 + (uint32_t)c0, v4);
            tc::tmem_ld16(lane_base + kColW3 + (uint32_t)c0, v3);
            tc::tmem_ld16(lane_base + kColW2 + (uint32_t)c0, v2);
            if (tid < kHid) {
#pragma unroll
                for (int c = 0; c < 16; ++c) {
                    G[oW3 + tid * kHid + c0 + c] = v3[c];
                    G[oW2 + tid * kHid + c0 + c] = v2[c];
                    if (tid < kLogits) G[oW4 + tid * kHid + c0 + c] = v4[c];
                }
            }
        }
        float v1[16];
        tc::tmem_ld16(lane_base + kColW1, v1);
        if (tid < kHid) {
#pragma unroll
            for (int c = 0; c < 16; ++c) G[oW1 + tid * kIn + c] = v1[c];
        }
    }
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((tid & 31) == 0) S.wloss[warp] = lsum;
    tc::fence_before_sync();
    __syncthreads();
    for (int i = tid; i < kHid; i += 128) {
        G[oB1 + i] = S.dbias[i];
        G[oB2 + i] = S.dbias[kHid + i];
        G[oB3 + i] = S.dbias[2 * kHid + i];
    }
    if (tid < 2) G[oB4 + tid] = S.dbias[3 * kHid + tid];
    if (tid == 0) G[kParams] = (((S.wloss[0] + S.wloss[1]) + S.wloss[2]) + S.wloss[3]) * scale;
    if (warp == 0) tc::tmem_dealloc(taddr, kGradCols);
}

// grad += the blocks' partial gradients summed in block order; loss += the
// blocks' partial losses.  Slots of the zero rows of the last layer are not
// written by the blocks and are skipped.
__global__ void k_mlp_grad_reduce(int nb, const float* __restrict__ part, float* __restrict__ G,
                                  float* __restrict__ loss_out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > mlp::kParams) return;
    bool dead = i < mlp::kParams &&
                ((i >= mlp::oW4 + 2 * mlp::kHid && i < mlp::oB4) || i >= mlp::oB4 + 2);
    if (dead) return;
    float s = 0.0f;
    for (int b = 0; b < nb; ++b) s += part[(size_t)b * kGradPart + i];
    if (i < mlp::kParams) G[i] += s;
    else loss_out[0] += s;
}

// Adam step on the flat parameters; the gradient is consumed (zeroed).
// Rows 2..15 of W4 and entries 2..15 of b4 stay zero.
__global__ void k_mlp_adam(float* __restrict__ P, float* __restrict__ G, float* __restrict__ M1,
                           float* __restrict__ M2, float lr, float beta1, float beta2, float eps, float c1,
                           float c2) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= mlp::kParams) return;
    bool dead = (i >= mlp::oW4 + 2 * mlp::kHid && i < mlp::oB4) || i >= mlp::oB4 + 2;
    float g = G[i];
    G[i] = 0.0f;
    if (dead) return;
    float m = beta1 * M1[i] + (1.0f - beta1) * g;
    float v = beta2 * M2[i] + (1.0f - beta2) * g * g;
    M1[i] = m;
    M2[i] = v;
    P[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

}  // namespace uds

extern "C" int uds_mlp_param_count(void) { return uds::mlp::kParams; }

extern "C" int uds_mlp_forward(int R, const float* X, const float* params, float* logits, int* err, void* stream) {
    using namespace uds;
    if (R < 0 || (R > 0 && (!X || !params || !logits)) || !err) return UDS_ERR_ARGUMENT;
    if (R == 0) return UDS_OK;
    static bool attr = false;
    size_t smem = sizeof(MlpFwdSmem) + 1024;
    if (!attr) {
        cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    int tiles = (R + mlp::kTile - 1) / mlp::kTile;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int grid = tiles < 4 * sms ? tiles : 4 * sms;
    k_mlp_forward<<<grid, 128, smem, as_stream(stream)>>>(R, nullptr, X, params, logits, err);
    return launch_status();
}

// Same, with the row count read on the device from *R_dev (at most R_max).
extern "C" int uds_mlp_forward_dev(int R_max, const int* R_dev, const float* X, const float* params, float* logits,
                                   int* err, void* stream) {
    using namespace uds;
    if (R_max < 0 || !R_dev || (R_max > 0 && (!X || !params || !logits)) || !err) return UDS_ERR_ARGUMENT;
    if (R_max == 0) return UDS_OK;
    static bool attr = false;
    size_t smem = sizeof(MlpFwdSmem) + 1024;
    if (!attr) {
        cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    int tiles = (R_max + mlp::kTile - 1) / mlp::kTile;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int grid = tiles < 4 * sms ? tiles : 4 * sms;
    k_mlp_forward<<<grid, 128, smem, as_stream(stream)>>>(R_max, R_dev, X, params, logits, err);
    return launch_status();
}

static int mlp_grad_blocks(int R) {
    int tiles = (R + uds::mlp::kTile - 1) / uds::mlp::kTile;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return tiles < sms ? tiles : sms;
}

extern "C" size_t uds_mlp_grad_workspace_size(int R) {
    if (R <= 0) return 0;
    return sizeof(float) * (size_t)uds::kGradPart * (size_t)mlp_grad_blocks(R);
}

extern "C" int uds_mlp_grad(int R, const float* X, const float* target, const float* params, float* grad,
                            float* loss, int* err, void* workspace, size_t workspace_bytes, void* stream) {
    using namespace uds;
    if (R < 0 || (R > 0 && (!X || !target || !params || !grad || !loss)) || !err) return UDS_ERR_ARGUMENT;
    if (R == 0) return UDS_OK;
    if (!workspace || workspace_bytes < uds_mlp_grad_workspace_size(R)) return UDS_ERR_WORKSPACE;
    static bool attr = false;
    size_t smem = sizeof(MlpGradSmem) + 1024;
    if (!attr) {
        cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    int grid = mlp_grad_blocks(R);
    float* part = reinterpret_cast<float*>(workspace);
    cudaStream_t s = as_stream(stream);
    k_mlp_grad<<<grid, 128, smem, s>>>(R, X, target, 1.0f / (float)R, params, part, err);
    k_mlp_grad_reduce<<<cdiv(kGradPart, 256), 256, 0, s>>>(grid, part, grad, loss);
    return launch_status(2);
}

extern "C" int uds_mlp_adam(float* params, float* grad, float* m1, float* m2, int step, float lr, float beta1,
                            float beta2, float eps, void* stream) {
    using namespace uds;
    if (!params || !grad || !m1 || !m2 || step < 1) return UDS_ERR_ARGUMENT;
    float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    k_mlp_adam<<<cdiv(mlp::kParams, 256), 256, 0, as_stream(stream)>>>(params, grad, m1, m2, lr, beta1, beta2, eps,
                                                                      c1, c2);
    return launch_status();
}

// Feature rows given as bf16 tiles in the operand layout (uds_sample's
// proposal descent writes them so); the row count is read on the device.
extern "C" int uds_mlp_forward_tiles(int R_max, const int* R_dev, const void* X_tiles, const float* params,
                                     float* logits, int* err, void* stream) {
    using namespace uds;
    if (R_max < 0 || (R_max > 0 && (!X_tiles || !params || !logits)) || !err) return UDS_ERR_ARGUMENT;
    if ((reinterpret_cast<uintptr_t>(X_tiles) & 15) != 0) return UDS_ERR_ARGUMENT;
    if (R_max == 0) return UDS_OK;
    static bool attr = false;
    size_t smem = sizeof(MlpTileSmem) + 1024;
    if (!attr) {
        cudaFuncSetAttribute(k_mlp_forward_tiles, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    int tiles = (R_max + mlp::kTile - 1) / mlp::kTile;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int grid = tiles < 4 * sms ? tiles : 4 * sms;
    k_mlp_forward_tiles<<<grid, 128, smem, as_stream(stream)>>>(R_max, R_dev,
                                                               reinterpret_cast<const unsigned char*>(X_tiles),
                                                               params, logits, err);
    return launch_status();
}
