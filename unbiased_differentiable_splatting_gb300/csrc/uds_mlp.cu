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
__global__ void __launch_bounds__(128) k_mlp_forward(int R, const float* __restrict__ X,
                                                     const float* __restrict__ P, float* __restrict__ out,
                                                     int* __restrict__ err) {
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
#pragma unroll
        for (int k = 0; k < kIn; ++k)
            put_bf16(S.x, tc::kmajor_offset(tid, k, kIn), row < R ? X[(size_t)row * kIn + k] : 0.0f);
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
                for (int c = 0; c < 16; ++c)
                    put_bf16(S.h, tc::kmajor_offset(tid, c0 + c, kHid), fmaxf(v[c] + S.bias[l * kHid + c0 + c], 0.0f));
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
    k_mlp_forward<<<grid, 128, smem, as_stream(stream)>>>(R, X, params, logits, err);
    return launch_status();
}
