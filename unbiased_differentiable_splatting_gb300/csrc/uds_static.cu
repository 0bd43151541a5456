// EWA splatting forward that allocates nothing, for callers that cannot
// provide scratch memory.
//
// uds_splat_forward needs a caller-owned workspace for the per-splat Gaussian
// constants.  Some callers cannot hand one over: a plugin slot in a host
// application that only passes the op's input and output buffers, a binding
// from a language runtime that has no way to allocate device memory, or a
// real-time loop that must not touch any allocator after start-up.  This
// variant keeps that scratch in a fixed array in the library's own device
// memory instead, so the caller passes only inputs and outputs.
//
// Limits and rules of use:
//  - at most kStaticMaxSplats = 262144 (view, splat) pairs (B * N) per call;
//    larger calls are rejected with UDS_ERR_ARGUMENT and a message in
//    uds_last_error();
//  - the array occupies 8 MiB on every GPU that loads this library, until the
//    process exits;
//  - every call asks the runtime for the array's device address on the
//    current device (cudaGetSymbolAddress, a host-side query, with its return
//    code checked), so the address is never stale, also not after a device
//    reset; the first call on a device may load the library's device code,
//    so make that first call before any stream capture;
//  - every call uses the same array: calls that overlap on the GPU (different
//    streams, or different host threads without ordering) race on it.
//    Nothing in it needs to start at zero: each call writes the constants of
//    all its splats before reading any.
#include "uds_ewa.cuh"

namespace uds {

constexpr int kStaticMaxSplats = 1 << 18;

// Two float4 of Gaussian constants per (view, splat) pair.
static __device__ __align__(256) float4 g_splat_scratch[2 * kStaticMaxSplats];

void set_last_error_message(const char* msg);

__global__ void k_static_consts(int B, int N, float W, float H, float f, const float* __restrict__ pts,
                                const float* __restrict__ nrm, const float* __restrict__ sd, int sdB, float sm,
                                float4* __restrict__ consts) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int b = blockIdx.y;
    if (x >= N) return;
    size_t o = (size_t)x + (size_t)N * b;
    float p[3] = {pts[3 * o], pts[3 * o + 1], pts[3 * o + 2]};
    float n[3] = {nrm[3 * o], nrm[3 * o + 1], nrm[3 * o + 2]};
    size_t so = sdB > 1 ? o : (size_t)x;
    float s[2] = {sd[2 * so], sd[2 * so + 1]};
    EwaFrame F;
    ewa_frame(W, H, f, p, n, s, sm, F);
    float4 a, c;
    ewa_gauss_consts(F, a, c);
    consts[2 * o] = a;
    consts[2 * o + 1] = c;
}

__global__ void k_static_forward(int B, int W, int H, int K, const int* __restrict__ idx,
                                 const float4* __restrict__ consts, int N, float* __restrict__ w) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y;
    int b = blockIdx.z;
    if (j >= H) return;
    size_t pix = (size_t)j + (size_t)H * ((size_t)i + (size_t)W * b);
    float px = (float)i, py = (float)j;
    for (int s = 0; s < K; ++s) {
        size_t off = (size_t)s + (size_t)K * pix;
        int id = idx[off];
        float out = 0.0f;
        if (id >= 0 && id < N) {
            size_t o = (size_t)id + (size_t)N * b;
            out = fminf(ewa_gauss(consts[2 * o], consts[2 * o + 1], px, py), 1.0f);
        }
        w[off] = out;
    }
}

// Device address of the scratch array on the current device.  Host code
// cannot use the array's name as a device pointer (it names a host-side
// stand-in), so the address comes from the runtime, asked on every call with
// the caller's device current.
static int scratch_address(float4** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_splat_scratch);
    if (e != cudaSuccess) { set_last_error(e); return UDS_ERR_CUDA; }
    *out = reinterpret_cast<float4*>(p);
    return UDS_OK;
}

}  // namespace uds

using namespace uds;

extern "C" int uds_splat_forward_static(int B, int W, int H, int K, float focal, const int32_t* indices,
                                        const float* points, const float* normals, int std_batch, int N,
                                        const float* std_devs, float smoothing, float* weights, void* stream) {
    if (B <= 0 || W <= 0 || H <= 0 || K <= 0 || N < 0 || (std_batch != 1 && std_batch != B)) return UDS_ERR_ARGUMENT;
    if (!indices || !weights || (N > 0 && (!points || !normals || !std_devs))) return UDS_ERR_ARGUMENT;
    if ((long long)B * N > kStaticMaxSplats) {
        set_last_error_message("B*N exceeds the 262144 (view, splat) pairs of the static scratch; "
                               "use uds_splat_forward with a workspace");
        return UDS_ERR_ARGUMENT;
    }
    float4* consts = nullptr;
    int st = scratch_address(&consts);
    if (st) return st;
    cudaStream_t s = as_stream(stream);
    if (N > 0) {
        k_static_consts<<<dim3(cdiv(N, 128), B), 128, 0, s>>>(B, N, (float)W, (float)H, focal, points, normals,
                                                             std_devs, std_batch, smoothing, consts);
        if ((st = launch_status())) return st;
    }
    k_static_forward<<<dim3(cdiv(H, 64), W, B), 64, 0, s>>>(B, W, H, K, indices, consts, N, weights);
    return launch_status();
}
