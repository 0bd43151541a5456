// Status plumbing of the C ABI: status names, the last CUDA error of the
// calling host thread, library version.
#include "uds_common.cuh"

namespace uds {

static thread_local char g_last_error[256] = "no error";

void set_last_error(cudaError_t e) {
    const char* name = cudaGetErrorName(e);
    const char* text = cudaGetErrorString(e);
    int k = 0;
    for (const char* p = name; *p && k < 120; ++p) g_last_error[k++] = *p;
    g_last_error[k++] = ':';
    g_last_error[k++] = ' ';
    for (const char* p = text; *p && k < 254; ++p) g_last_error[k++] = *p;
    g_last_error[k] = 0;
}

unsigned long long g_launches = 0;  // kernels enqueued by this library

void set_last_error_message(const char* msg) {
    int k = 0;
    for (const char* p = msg; *p && k < 254; ++p) g_last_error[k++] = *p;
    g_last_error[k] = 0;
}

int launch_status(int launches) {
    __atomic_fetch_add(&g_launches, (unsigned long long)launches, __ATOMIC_RELAXED);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return UDS_OK;
    set_last_error(e);
    return UDS_ERR_LAUNCH;
}

}  // namespace uds

extern "C" const char* uds_status_string(int status) {
    switch (status) {
        case UDS_OK: return "ok";
        case UDS_ERR_ARGUMENT: return "invalid argument";
        case UDS_ERR_WORKSPACE: return "workspace too small";
        case UDS_ERR_LAUNCH: return "kernel launch failed";
        case UDS_ERR_CUDA: return "CUDA runtime error";
        default: return "unknown status";
    }
}

extern "C" const char* uds_last_error(void) { return uds::g_last_error; }

extern "C" int uds_version(void) { return 100; }

extern "C" unsigned long long uds_launch_count(void) { return __atomic_load_n(&uds::g_launches, __ATOMIC_RELAXED); }
