// Status codes, error messages and device queries of the C ABI.
#include <stdarg.h>
#include <string.h>

#include "dfcsr_common.cuh"

namespace dfcsr {

static thread_local char g_msg[1024] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
}

void clear_error() { g_msg[0] = '\0'; }

int num_sms() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 148;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 148;
    return n;
}

}  // namespace dfcsr

extern "C" int dfcsr_version(void) { return 100; }

extern "C" const char *dfcsr_last_error(void) { return dfcsr::g_msg; }

extern "C" const char *dfcsr_status_name(int status) {
    switch (status) {
        case DFCSR_OK: return "OK";
        case DFCSR_BAD_ARG: return "BAD_ARG";
        case DFCSR_OOM: return "OOM";
        case DFCSR_TIMEOUT: return "TIMEOUT";
        case DFCSR_KERNEL_ERROR: return "KERNEL_ERROR";
        case DFCSR_CUDA_ERROR: return "CUDA_ERROR";
        case DFCSR_ADMISSION_REFUSED: return "ADMISSION_REFUSED";
        default: return "UNKNOWN";
    }
}

// Sizes of the ABI structs, so bindings can verify their layout.
extern "C" size_t dfcsr_abi_sizeof(int which) {
    switch (which) {
        case 0: return sizeof(dfcsr_df_params);
        case 1: return sizeof(dfcsr_wake_job);
        default: return 0;
    }
}
