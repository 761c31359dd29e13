// Status codes, error messages and device queries of the C ABI.
#include <stdarg.h>
#include <string.h>

#include <atomic>

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

static std::atomic<long long> g_launches{0};

void note_launch(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

// SM count of the current device; without one (argument checks on a host
// with no GPU) that of a GB300
int num_sms() {
    constexpr int kGb300Sms = 152;
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return kGb300Sms;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return kGb300Sms;
    return n;
}

}  // namespace dfcsr

extern "C" int dfcsr_version(void) { return 100; }

extern "C" long long dfcsr_kernel_launches(void) { return dfcsr::g_launches.load(); }

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

// --------------------------------------------------------- bounds checks
extern "C" int dfcsr_bounds_checked(void) { return DFCSR_BOUNDS_CHECK ? 1 : 0; }

extern "C" int dfcsr_bounds_status(unsigned long long *first_failure, int reset) {
    dfcsr::clear_error();
    DFCSR_CHECK_ARG(first_failure, "dfcsr_bounds_status: null pointer");
    *first_failure = 0;
#if DFCSR_BOUNDS_CHECK
    DFCSR_CUDA_TRY(cudaDeviceSynchronize());
    cudaError_t (*const readers[])(unsigned long long *, bool) = {
        dfcsr::bounds_read_beam_ops, dfcsr::bounds_read_deposit, dfcsr::bounds_read_dfstage,
        dfcsr::bounds_read_history,  dfcsr::bounds_read_interp,  dfcsr::bounds_read_probe,
        dfcsr::bounds_read_wake_fp64, dfcsr::bounds_read_wake_mixed};
    for (auto rd : readers) {
        unsigned long long v = 0;
        DFCSR_CUDA_TRY(rd(&v, reset != 0));
        if (*first_failure == 0) *first_failure = v;
    }
#else
    (void)reset;   // the release library has no status words
#endif
    return DFCSR_OK;
}

// --------------------------------------------------------------- timing
// Optional per-kernel timing: when enabled, entry points bracket their main
// kernels with CUDA events recorded on the launch stream.  Events are read
// (and the totals folded) only by dfcsr_timing_collect, after the timed
// region, so enabling this adds two event records per kernel and no sync.
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace dfcsr {

struct PendingTiming {
    std::string name;
    cudaEvent_t a, b;
};

static std::mutex g_tmu;
static bool g_timing = false;
static std::vector<PendingTiming> g_pending;
static std::map<std::string, std::pair<double, long long>> g_totals;

bool timing_on() { return g_timing; }

void timing_begin(const char *name, cudaStream_t s, void **token) {
    *token = nullptr;
    if (!g_timing) return;
    PendingTiming *p = new PendingTiming{name, nullptr, nullptr};
    if (cudaEventCreate(&p->a) != cudaSuccess || cudaEventCreate(&p->b) != cudaSuccess) {
        delete p;
        return;
    }
    cudaEventRecord(p->a, s);
    *token = p;
}

void timing_end(void *token, cudaStream_t s) {
    if (!token) return;
    PendingTiming *p = static_cast<PendingTiming *>(token);
    cudaEventRecord(p->b, s);
    std::lock_guard<std::mutex> g(g_tmu);
    g_pending.push_back(*p);
    delete p;
}

}  // namespace dfcsr

extern "C" void dfcsr_timing_enable(int on) { dfcsr::g_timing = on != 0; }

extern "C" int dfcsr_timing_collect(void) {
    using namespace dfcsr;
    std::lock_guard<std::mutex> g(g_tmu);
    for (auto &p : g_pending) {
        float ms = 0.f;
        if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            auto &t = g_totals[p.name];
            t.first += ms;
            t.second += 1;
        }
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    g_pending.clear();
    return DFCSR_OK;
}

extern "C" int dfcsr_timing_get(const char *name, double *total_ms, long long *launches) {
    using namespace dfcsr;
    std::lock_guard<std::mutex> g(g_tmu);
    auto it = g_totals.find(name ? name : "");
    *total_ms = (it == g_totals.end()) ? 0.0 : it->second.first;
    *launches = (it == g_totals.end()) ? 0 : it->second.second;
    return DFCSR_OK;
}

extern "C" void dfcsr_timing_reset(void) {
    using namespace dfcsr;
    std::lock_guard<std::mutex> g(g_tmu);
    for (auto &p : g_pending) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    g_pending.clear();
    g_totals.clear();
}
