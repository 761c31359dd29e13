// Deposit without any device allocation: dfcsr_deposit_cic2d_noalloc.
//
// Some callers cannot allocate device memory at the point where they deposit:
// a host code that plans all of its device memory up front and forbids
// allocation inside its step loop, a plugin host that owns every allocation
// through its own pool and offers the library no allocator, or a real-time
// loop where a cudaMalloc (which may synchronise the device) is not allowed.
// For them the scratch of the sort-by-cell deposit lives in one file-scope
// __device__ array of fixed size, reserved when the library is loaded onto a
// GPU and held by every GPU that loads it until the process exits.
//
// Limits: at most kNoAllocMaxParticles particles and a grid whose
// (nb1 + 1) * (nb2 + 1) lower-cell keys fit kNoAllocMaxKeys (a 256 x 256 grid);
// larger requests are rejected with DFCSR_BAD_ARG.  All calls share the one
// array: calls whose work overlaps on the GPU (other streams, other host
// threads) race on it and must be serialised by the caller.  Each call clears
// what must start at zero (the cell ranges) before use; the rest of the array
// keeps the previous call's contents, which are never read.
#include <mutex>

#include "dfcsr_common.cuh"

namespace dfcsr {

constexpr long long kNoAllocMaxParticles = 1ll << 20;        // 1,048,576
constexpr long long kNoAllocMaxKeys = 257ll * 257ll;         // 256 x 256 grid
constexpr size_t kNoAllocScratchBytes = (size_t)24 << 20;    // 24 MiB

static __device__ __align__(256) unsigned char g_deposit_scratch[kNoAllocScratchBytes];

static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[128];   // device address of g_deposit_scratch per device

// Set-up, with the calling device current: the host-side name of a
// __device__ array is not a device address, so the address is resolved with
// cudaGetSymbolAddress.  It is resolved again on every call made outside a
// stream capture (after a cudaDeviceReset the module is loaded anew and an
// address kept from before would be stale); a call made while `stream` is
// being captured uses the address resolved by the device's last call outside
// a capture, so the first call on a device must come before any capture.
static int noalloc_scratch(cudaStream_t stream, void **out) {
    int dev = 0;
    DFCSR_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128) {
        set_error("dfcsr_deposit_cic2d_noalloc: device ordinal %d out of range", dev);
        return DFCSR_BAD_ARG;
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    DFCSR_CUDA_TRY(cudaStreamIsCapturing(stream, &cap));
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (cap != cudaStreamCaptureStatusNone) {
        if (!g_noalloc_ptr[dev]) {
            set_error("dfcsr_deposit_cic2d_noalloc: the first call on device %d must come before "
                      "any stream capture", dev);
            return DFCSR_BAD_ARG;
        }
    } else {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_deposit_scratch);
        if (e != cudaSuccess || !p) {
            set_error("dfcsr_deposit_cic2d_noalloc: cudaGetSymbolAddress failed: %s",
                      cudaGetErrorString(e));
            return DFCSR_CUDA_ERROR;
        }
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return DFCSR_OK;
}

}  // namespace dfcsr

using namespace dfcsr;

extern "C" size_t dfcsr_deposit_noalloc_max_bytes(void) { return kNoAllocScratchBytes; }

extern "C" int dfcsr_deposit_cic2d_noalloc(const double *q1, const double *q2, const double *w0,
                                           const double *w1, int64_t n, int nb1, double start1,
                                           double end1, int nb2, double start2, double end2,
                                           double *out0, double *out1, void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(n >= 0 && n <= kNoAllocMaxParticles,
                    "dfcsr_deposit_cic2d_noalloc: %lld particles exceed the no-alloc maximum of "
                    "%lld", (long long)n, kNoAllocMaxParticles);
    DFCSR_CHECK_ARG(nb1 > 0 && nb2 > 0 && ((long long)nb1 + 1) * ((long long)nb2 + 1) <= kNoAllocMaxKeys,
                    "dfcsr_deposit_cic2d_noalloc: grid %d x %d exceeds the no-alloc maximum "
                    "((nb1 + 1) * (nb2 + 1) <= %lld, i.e. 256 x 256)", nb1, nb2, kNoAllocMaxKeys);
    const size_t need = dfcsr_deposit_workspace_bytes(n, nb1, nb2);
    DFCSR_CHECK_ARG(need <= kNoAllocScratchBytes,
                    "dfcsr_deposit_cic2d_noalloc: needs %zu bytes of scratch, more than the "
                    "%zu reserved", need, kNoAllocScratchBytes);
    void *scratch = nullptr;
    const int st = noalloc_scratch(as_stream(stream), &scratch);
    if (st != DFCSR_OK) return st;
    return dfcsr_deposit_cic2d(q1, q2, w0, w1, n, nb1, start1, end1, nb2, start2, end2, out0, out1,
                               scratch, kNoAllocScratchBytes, stream);
}
