// Arithmetic-rate probe: the FP32 and FP64 fused multiply-add throughput of
// this GPU, measured by the benchmark next to its results (the roofline
// denominators for the FP32-bound and FP64-bound kernels of the wake path);
// and the probe of the bounds-checked build's index check.
#include "dfcsr_common.cuh"

namespace dfcsr {

constexpr int PROBE_THREADS = 256;
constexpr int PROBE_BLOCKS_PER_SM = 4;
constexpr int PROBE_CHAINS = 8;

// Eight independent FMA chains per thread (enough to cover the FMA latency at
// the probe's occupancy); the values stay bounded (a <- a * m + c with
// 0 < m < 1).  The final sum is stored only if it equals an impossible value,
// which keeps the chains live without writing memory.
template <typename T>
__global__ void __launch_bounds__(PROBE_THREADS)
fma_probe(int64_t iters, T m, T c, T *sink) {
    T a[PROBE_CHAINS];
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; ++k) a[k] = (T)(threadIdx.x + k);
    for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < PROBE_CHAINS; ++k) a[k] = fma(a[k], m, c);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; ++k) s += a[k];
    if (s == (T)-1.0) sink[0] = s;
}

}  // namespace dfcsr

using namespace dfcsr;

// One thread tests `index` against [0, size) with the bounds-checked
// build's check (no memory is accessed at that index).
__global__ void bounds_probe(long long index, long long size, unsigned site) {
    if (!dfcsr::bounds_ok(index, size, site)) return;
}

extern "C" int dfcsr_bounds_probe(long long index, long long size, int site, void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(site > 0 && site < 0x8000, "dfcsr_bounds_probe: site %d outside 1..32767", site);
    note_launch();
    bounds_probe<<<1, 1, 0, as_stream(stream)>>>(index, size, (unsigned)site);
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}

extern "C" int dfcsr_probe_fma(int fp64, int64_t iters, void *sink, double *flops, void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(iters > 0 && sink && flops, "dfcsr_probe_fma: bad argument");
    const int blocks = PROBE_BLOCKS_PER_SM * num_sms();
    *flops = 2.0 * PROBE_CHAINS * (double)iters * (double)blocks * PROBE_THREADS;
    cudaStream_t st = as_stream(stream);
    note_launch();
    if (fp64)
        fma_probe<double><<<blocks, PROBE_THREADS, 0, st>>>(iters, 0.999999, 1e-7,
                                                            reinterpret_cast<double *>(sink));
    else
        fma_probe<float><<<blocks, PROBE_THREADS, 0, st>>>(iters, 0.999999f, 1e-7f,
                                                           reinterpret_cast<float *>(sink));
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}

DFCSR_BOUNDS_READER(probe)
