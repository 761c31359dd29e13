// Shared helpers of the dfcsr_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/dfcsr_gb300.h"

namespace dfcsr {

// ---------------------------------------------------------------- errors
// Thread-local message of the last failing call (defined in capi.cu).
void set_error(const char *fmt, ...);
void clear_error();

#define DFCSR_CHECK_ARG(cond, ...)                  \
    do {                                            \
        if (!(cond)) {                              \
            ::dfcsr::set_error(__VA_ARGS__);        \
            return DFCSR_BAD_ARG;                   \
        }                                           \
    } while (0)

#define DFCSR_CUDA_TRY(expr)                                                     \
    do {                                                                         \
        cudaError_t e_ = (expr);                                                 \
        if (e_ != cudaSuccess) {                                                 \
            ::dfcsr::set_error("%s failed: %s", #expr, cudaGetErrorString(e_));  \
            return DFCSR_CUDA_ERROR;                                             \
        }                                                                        \
    } while (0)

#define DFCSR_LAUNCH_CHECK()                                                     \
    do {                                                                         \
        cudaError_t e_ = cudaGetLastError();                                     \
        if (e_ != cudaSuccess) {                                                 \
            ::dfcsr::set_error("kernel launch failed: %s", cudaGetErrorString(e_)); \
            return DFCSR_CUDA_ERROR;                                             \
        }                                                                        \
    } while (0)

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Carve typed sub-buffers out of a caller-provided workspace.
struct Carver {
    char *base;
    size_t size, used;
    template <class T>
    T *take(size_t count) {
        used = align_up(used, 256);
        T *p = reinterpret_cast<T *>(base + used);
        used += count * sizeof(T);
        return p;
    }
    bool ok() const { return used <= size; }
};

int num_sms();

// Host-side count of kernel launches issued by this library (defined in
// capi.cu; read through dfcsr_kernel_launches).
void note_launch(int k = 1);

// Kernel timing hooks (capi.cu): no-ops unless dfcsr_timing_enable(1).
bool timing_on();
void timing_begin(const char *name, cudaStream_t s, void **token);
void timing_end(void *token, cudaStream_t s);

struct ScopedTiming {
    void *tok;
    cudaStream_t s;
    ScopedTiming(const char *name, cudaStream_t st) : tok(nullptr), s(st) { timing_begin(name, st, &tok); }
    ~ScopedTiming() { timing_end(tok, s); }
};

// ------------------------------------------------- bounds-checked build
// Built with -DDFCSR_BOUNDS_CHECK=1 (libdfcsr_gb300_checked.so), the
// kernels test each computed global-memory index (history cells, records,
// sort positions, particle indices, table cells) against the extent of its
// buffer before the access.  A failing test records
//   bit 63 | site << 48 | (index & 0xffffffffffff)
// in the translation unit's status word (the first failure wins), and the
// access is skipped: nothing traps, the context stays usable, and
// dfcsr_bounds_status reports the site and index.  In the release library
// bounds_ok is the constant true and the tests compile away.
enum BoundsSite : unsigned {
    BS_PROBE = 1,             // dfcsr_bounds_probe
    BS_MIXED_RING = 10,       // mixed integral: history cell (slot, x, z)
    BS_MIXED_REC = 11,        // mixed integral: column / row records of a point
    BS_MIXED_ROWS = 12,       // mixed integral: valid row range of a region
    BS_MIXED_SETUP = 13,      // mixed set-up / band: history cells (FP64 gathers)
    BS_GEO_REC = 20,          // mixed geometry: record writes
    BS_FP64_RING = 30,        // FP64 wake and FP64 gathers: history cells
    BS_ORBIT = 31,            // orbit-table sample (interpolate1D of the lattice tables)
    BS_DEP_SCATTER = 40,      // deposit: radix scatter position
    BS_DEP_PARTICLE = 41,     // deposit: particle index of a sorted entry
    BS_DEP_CELL = 42,         // deposit: cell key
    BS_DEP_CHUNK = 43,        // deposit: chunk part slot
    BS_REGRID = 50,           // history regrid: source cell
    BS_KICK = 60,             // apply_wakes: kick table cell
    BS_DF = 70,               // DF stage: grid cell
    BS_INTERP = 80,           // interpolate3D / interpolate1D: table cell
};

#ifndef DFCSR_BOUNDS_CHECK
#define DFCSR_BOUNDS_CHECK 0
#endif

#if DFCSR_BOUNDS_CHECK
static __device__ unsigned long long g_bounds_fail;   // one per translation unit

static __device__ __noinline__ void bounds_record(long long i, unsigned site) {
    const unsigned long long code = (1ull << 63) | ((unsigned long long)(site & 0x7fffu) << 48) |
                                    ((unsigned long long)i & 0xffffffffffffull);
    atomicCAS(&g_bounds_fail, 0ull, code);
}

__device__ __forceinline__ bool bounds_ok(long long i, long long n, unsigned site) {
    if (i >= 0 && i < n) return true;
    bounds_record(i, site);
    return false;
}
#else
__device__ __forceinline__ constexpr bool bounds_ok(long long, long long, unsigned) { return true; }
#endif

// Host: this translation unit's status word (0: no failure), cleared when
// `reset`.  Each unit with kernels defines its reader with
// DFCSR_BOUNDS_READER(name); capi.cu's dfcsr_bounds_status reads them all.
#if DFCSR_BOUNDS_CHECK
#define DFCSR_BOUNDS_READER(name)                                                          \
    namespace dfcsr {                                                                      \
    cudaError_t bounds_read_##name(unsigned long long *v, bool reset) {                    \
        cudaError_t e = cudaMemcpyFromSymbol(v, g_bounds_fail, sizeof(*v));                \
        if (e == cudaSuccess && reset) {                                                   \
            const unsigned long long z = 0;                                                \
            e = cudaMemcpyToSymbol(g_bounds_fail, &z, sizeof(z));                          \
        }                                                                                  \
        return e;                                                                          \
    }                                                                                      \
    }
#else
#define DFCSR_BOUNDS_READER(name)                                                          \
    namespace dfcsr {                                                                      \
    cudaError_t bounds_read_##name(unsigned long long *v, bool) {                          \
        *v = 0;                                                                            \
        return cudaSuccess;                                                                \
    }                                                                                      \
    }
#endif
cudaError_t bounds_read_beam_ops(unsigned long long *v, bool reset);
cudaError_t bounds_read_deposit(unsigned long long *v, bool reset);
cudaError_t bounds_read_dfstage(unsigned long long *v, bool reset);
cudaError_t bounds_read_history(unsigned long long *v, bool reset);
cudaError_t bounds_read_interp(unsigned long long *v, bool reset);
cudaError_t bounds_read_probe(unsigned long long *v, bool reset);
cudaError_t bounds_read_wake_fp64(unsigned long long *v, bool reset);
cudaError_t bounds_read_wake_mixed(unsigned long long *v, bool reset);

// ------------------------------------------------------------ device math
// Reference axis rule of interpolate3D / interpolate1D: i0 = int(u)
// (truncation toward zero), i1 = i0 unless i0 is the last index, in range iff
// -1 < u < n.  Returns false when out of range.
__device__ __forceinline__ bool axis_index(double u, int n, int &i0, int &i1, double &frac) {
    if (!(u > -1.0 && u < (double)n)) return false;
    int a = (int)u;  // truncates toward zero
    i0 = a;
    i1 = (a == n - 1) ? a : a + 1;
    frac = __dsub_rn(u, (double)a);
    return true;
}

// numpy.linspace element i of linspace(start, stop, num): i*step + start,
// last element exactly stop, step == 0 handled like numpy.
__device__ __forceinline__ double np_linspace_at(double start, double stop, int num, int i) {
    if (num == 1) return start;
    if (i == num - 1) return stop;
    const int div = num - 1;
    const double delta = __dsub_rn(stop, start);
    const double step = __ddiv_rn(delta, (double)div);
    if (step == 0.0) return __dadd_rn(__dmul_rn(__ddiv_rn((double)i, (double)div), delta), start);
    return __dadd_rn(__dmul_rn((double)i, step), start);
}

// numpy pairwise summation (PW_BLOCKSIZE 128, 8 partial accumulators):
// blocks of at most 128 values summed with 8 accumulators ...
__device__ inline double np_pairwise_block(const double *a, int n) {
    if (n < 8) {
        double r = (n > 0) ? a[0] : 0.0;
        for (int i = 1; i < n; ++i) r = __dadd_rn(r, a[i]);
        return r;
    }
    double r[8];
    for (int k = 0; k < 8; ++k) r[k] = a[k];
    int i;
    for (i = 8; i < n - (n % 8); i += 8)
        for (int k = 0; k < 8; ++k) r[k] = __dadd_rn(r[k], a[i + k]);
    double res = __dadd_rn(__dadd_rn(__dadd_rn(r[0], r[1]), __dadd_rn(r[2], r[3])),
                           __dadd_rn(__dadd_rn(r[4], r[5]), __dadd_rn(r[6], r[7])));
    for (; i < n; ++i) res = __dadd_rn(res, a[i]);
    return res;
}

// ... and longer runs split in halves (the first a multiple of 8), summed
// left then right.  numpy recurses; this walks the same tree with an
// explicit stack, so the frame is static (a recursive device function's
// depth is not in the compiler's stack estimate).  A split at least halves
// the length, so 31 levels cover any int n.
__device__ inline double np_pairwise(const double *a, int n) {
    if (n <= 128) return np_pairwise_block(a, n);
    int off_s[32], len_s[32];
    double left_s[32];
    unsigned char st_s[32];
    int sp = 0;
    off_s[0] = 0; len_s[0] = n; st_s[0] = 0;
    double ret = 0.0;
    for (;;) {
        const int off = off_s[sp], len = len_s[sp];
        if (len <= 128) {
            ret = np_pairwise_block(a + off, len);
            --sp;   // the root is longer than 128, so sp >= 0 here
            continue;
        }
        int n2 = len / 2;
        n2 -= n2 % 8;
        if (st_s[sp] == 0) {            // left half
            st_s[sp] = 1;
            ++sp; off_s[sp] = off; len_s[sp] = n2; st_s[sp] = 0;
        } else if (st_s[sp] == 1) {     // right half
            left_s[sp] = ret;
            st_s[sp] = 2;
            ++sp; off_s[sp] = off + n2; len_s[sp] = len - n2; st_s[sp] = 0;
        } else {                        // both done
            ret = __dadd_rn(left_s[sp], ret);
            if (sp == 0) return ret;
            --sp;
        }
    }
}

// Deterministic block reduction of a double (fixed shuffle tree + fixed
// warp order).  `red` must hold blockDim.x / 32 doubles.  Result valid in
// thread 0.
__device__ inline double block_sum(double v, double *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        r = red[0];
        for (int w = 1; w < nw; ++w) r += red[w];
    }
    __syncthreads();
    return r;
}

}  // namespace dfcsr
