// Beam moments and the deterministic cloud-in-cell deposit.
//
// histogram_cic_2d (pyDFCSR_2D/deposit.py:43-87) scatters four corner weights
// per particle serially.  Here particles are sorted by their lower cell with
// a stable LSD radix sort (9-bit digits, per-warp match_any ranking, no
// float atomics), fixed-size chunks of the sorted particles are reduced per lower
// cell into four moments per weight channel (sum w, w f1, w f2, w f1 f2 of
// the fractional offsets), and a gather pass forms the four corner sums that
// land on each output cell.  Same result for the same input on every run; no
// floating-point atomics anywhere.  GB300 runs FP64 at about 1/72 of the
// FP32 rate (measured FMA rates), so the per-particle FP64 work is kept to
// 6 (keys) + 10 (sums) operations.
#include "dfcsr_common.cuh"

namespace dfcsr {

// ------------------------------------------------------------------ moments
// Two passes over (x, z), each a grid-stride loop with per-block partial sums
// and a one-block finish in a fixed order (deterministic).
//   pass 1: sums of dx, dz, dx^2, dz^2, dx dz with d = value - first value
//           (the shift keeps the variance free of cancellation for beams far
//           from the origin) -> means, sigma_x, sigma_z, cov, least-squares
//           slope and intercept of x on z (numpy.polyfit(z, x, 1));
//   pass 2: the |z| < 0.1 sigma_z slice (count, sum and square sum of
//           x - mean_x) and x_transform = x - (slope z + intercept) (sum and
//           square sum) -> sigma_x of the slice, mean and sigma of x_transform.
// FP64 operations per particle: 7 in pass 1, 8 in pass 2.
// 128-thread CTAs of 32 registers: one fits beside the wake's persistent
// integral CTAs (which leave 4096 registers per SM), so the next step's
// moments can run during the integral on the FP64 pipe it leaves idle.  At
// most one CTA per SM (152): four warps with five independent sums each keep
// the FP64 pipe busy, and more CTAs only take SM space that the integral's
// CTAs, launched later, then wait for (pipelined step 1.27 -> 1.25 ms).
constexpr int MOM_THREADS = 128;
constexpr int MOM_MAX_BLOCKS = 152;
constexpr int MOM_K = 5;   // partial sums per pass

static int moment_blocks(int64_t n) {
    int64_t b = (n + MOM_THREADS * 8 - 1) / (MOM_THREADS * 8);
    if (b < 1) b = 1;
    if (b > MOM_MAX_BLOCKS) b = MOM_MAX_BLOCKS;
    return (int)b;
}

// stats layout (see header): 0 n, 1 mean_x, 2 mean_z, 3 sigma_x, 4 sigma_z,
// 5 slope, 6 intercept, 7 n_slice, 8 sigma_x_slice, 9 mean_xt, 10 sigma_xt,
// 11 cov_xz, 12..15 reserved (zero)
template <int PASS>
__global__ void __launch_bounds__(MOM_THREADS)
moments_pass(const double *__restrict__ x, const double *__restrict__ z, int64_t n,
             const double *__restrict__ stats, double *__restrict__ partial) {
    __shared__ double red[MOM_THREADS / 32];
    double a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    double x0, z0, lim = 0, slope = 0, icpt = 0;
    if (PASS == 1) {
        x0 = x[0];
        z0 = z[0];
    } else {
        x0 = stats[1];
        z0 = 0.0;
        lim = __dmul_rn(0.1, stats[4]);
        slope = stats[5];
        icpt = stats[6];
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double xi = x[i], zi = z[i];
        if (PASS == 1) {
            const double dx = xi - x0, dz = zi - z0;
            a0 += dx;
            a1 += dz;
            a2 = fma(dx, dx, a2);
            a3 = fma(dz, dz, a3);
            a4 = fma(dx, dz, a4);
        } else {
            if (fabs(zi) < lim) {
                const double d = xi - x0;
                a0 += 1.0;
                a1 += d;
                a2 = fma(d, d, a2);
            }
            const double xt = xi - fma(slope, zi, icpt);
            a3 += xt;
            a4 = fma(xt, xt, a4);
        }
    }
    double v[MOM_K] = {a0, a1, a2, a3, a4};
    for (int k = 0; k < MOM_K; ++k) {
        const double s = block_sum(v[k], red);
        if (threadIdx.x == 0) partial[(size_t)blockIdx.x * MOM_K + k] = s;
    }
}

template <int PASS>
__global__ void __launch_bounds__(MOM_THREADS)
moments_finish(const double *__restrict__ x, const double *__restrict__ z,
               const double *__restrict__ partial, int nblk, int64_t n, double *__restrict__ stats) {
    __shared__ double red[MOM_THREADS / 32];
    double tot[MOM_K];
    for (int k = 0; k < MOM_K; ++k) {
        double a = 0;
        for (int b = threadIdx.x; b < nblk; b += blockDim.x) a += partial[(size_t)b * MOM_K + k];
        tot[k] = block_sum(a, red);
    }
    if (threadIdx.x != 0) return;
    const double dn = (double)n;
    if (PASS == 1) {
        const double mdx = tot[0] / dn, mdz = tot[1] / dn;
        const double vx = fmax(tot[2] / dn - mdx * mdx, 0.0);
        const double vz = fmax(tot[3] / dn - mdz * mdz, 0.0);
        const double cov = tot[4] / dn - mdx * mdz;
        stats[0] = dn;
        stats[1] = x[0] + mdx;
        stats[2] = z[0] + mdz;
        stats[3] = sqrt(vx);
        stats[4] = sqrt(vz);
        stats[11] = cov;
        const double slope = cov / vz;
        stats[5] = slope;
        stats[6] = stats[1] - slope * stats[2];
    } else {
        const double ms = tot[1] / tot[0];        // NaN when the slice is empty
        stats[7] = tot[0];
        stats[8] = sqrt(fmax(tot[2] / tot[0] - ms * ms, 0.0));
        const double mt = tot[3] / dn;
        stats[9] = mt;
        stats[10] = sqrt(fmax(tot[4] / dn - mt * mt, 0.0));
    }
}

// ----------------------------------------------------------------- CIC keys
// Lower-cell key of a particle: (i1 + 1) * (nb2 + 1) + (i2 + 1) for
// i1 in [-1, nb1 - 1], i2 in [-1, nb2 - 1]; particles with no corner inside
// the grid get the sentinel nkeys and sort to the end.
// The cell coordinate is the reference's (q - start) * inv_spacing; its
// floor is taken by one round-toward-minus-infinity conversion (saturating
// for huge or infinite values) and NaN coordinates are caught on the bit
// pattern, so the FP64 pipe does six operations per particle.
__device__ __forceinline__ bool is_nan_bits(double v) {
    return (__double_as_longlong(v) & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
}

// Grid of a deposit: first bin edge and inverse spacing per axis.  Passed by
// value, or (gp non-null) read from device memory, where a kernel of the
// same stream wrote it from the beam's moments.
struct DepGrid {
    double start1, inv1, start2, inv2;
};

__global__ void cic_keys(const double *__restrict__ q1, const double *__restrict__ q2, int64_t n,
                         int nb1, int nb2, DepGrid g, const DepGrid *__restrict__ gp,
                         uint32_t nkeys, uint32_t *__restrict__ keys, uint32_t *__restrict__ vals) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (gp) g = *gp;
    const double a = q1[i], b = q2[i];
    const int i1 = __double2int_rd(__dmul_rn(__dsub_rn(a, g.start1), g.inv1));
    const int i2 = __double2int_rd(__dmul_rn(__dsub_rn(b, g.start2), g.inv2));
    uint32_t key = nkeys;
    if (i1 >= -1 && i1 < nb1 && i2 >= -1 && i2 < nb2 && !is_nan_bits(a) && !is_nan_bits(b))
        key = (uint32_t)(i1 + 1) * (uint32_t)(nb2 + 1) + (uint32_t)(i2 + 1);
    keys[i] = key;
    vals[i] = (uint32_t)i;
}

// ------------------------------------------------------------- radix sort
constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_BITS = 9;                 // digit width: keys of grids up to 361^2 in 2 passes
constexpr int RS_BINS = 1 << RS_BITS;
constexpr uint32_t RS_MASK = RS_BINS - 1;

__global__ void __launch_bounds__(RS_THREADS)
radix_upsweep(const uint32_t *__restrict__ keys, int64_t n, int shift, int ntiles,
              uint32_t *__restrict__ hist) {
    __shared__ uint32_t cnt[RS_BINS];
    for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS) cnt[d] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ITEMS; ++r) {
        const int64_t idx = base + (int64_t)r * RS_THREADS + threadIdx.x;
        if (idx < n) atomicAdd(&cnt[(keys[idx] >> shift) & RS_MASK], 1u);   // integer: exact
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS)
        hist[(size_t)d * ntiles + blockIdx.x] = cnt[d];
}

// One block per digit: exclusive scan of hist[digit][0..ntiles) in place,
// row total to dtot[digit].
__global__ void __launch_bounds__(1024)
radix_scan_rows(uint32_t *__restrict__ hist, int ntiles, uint32_t *__restrict__ dtot) {
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t carry_s;
    uint32_t *row = hist + (size_t)blockIdx.x * ntiles;
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int off = 0; off < ntiles; off += blockDim.x) {
        const int i = off + threadIdx.x;
        const uint32_t v = (i < ntiles) ? row[i] : 0u;
        uint32_t inc = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) wsum[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = wsum[lane];
            uint32_t winc = w;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, winc, o);
                if (lane >= o) winc += t;
            }
            wsum[lane] = winc - w;   // exclusive warp offsets
        }
        __syncthreads();
        const uint32_t carry = carry_s;
        if (i < ntiles) row[i] = carry + wsum[warp] + inc - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry_s = carry + wsum[warp] + inc;
        __syncthreads();
    }
    if (threadIdx.x == 0) dtot[blockIdx.x] = carry_s;
}

// Stable scatter of one tile (RS_TILE keys): warp-level ranks of equal
// digits (__match_any_sync, in element order), then the tile is reordered by
// digit in shared memory and written out so that consecutive threads write
// consecutive positions of a digit's run (coalesced stores instead of one
// scattered 4-byte store per key).
struct ScatterSmem {
    union {
        uint32_t wcnt[RS_WARPS][RS_BINS];             // ranking phase
        struct { uint32_t key[RS_TILE], val[RS_TILE]; } t;   // reordered tile
    } u;
    uint32_t dbase[RS_BINS];   // global start of each digit
    uint32_t toff[RS_BINS];    // tile-local start of each digit
};

__global__ void __launch_bounds__(RS_THREADS)
radix_scatter(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals, int64_t n,
              int shift, int ntiles, const uint32_t *__restrict__ hist,
              const uint32_t *__restrict__ dtot, uint32_t *__restrict__ keys_out,
              uint32_t *__restrict__ vals_out) {
    extern __shared__ __align__(16) unsigned char rs_smem[];
    ScatterSmem &sm = *reinterpret_cast<ScatterSmem *>(rs_smem);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int d = threadIdx.x; d < RS_WARPS * RS_BINS; d += RS_THREADS) (&sm.u.wcnt[0][0])[d] = 0;
    if (warp == 0) {
        // exclusive scan of the digit totals (RS_BINS / 32 per lane)
        constexpr int PER = RS_BINS / 32;
        uint32_t loc[PER], s = 0;
        for (int k = 0; k < PER; ++k) { loc[k] = dtot[lane * PER + k]; s += loc[k]; }
        uint32_t inc = s;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        uint32_t run = inc - s;
        for (int k = 0; k < PER; ++k) { sm.dbase[lane * PER + k] = run + hist[(size_t)(lane * PER + k) * ntiles + blockIdx.x]; run += loc[k]; }
    }
    __syncthreads();
    const int64_t tile0 = (int64_t)blockIdx.x * RS_TILE;
    const int64_t base = tile0 + (int64_t)warp * (32 * RS_ITEMS);
    uint32_t k[RS_ITEMS], v[RS_ITEMS], rank[RS_ITEMS];
    int dig[RS_ITEMS];
    const unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r) {
        const int64_t idx = base + r * 32 + lane;
        const bool valid = idx < n;
        const uint32_t key = valid ? keys[idx] : 0u;
        const int d = valid ? (int)((key >> shift) & RS_MASK) : RS_BINS;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int leader = __ffs(peers) - 1;
        uint32_t before = 0;
        if (valid) before = sm.u.wcnt[warp][d];
        __syncwarp();
        if (valid && lane == leader) sm.u.wcnt[warp][d] = before + __popc(peers);
        __syncwarp();
        rank[r] = before + __popc(peers & lt_mask);
        dig[r] = d;
        k[r] = key;
        v[r] = valid ? vals[idx] : 0u;
    }
    __syncthreads();
    // per digit: exclusive prefix over the warps (in place) and the tile total
    for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS) {
        uint32_t run = 0;
        for (int w = 0; w < RS_WARPS; ++w) {
            const uint32_t t = sm.u.wcnt[w][d];
            sm.u.wcnt[w][d] = run;
            run += t;
        }
        sm.toff[d] = run;
    }
    __syncthreads();
    if (warp == 0) {   // tile-local digit starts: exclusive scan of the totals
        constexpr int PER = RS_BINS / 32;
        uint32_t loc[PER], s = 0;
        for (int q = 0; q < PER; ++q) { loc[q] = sm.toff[lane * PER + q]; s += loc[q]; }
        uint32_t inc = s;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        uint32_t run = inc - s;
        for (int q = 0; q < PER; ++q) { sm.toff[lane * PER + q] = run; run += loc[q]; }
    }
    __syncthreads();
    // rank -> tile-local position
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r)
        if (dig[r] < RS_BINS) rank[r] += sm.toff[dig[r]] + sm.u.wcnt[warp][dig[r]];
    __syncthreads();   // wcnt is overwritten by the reordered tile
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r) {
        if (dig[r] < RS_BINS) {
            sm.u.t.key[rank[r]] = k[r];
            sm.u.t.val[rank[r]] = v[r];
        }
    }
    __syncthreads();
    const int cnt = (int)((n - tile0) < RS_TILE ? (n - tile0) : RS_TILE);
    for (int i = threadIdx.x; i < cnt; i += RS_THREADS) {
        const uint32_t key = sm.u.t.key[i];
        const int d = (int)((key >> shift) & RS_MASK);
        const uint32_t pos = sm.dbase[d] + (uint32_t)i - sm.toff[d];
        if (!bounds_ok(pos, n, BS_DEP_SCATTER)) continue;
        keys_out[pos] = key;
        vals_out[pos] = sm.u.t.val[i];
    }
}

// ------------------------------------------------------------- cell sums
__global__ void cell_ranges(const uint32_t *__restrict__ keys, int64_t n, uint32_t nkeys,
                            uint32_t *__restrict__ cstart, uint32_t *__restrict__ cend) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = keys[i];
    if (!bounds_ok(k, (long long)nkeys + 1, BS_DEP_CELL)) return;   // nkeys: outside the grid
    if (i == 0 || keys[i - 1] != k) cstart[k] = (uint32_t)i;
    if (i == n - 1 || keys[i + 1] != k) cend[k] = (uint32_t)(i + 1);
}

// Eight partial sums per lower cell (corners 00, 01, 10, 11 for channel 0
// then channel 1), deterministic and load-balanced over the sorted particles.
//
// seg_sums: thread t takes the SEG_K sorted positions [t*K, t*K + K) (staged
// through shared memory) and sums each run of equal cell keys in order.  A
// run whose cell lies wholly inside the chunk is the cell's sum and is
// written to partial[cell]; a cell that crosses a chunk edge leaves its part
// of this chunk in chunk_first[t] (the run that starts the chunk) or
// chunk_last[t] (the run that ends it).
// seg_combine: one thread per cell adds the chunk parts of crossing cells in
// chunk order and writes zeros for empty cells.
// The order of every addition depends only on the sorted order, which the
// stable sort fixes: the result does not change from run to run.
constexpr int SEG_K = 16;
constexpr int SEG_THREADS = 256;
constexpr int SEG_TILE = SEG_K * SEG_THREADS;
// the chunk parts (8 doubles per SEG_K particles) live in the idle pair of
// 4-byte sort buffers after the sort: each buffer must hold a chunk's part
static_assert(SEG_K * 4 >= 8 * 8, "chunk parts do not fit the idle sort buffers");
// the staged keys and values of a tile must fit the static shared memory
static_assert(2 * (SEG_TILE + SEG_TILE / SEG_K) * 4 <= 48 * 1024, "seg_sums tile too large");

// Per-cell moments of the fractional offsets f = c - floor(c) for each
// weight channel: [sum w, sum w f1, sum w f2, sum w f1 f2].  The CIC corner
// weights (1 - f1)(1 - f2), (1 - f1) f2, f1 (1 - f2), f1 f2 are linear in
// these, so cic_assemble forms the corner sums from the moments.  Per
// particle: 2 FP64 operations for f1, f2, one for f1 f2, and 3 + 4 for the
// two channels (channel 0 without weights counts particles as an integer).
template <bool W0, bool W1>
__device__ __forceinline__ void cell_accumulate(uint32_t idx, double c1, double c2,
                                                const double *__restrict__ q1, const double *__restrict__ q2,
                                                const double *__restrict__ w0, const double *__restrict__ w1,
                                                double inv1, double inv2, double acc[8]) {
    // f = (q - start) inv - i as one FMA, q inv - (start inv + i), with the
    // run constant c = start inv + i: the offset within the lower cell to
    // ~1e-13 (it may step a hair outside [0, 1) at a cell edge, where the
    // corner weights are continuous)
    const double f1 = __fma_rn(q1[idx], inv1, -c1);
    const double f2 = __fma_rn(q2[idx], inv2, -c2);
    const double p = __dmul_rn(f1, f2);
    if (W0) {
        const double w = w0[idx];
        acc[0] = __dadd_rn(acc[0], w);
        acc[1] = __fma_rn(w, f1, acc[1]);
        acc[2] = __fma_rn(w, f2, acc[2]);
        acc[3] = __fma_rn(w, p, acc[3]);
    } else {
        acc[1] = __dadd_rn(acc[1], f1);
        acc[2] = __dadd_rn(acc[2], f2);
        acc[3] = __dadd_rn(acc[3], p);
    }
    if (W1) {
        const double w = w1[idx];
        acc[4] = __dadd_rn(acc[4], w);
        acc[5] = __fma_rn(w, f1, acc[5]);
        acc[6] = __fma_rn(w, f2, acc[6]);
        acc[7] = __fma_rn(w, p, acc[7]);
    }
}

__device__ __forceinline__ void store8(double *dst, const double acc[8]) {
    double2 *o = reinterpret_cast<double2 *>(dst);
    o[0] = make_double2(acc[0], acc[1]);
    o[1] = make_double2(acc[2], acc[3]);
    o[2] = make_double2(acc[4], acc[5]);
    o[3] = make_double2(acc[6], acc[7]);
}

// shared-memory slot of tile element i: one pad word per SEG_K so that the
// threads of a warp, each reading its own SEG_K-run, hit distinct banks
__device__ __forceinline__ int seg_slot(int i) { return i + i / SEG_K; }

template <bool W0, bool W1>
__global__ void __launch_bounds__(SEG_THREADS)
seg_sums(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals, int64_t n,
         uint32_t nkeys, int nb2, const uint32_t *__restrict__ cstart, const uint32_t *__restrict__ cend,
         const double *__restrict__ q1, const double *__restrict__ q2,
         const double *__restrict__ w0, const double *__restrict__ w1,
         DepGrid g, const DepGrid *__restrict__ gp,
         double *__restrict__ partial, double *__restrict__ chunk_first, double *__restrict__ chunk_last) {
    if (gp) g = *gp;
    const double inv1 = g.inv1, inv2 = g.inv2;
    __shared__ uint32_t sk[SEG_TILE + SEG_TILE / SEG_K];
    __shared__ uint32_t sv[SEG_TILE + SEG_TILE / SEG_K];
    const int64_t base = (int64_t)blockIdx.x * SEG_TILE;
    for (int i = threadIdx.x; i < SEG_TILE; i += SEG_THREADS) {
        const int64_t g = base + i;
        sk[seg_slot(i)] = g < n ? keys[g] : 0xffffffffu;
        sv[seg_slot(i)] = g < n ? vals[g] : 0u;
    }
    __syncthreads();
    const int64_t t = (int64_t)blockIdx.x * SEG_THREADS + threadIdx.x;
    const int64_t b = t * SEG_K;
    const int64_t e = (b + SEG_K < n) ? b + SEG_K : n;
    const int off = threadIdx.x * SEG_K;
    const int m = (int)(e > b ? e - b : 0);
    // Fixed trip count: every thread accumulates one particle per iteration,
    // so the FP64 work runs on full warps; only the flush at the end of a
    // run (integer work and stores) diverges.
    uint32_t k = m > 0 ? sk[seg_slot(off)] : nkeys;
    const double s1i = __dmul_rn(g.start1, inv1), s2i = __dmul_rn(g.start2, inv2);
    double fi1 = __dadd_rn(s1i, (double)((int)(k / (uint32_t)(nb2 + 1)) - 1));
    double fi2 = __dadd_rn(s2i, (double)((int)(k % (uint32_t)(nb2 + 1)) - 1));
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int j0 = 0;
#pragma unroll 1
    for (int j = 0; j < SEG_K; ++j) {
        const bool live = j < m && k < nkeys;      // outside-grid particles sort last
        if (live && bounds_ok(sv[seg_slot(off + j)], n, BS_DEP_PARTICLE))
            cell_accumulate<W0, W1>(sv[seg_slot(off + j)], fi1, fi2, q1, q2, w0, w1, inv1, inv2,
                                    acc);
        const uint32_t kn = (j + 1 < m) ? sk[seg_slot(off + j + 1)] : 0xffffffffu;
        if (live && kn != k) {                     // the run of key k ends at j
            if (!W0) acc[0] = (double)(j + 1 - j0);
            const int64_t cs = cstart[k], ce = cend[k];
            if (cs >= b && ce <= e) store8(partial + (size_t)k * 8, acc);
            else if (!bounds_ok(t, (n + SEG_K - 1) / SEG_K, BS_DEP_CHUNK)) {}
            else if (j0 == 0) store8(chunk_first + (size_t)t * 8, acc);
            else store8(chunk_last + (size_t)t * 8, acc);
#pragma unroll
            for (int c = 0; c < 8; ++c) acc[c] = 0.0;
            j0 = j + 1;
            k = kn;
            if (k < nkeys) {
                fi1 = __dadd_rn(s1i, (double)((int)(k / (uint32_t)(nb2 + 1)) - 1));
                fi2 = __dadd_rn(s2i, (double)((int)(k % (uint32_t)(nb2 + 1)) - 1));
            }
        }
    }
}

__global__ void seg_combine(const uint32_t *__restrict__ cstart, const uint32_t *__restrict__ cend,
                            uint32_t nkeys, int64_t nchunks, const double *__restrict__ chunk_first,
                            const double *__restrict__ chunk_last, double *__restrict__ partial) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nkeys) return;
    const uint32_t cs = cstart[k], ce = cend[k];
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (ce == 0) {                                  // empty cell
        store8(partial + (size_t)k * 8, acc);
        return;
    }
    const uint32_t t0 = cs / SEG_K, t1 = (ce - 1) / SEG_K;
    if (t0 == t1) return;                           // summed whole by seg_sums
    if (!bounds_ok(t1, nchunks, BS_DEP_CHUNK)) return;
    const double *first = (cs == t0 * SEG_K) ? chunk_first : chunk_last;
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[c] = first[(size_t)t0 * 8 + c];
    // the later chunks' parts in four interleaved partial sums (chunk t goes
    // to sum (t - t0 - 1) % 4), then ((acc + s0) + s1) + (s2 + s3): a dense
    // cell spans tens of chunks, and a running sum would be a chain of that
    // many dependent FP64 additions (some hundred cycles each on this GPU)
    double ps[4][8];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int c = 0; c < 8; ++c) ps[q][c] = 0.0;
    uint32_t t = t0 + 1;
    for (; t + 3 <= t1; t += 4) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const double2 *src = reinterpret_cast<const double2 *>(chunk_first + (size_t)(t + q) * 8);
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                const double2 v = src[h];
                ps[q][2 * h] = __dadd_rn(ps[q][2 * h], v.x);
                ps[q][2 * h + 1] = __dadd_rn(ps[q][2 * h + 1], v.y);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        if (t + q <= t1) {
            const double2 *src = reinterpret_cast<const double2 *>(chunk_first + (size_t)(t + q) * 8);
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                const double2 v = src[h];
                ps[q][2 * h] = __dadd_rn(ps[q][2 * h], v.x);
                ps[q][2 * h + 1] = __dadd_rn(ps[q][2 * h + 1], v.y);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 8; ++c)
        acc[c] = __dadd_rn(__dadd_rn(__dadd_rn(acc[c], ps[0][c]), ps[1][c]), __dadd_rn(ps[2][c], ps[3][c]));
    store8(partial + (size_t)k * 8, acc);
}

// Corner sums of lower cell k from its moments m = [S, Sf1, Sf2, Sf1f2]:
// 00 = S - Sf1 - Sf2 + Sf1f2, 01 = Sf2 - Sf1f2, 10 = Sf1 - Sf1f2, 11 = Sf1f2.
__device__ __forceinline__ double corner00(const double *m) {
    return __dadd_rn(__dsub_rn(__dsub_rn(m[0], m[1]), m[2]), m[3]);
}
__device__ __forceinline__ double corner01(const double *m) { return __dsub_rn(m[2], m[3]); }
__device__ __forceinline__ double corner10(const double *m) { return __dsub_rn(m[1], m[3]); }

__global__ void cic_assemble(const double *__restrict__ partial, int nb1, int nb2,
                             double *__restrict__ out0, double *__restrict__ out1) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nb1 * nb2) return;
    const int a = (int)(t / nb2), b = (int)(t % nb2);
    const int W = nb2 + 1;
    // key of lower cell (i1, i2) = (i1 + 1) * W + (i2 + 1)
    const size_t k00 = (size_t)(a + 1) * W + (b + 1);   // this cell as lower corner
    const size_t k01 = (size_t)(a + 1) * W + b;         // (a, b-1) -> its corner 01
    const size_t k10 = (size_t)a * W + (b + 1);         // (a-1, b) -> its corner 10
    const size_t k11 = (size_t)a * W + b;               // (a-1, b-1) -> its corner 11
    for (int ch = 0; ch < (out1 ? 2 : 1); ++ch) {
        const int o = 4 * ch;
        const double v = __dadd_rn(__dadd_rn(__dadd_rn(corner00(partial + k00 * 8 + o),
                                                        corner01(partial + k01 * 8 + o)),
                                             corner10(partial + k10 * 8 + o)),
                                   partial[k11 * 8 + o + 3]);
        (ch ? out1 : out0)[t] = v;
    }
}

struct DepositLayout {
    uint32_t nkeys;
    int bits, passes, ntiles;
};

static DepositLayout deposit_layout(int64_t n, int nb1, int nb2) {
    DepositLayout L;
    L.nkeys = (uint32_t)(nb1 + 1) * (uint32_t)(nb2 + 1);
    int bits = 1;
    while ((1ull << bits) <= (unsigned long long)L.nkeys) ++bits;   // sentinel included
    L.bits = bits;
    L.passes = (bits + RS_BITS - 1) / RS_BITS;
    L.ntiles = (int)((n + RS_TILE - 1) / RS_TILE);
    if (L.ntiles < 1) L.ntiles = 1;
    return L;
}

static size_t deposit_carve(Carver &c, int64_t n, const DepositLayout &L, uint32_t **ka,
                            uint32_t **va, uint32_t **kb, uint32_t **vb, uint32_t **hist,
                            uint32_t **dtot, uint32_t **cs, uint32_t **ce, double **part,
                            DepGrid **grid) {
    const size_t nn = (size_t)(n > 0 ? n : 1);
    // the four sort buffers hold a multiple of SEG_K entries: after the sort
    // the idle pair (4 B x that many each) is reused as the seg_sums chunk
    // parts (8 doubles per SEG_K particles each)
    const size_t nk = (nn + SEG_K - 1) / SEG_K * SEG_K;
    *ka = c.take<uint32_t>(nk);
    *va = c.take<uint32_t>(nk);
    *kb = c.take<uint32_t>(nk);
    *vb = c.take<uint32_t>(nk);
    *hist = c.take<uint32_t>((size_t)RS_BINS * L.ntiles);
    *dtot = c.take<uint32_t>(RS_BINS);
    *cs = c.take<uint32_t>((size_t)L.nkeys + 1);
    *ce = c.take<uint32_t>((size_t)L.nkeys + 1);
    *part = c.take<double>((size_t)L.nkeys * 8);
    *grid = c.take<DepGrid>(1);
    return c.used;
}

}  // namespace dfcsr

using namespace dfcsr;

extern "C" size_t dfcsr_moments_workspace_bytes(int64_t n) {
    return align_up((size_t)moment_blocks(n) * MOM_K * sizeof(double), 256) + 256;
}

extern "C" int dfcsr_beam_moments(const double *x, const double *z, int64_t n, double *out,
                                  void *workspace, size_t workspace_bytes, void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(x && z && out, "dfcsr_beam_moments: null pointer");
    DFCSR_CHECK_ARG(n > 0, "dfcsr_beam_moments: n must be positive (got %lld)", (long long)n);
    const int nblk = moment_blocks(n);
    if (!workspace || workspace_bytes < dfcsr_moments_workspace_bytes(n)) {
        set_error("dfcsr_beam_moments: workspace too small (%zu < %zu)", workspace_bytes,
                  dfcsr_moments_workspace_bytes(n));
        return DFCSR_OOM;
    }
    cudaStream_t s = as_stream(stream);
    double *part = reinterpret_cast<double *>(workspace);
    ScopedTiming tm("beam_moments", s);
    DFCSR_CUDA_TRY(cudaMemsetAsync(out, 0, 16 * sizeof(double), s));
    note_launch();
    moments_pass<1><<<nblk, MOM_THREADS, 0, s>>>(x, z, n, out, part);
    note_launch();
    moments_finish<1><<<1, MOM_THREADS, 0, s>>>(x, z, part, nblk, n, out);
    note_launch();
    moments_pass<2><<<nblk, MOM_THREADS, 0, s>>>(x, z, n, out, part);
    note_launch();
    moments_finish<2><<<1, MOM_THREADS, 0, s>>>(x, z, part, nblk, n, out);
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}

extern "C" size_t dfcsr_deposit_workspace_bytes(int64_t n, int nb1, int nb2) {
    if (n < 0 || nb1 <= 0 || nb2 <= 0) return 0;
    if (((int64_t)nb1 + 1) * ((int64_t)nb2 + 1) >= (1ll << 30)) return 0;   // refused by the deposit
    const DepositLayout L = deposit_layout(n, nb1, nb2);
    Carver c{nullptr, 0, 0};
    uint32_t *a, *b, *cc, *d, *e, *f, *g, *h;
    double *p;
    DepGrid *gr;
    return deposit_carve(c, n, L, &a, &b, &cc, &d, &e, &f, &g, &h, &p, &gr) + 256;
}

// The grid of get_DF (deposit.py:147-159) from the beam moments on the
// device (m[1], m[2]: means of x and z; m[3], m[4]: their standard
// deviations): start = mean - lim sigma, end = mean + lim sigma, and the
// deposit's inverse spacing 1 / ((end - start) / nbins), in the host's
// operation order.  One thread.
__global__ void grid_from_moments(const double *__restrict__ m, double lim1, double lim2, int nb1,
                                  int nb2, DepGrid *__restrict__ out) {
    const double s1 = __dsub_rn(m[1], __dmul_rn(lim1, m[3]));
    const double e1 = __dadd_rn(m[1], __dmul_rn(lim1, m[3]));
    const double s2 = __dsub_rn(m[2], __dmul_rn(lim2, m[4]));
    const double e2 = __dadd_rn(m[2], __dmul_rn(lim2, m[4]));
    out->start1 = s1;
    out->inv1 = __ddiv_rn(1.0, __ddiv_rn(__dsub_rn(e1, s1), (double)nb1));
    out->start2 = s2;
    out->inv2 = __ddiv_rn(1.0, __ddiv_rn(__dsub_rn(e2, s2), (double)nb2));
}

static int deposit_check(const char *fn, const double *q1, const double *q2, const double *w1,
                         int64_t n, int nb1, int nb2, double *out0, double *out1) {
    DFCSR_CHECK_ARG(out0, "%s: out0 is null", fn);
    DFCSR_CHECK_ARG(nb1 > 0 && nb2 > 0, "%s: bins must be positive (%d, %d)", fn, nb1, nb2);
    DFCSR_CHECK_ARG(((int64_t)nb1 + 1) * ((int64_t)nb2 + 1) < (1ll << 30), "%s: grid %d x %d too large",
                    fn, nb1, nb2);
    DFCSR_CHECK_ARG(n >= 0 && n < (1ll << 32) - 1, "%s: bad particle count %lld", fn, (long long)n);
    DFCSR_CHECK_ARG(n == 0 || (q1 && q2), "%s: null coordinates", fn);
    DFCSR_CHECK_ARG(!(out1 && n > 0 && !w1), "%s: out1 given without w1", fn);
    return DFCSR_OK;
}

// Keys, sort, per-cell sums and assembly on stream s.  The grid is `g`, or
// the DepGrid that grid_from_moments writes into the workspace first when
// `moments` is given.
static int deposit_run(const char *fn, const double *q1, const double *q2, const double *w0,
                       const double *w1, int64_t n, int nb1, int nb2, DepGrid g,
                       const double *moments, double lim1, double lim2, double *out0, double *out1,
                       void *workspace, size_t workspace_bytes, cudaStream_t s) {
    const DepositLayout L = deposit_layout(n, nb1, nb2);
    Carver c{reinterpret_cast<char *>(workspace), workspace_bytes, 0};
    uint32_t *ka, *va, *kb, *vb, *hist, *dtot, *cs, *ce;
    double *part;
    DepGrid *gslot;
    deposit_carve(c, n, L, &ka, &va, &kb, &vb, &hist, &dtot, &cs, &ce, &part, &gslot);
    if (!workspace || !c.ok()) {
        set_error("%s: workspace too small (%zu < %zu)", fn, workspace_bytes, c.used);
        return DFCSR_OOM;
    }
    const DepGrid *gp = nullptr;
    if (moments) {
        note_launch();
        grid_from_moments<<<1, 1, 0, s>>>(moments, lim1, lim2, nb1, nb2, gslot);
        gp = gslot;
    }
    DFCSR_CUDA_TRY(cudaMemsetAsync(cs, 0, sizeof(uint32_t) * ((size_t)L.nkeys + 1), s));
    DFCSR_CUDA_TRY(cudaMemsetAsync(ce, 0, sizeof(uint32_t) * ((size_t)L.nkeys + 1), s));
    // timed from here: on a second stream the memsets above can wait for SM
    // space behind another stream's persistent kernel
    ScopedTiming tm("deposit_cic2d", s);
    if (n > 0) {
        const int tb = 256;
        note_launch();
        cic_keys<<<(unsigned)((n + tb - 1) / tb), tb, 0, s>>>(q1, q2, n, nb1, nb2, g, gp, L.nkeys, ka,
                                                              va);
        uint32_t *kin = ka, *vin = va, *kout = kb, *vout = vb;
        for (int p = 0; p < L.passes; ++p) {
            const int shift = RS_BITS * p;
            note_launch();
            radix_upsweep<<<L.ntiles, RS_THREADS, 0, s>>>(kin, n, shift, L.ntiles, hist);
            note_launch();
            radix_scan_rows<<<RS_BINS, 1024, 0, s>>>(hist, L.ntiles, dtot);
            note_launch();
            radix_scatter<<<L.ntiles, RS_THREADS, sizeof(ScatterSmem), s>>>(kin, vin, n, shift, L.ntiles,
                                                                             hist, dtot, kout, vout);
            uint32_t *t = kin; kin = kout; kout = t;
            t = vin; vin = vout; vout = t;
        }
        note_launch();
        cell_ranges<<<(unsigned)((n + tb - 1) / tb), tb, 0, s>>>(kin, n, L.nkeys, cs, ce);
        double *cfirst = reinterpret_cast<double *>(kout);
        double *clast = reinterpret_cast<double *>(vout);
        const unsigned sb = (unsigned)((n + SEG_TILE - 1) / SEG_TILE);
#define DFCSR_SEG(A, B)                                                                       \
    seg_sums<A, B><<<sb, SEG_THREADS, 0, s>>>(kin, vin, n, L.nkeys, nb2, cs, ce, q1, q2, w0, w1, \
                                              g, gp, part, cfirst, clast)
        note_launch();
        if (w0 && w1) DFCSR_SEG(true, true);
        else if (w0) DFCSR_SEG(true, false);
        else if (w1) DFCSR_SEG(false, true);
        else DFCSR_SEG(false, false);
#undef DFCSR_SEG
        note_launch();
        seg_combine<<<(unsigned)((L.nkeys + 255) / 256), 256, 0, s>>>(
            cs, ce, L.nkeys, (n + SEG_K - 1) / SEG_K, cfirst, clast, part);
    } else {
        DFCSR_CUDA_TRY(cudaMemsetAsync(part, 0, sizeof(double) * (size_t)L.nkeys * 8, s));
    }
    const int64_t cells = (int64_t)nb1 * nb2;
    note_launch();
    cic_assemble<<<(unsigned)((cells + 255) / 256), 256, 0, s>>>(part, nb1, nb2, out0, out1);
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}

extern "C" int dfcsr_deposit_cic2d(const double *q1, const double *q2, const double *w0,
                                   const double *w1, int64_t n, int nb1, double start1,
                                   double end1, int nb2, double start2, double end2,
                                   double *out0, double *out1, void *workspace,
                                   size_t workspace_bytes, void *stream) {
    clear_error();
    const int st = deposit_check("dfcsr_deposit_cic2d", q1, q2, w1, n, nb1, nb2, out0, out1);
    if (st != DFCSR_OK) return st;
    DFCSR_CHECK_ARG(end1 != start1 && end2 != start2, "dfcsr_deposit_cic2d: empty bin range");
    DepGrid g;
    g.start1 = start1;
    g.inv1 = 1.0 / ((end1 - start1) / nb1);
    g.start2 = start2;
    g.inv2 = 1.0 / ((end2 - start2) / nb2);
    return deposit_run("dfcsr_deposit_cic2d", q1, q2, w0, w1, n, nb1, nb2, g, nullptr, 0.0, 0.0,
                       out0, out1, workspace, workspace_bytes, as_stream(stream));
}

extern "C" int dfcsr_deposit_cic2d_moments(const double *q1, const double *q2, const double *w0,
                                           const double *w1, int64_t n, int nb1, int nb2,
                                           const double *moments, double lim1, double lim2,
                                           double *out0, double *out1, void *workspace,
                                           size_t workspace_bytes, void *stream) {
    clear_error();
    const int st = deposit_check("dfcsr_deposit_cic2d_moments", q1, q2, w1, n, nb1, nb2, out0, out1);
    if (st != DFCSR_OK) return st;
    DFCSR_CHECK_ARG(moments, "dfcsr_deposit_cic2d_moments: moments is null");
    DFCSR_CHECK_ARG(lim1 > 0.0 && lim2 > 0.0, "dfcsr_deposit_cic2d_moments: limits must be positive");
    return deposit_run("dfcsr_deposit_cic2d_moments", q1, q2, w0, w1, n, nb1, nb2, DepGrid{}, moments,
                       lim1, lim2, out0, out1, workspace, workspace_bytes, as_stream(stream));
}

DFCSR_BOUNDS_READER(deposit)
