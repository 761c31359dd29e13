// Distribution-function finalisation on the device: everything
// DF_tracker.get_DF does after the two deposits (pyDFCSR_2D/deposit.py:183-235).
//
// All arithmetic is FP64: threshold and division, Savitzky-Golay 'interp'
// smoothing along x then z, trapz normalisation, numpy.gradient with the
// host-computed non-uniform coefficients, smoothing of the derivatives, and
// the vx_x fill.  Elementwise operations are the reference's (numpy / scipy)
// operations; sums (stencils, trapz, means) are evaluated in fixed orders of
// their own, within ~1e-15 relative of numpy's.  The smoothing is a shared-memory tiled
// stencil: a CTA stages a 32 x (32 + halo) tile and produces 32 x 32 outputs.
//
// The whole stage is ONE cooperative launch: the phases are separated by a
// grid barrier (every CTA resident, bounded spin), and each phase loops over
// "virtual blocks" of a fixed work split - the reductions keep a fixed
// element-to-thread assignment over RED_BLOCKS x 256 threads and fixed
// combining trees, so the results do not depend on the grid size.  The
// elementwise steps (threshold division, gradients) are applied while the
// smoothing tiles are staged.  A 256^2 grid is ~65k cells, a few
// microseconds of work per phase: the stage is bound by its chain of
// dependent steps (FP64 latency, barriers), so sums are trees, not chains.
// Data written by other CTAs during the launch is read with ld.global.cg
// (from L2), never through the non-coherent L1.
#include <mutex>

#include "dfcsr_common.cuh"

namespace dfcsr {

constexpr int SG_TILE = 32;
constexpr int SG_MAX_WINDOW = 63;
constexpr int DF_THREADS = 256;
constexpr int DF_BLOCKS_PER_SM = 1;
constexpr int TRAPZ_ROWS = 32;   // 8 warps x 4 rows

// Deterministic reductions: RED_BLOCKS virtual blocks with a fixed
// element-to-thread assignment, partials combined in block order.
constexpr int RED_BLOCKS = 64;

// Grid barrier state (zeroed before the launch): arrivals, generation,
// error; arrivals of the trapz column CTAs.
struct GridBar {
    unsigned int count, gen, err, trapz;
};

// All CTAs of the cooperative launch meet here: `arrivals` CTAs are
// expected (the grid).  The spin is bounded by `max_spins` polls (the stage
// uses kBarSpins, about a second); on expiry the CTA records an error and
// continues.  Once an error is recorded no CTA waits at a barrier again (the
// arrival count is out of step after a wait gave up, so a later meeting
// could release early or never): every CTA runs to the end of the launch,
// and the stage then writes NaN scalars and its error flag.
constexpr unsigned int kBarSpins = 1u << 24;

__device__ __forceinline__ void grid_sync(GridBar *b, unsigned int arrivals, unsigned int max_spins) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int *verr = &b->err;
        if (*verr == 0u) {
            volatile unsigned int *vgen = &b->gen;
            const unsigned int g = *vgen;
            __threadfence();
            if (atomicAdd(&b->count, 1u) == arrivals - 1) {
                atomicExch(&b->count, 0u);
                __threadfence();
                atomicAdd(&b->gen, 1u);
            } else {
                unsigned int it = 0;
                while (*vgen == g && *verr == 0u) {
                    if (++it > max_spins) {
                        atomicExch(&b->err, 1u);
                        break;
                    }
                    __nanosleep(64);
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
}

// The stage's barrier: the grid's CTAs plus p.barrier_extra (0; 1 only to
// exercise the timeout path: an arrival that never comes), at most
// p.barrier_spins polls (0: kBarSpins).
__device__ __forceinline__ void grid_sync(GridBar *b, const dfcsr_df_params &p) {
    grid_sync(b, gridDim.x + (unsigned int)p.barrier_extra, p.barrier_spins ? p.barrier_spins : kBarSpins);
}

__device__ __forceinline__ double ldcg(const double *p) { return __ldcg(p); }

// FP64 on this GPU has a latency of some hundred cycles per dependent
// operation, so every reduction here is a fixed tree (a chain of log2 n
// operations) rather than a running sum (a chain of n).  The trees are
// fixed, so the results are deterministic.

// OP 0: fmax, else +.  The xor butterfly leaves the same bits in every lane
// (both operands of each step are the same pair, and + and fmax commute).
template <int OP>
__device__ __forceinline__ double comb(double a, double b) { return OP == 0 ? fmax(a, b) : a + b; }

template <int OP>
__device__ __forceinline__ double warp_tree(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = comb<OP>(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide tree; result valid in every thread.  red: blockDim / 32 slots.
template <int OP>
__device__ double block_tree(double v, double *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_tree<OP>(v);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    const double id = OP == 0 ? -INFINITY : 0.0;
    double r = (lane < (int)(blockDim.x >> 5)) ? red[lane] : id;
    r = warp_tree<OP>(r);
    __syncthreads();   // red is reused by the next call
    return r;
}

// Partials of one reduction over virtual blocks vb (elements vb * 256 + tid
// + k * RED_BLOCKS * 256).  OP 0: max(f); OP 1: sum(g) over f > thr2 and the
// count; OP 2: sum(f).
template <int OP>
__device__ void reduce_part(const double *f, const double *g, int n, double thr2, double *part,
                            double *red) {
    for (int vb = blockIdx.x; vb < RED_BLOCKS; vb += gridDim.x) {
        double a = (OP == 0) ? -INFINITY : 0.0, c = 0.0;
#pragma unroll 4
        for (int i = vb * DF_THREADS + threadIdx.x; i < n; i += RED_BLOCKS * DF_THREADS) {
            const double fi = ldcg(f + i);
            if (OP == 0) a = fmax(a, fi);
            else if (OP == 1) { if (fi > thr2) { a += ldcg(g + i); c += 1.0; } }
            else a += fi;
        }
        a = block_tree<OP == 0 ? 0 : 1>(a, red);
        if (OP == 1) c = block_tree<1>(c, red);
        if (threadIdx.x == 0) {
            part[vb * 2 + 0] = a;
            part[vb * 2 + 1] = c;
        }
    }
}

// The RED_BLOCKS partials combined by a fixed tree in warp 0 (every CTA that
// calls it gets the same bits); the result is returned in every thread.
template <int OP>
__device__ void reduce_combine(const double *part, double *stage, double &A, double &C) {
    static_assert(RED_BLOCKS == 64, "two partials per lane");
    if (threadIdx.x < 32) {
        const int l = threadIdx.x;
        A = warp_tree<OP == 0 ? 0 : 1>(comb<OP == 0 ? 0 : 1>(ldcg(part + 2 * l), ldcg(part + 2 * (l + 32))));
        C = warp_tree<1>(ldcg(part + 2 * l + 1) + ldcg(part + 2 * (l + 32) + 1));
        if (l == 0) { stage[0] = A; stage[1] = C; }
    }
    __syncthreads();
    A = stage[0];
    C = stage[1];
    __syncthreads();
}

// Savitzky-Golay along one axis for nf fields.  AXIS 0 filters along x
// (stride nz), AXIS 1 along z (contiguous).  Virtual block = one 32 x 32
// output tile of one field.  The input element (field f, filter-axis index
// l, other index m) comes from load(f, l, m), so that a preceding
// elementwise step (threshold division, gradients) is applied while the
// tile is staged instead of in a pass of its own.
template <int AXIS, class Load>
__device__ void sg_phase(const Load &load, double *const *dst, int nf, int nx, int nz, int w,
                         const double *__restrict__ coef, const double *__restrict__ elo,
                         const double *__restrict__ ehi, double *tile) {
    const int L = AXIS == 0 ? nx : nz;     // filter-axis length
    const int M = AXIS == 0 ? nz : nx;     // other-axis length
    const int sL = AXIS == 0 ? nz : 1;
    const int sM = AXIS == 0 ? 1 : nz;
    const int m = w / 2;
    const int nbl = (L + SG_TILE - 1) / SG_TILE, nbm = (M + SG_TILE - 1) / SG_TILE;
    const int ntiles = nbl * nbm * nf;
    const int ld = SG_TILE + 1;
    for (int vb = blockIdx.x; vb < ntiles; vb += gridDim.x) {
        const int bl = vb % nbl, bm = (vb / nbl) % nbm, bf = vb / (nbl * nbm);
        const int l0 = bl * SG_TILE, c0 = bm * SG_TILE;
        double *g = dst[bf];
        int lo = l0 - m;
        if (L - w < lo) lo = L - w;
        if (lo < 0) lo = 0;
        int hi = l0 + SG_TILE + m;
        if (hi < w) hi = w;
        if (hi > L) hi = L;
        const int rows = hi - lo;
        const int ncol = min(SG_TILE, M - c0);
#pragma unroll 4
        for (int idx = threadIdx.x; idx < rows * SG_TILE; idx += blockDim.x) {
            int r, c;
            if (AXIS == 0) { r = idx / SG_TILE; c = idx % SG_TILE; }
            else { c = idx / rows; r = idx % rows; }
            tile[r * ld + c] = (c < ncol && bounds_ok(lo + r, L, BS_DF) && bounds_ok(c0 + c, M, BS_DF))
                                   ? load(bf, lo + r, c0 + c)
                                   : 0.0;
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < SG_TILE * SG_TILE; idx += blockDim.x) {
            int rl, c;
            if (AXIS == 0) { rl = idx / SG_TILE; c = idx % SG_TILE; }
            else { c = idx / SG_TILE; rl = idx % SG_TILE; }
            const int l = l0 + rl;
            if (l >= L || c >= ncol) continue;
            // the window's weights (interior, left edge or right edge map) and
            // its first sample; two fused multiply-add chains (even / odd taps)
            const double *x, *e;
            int r0;   // the window's first staged row
            if (l >= m && l < L - m) {
                r0 = l - m - lo;
                e = coef;
            } else if (l < m) {
                r0 = 0 - lo;
                e = elo + (size_t)l * w;
            } else {
                r0 = L - w - lo;
                e = ehi + (size_t)(l - (L - m)) * w;
            }
            if (!(bounds_ok(r0, rows, BS_DF) && bounds_ok(r0 + w - 1, rows, BS_DF))) continue;
            x = tile + r0 * ld + c;
            double a0 = __dmul_rn(x[0], e[0]), a1 = 0.0;
            int k = 1;
            for (; k + 1 < w; k += 2) {
                a1 = __fma_rn(x[k * ld], e[k], a1);
                a0 = __fma_rn(x[(k + 1) * ld], e[k + 1], a0);
            }
            if (k < w) a1 = __fma_rn(x[k * ld], e[k], a1);
            g[(size_t)l * sL + (size_t)(c0 + c) * sM] = __dadd_rn(a0, a1);
        }
        __syncthreads();   // the tile is reused by the next virtual block
    }
}

// Loaders of the smoothing phases (f: field, l: filter-axis index, m: other).
template <int AXIS>
struct LoadPlain {   // fields src[f] as they are
    const double *src[3];
    int nz;
    __device__ double operator()(int f, int l, int m) const {
        const int i = AXIS == 0 ? l : m, j = AXIS == 0 ? m : l;
        return ldcg(src[f] + (size_t)i * nz + j);
    }
};

struct LoadThrDiv {  // density, and vx / density where density > thr (deposit.py:183-184)
    const double *d, *vx;
    double thr;
    int nz;
    __device__ double operator()(int f, int l, int m) const {
        const size_t k = (size_t)l * nz + m;
        const double dk = ldcg(d + k);
        if (f == 0) return dk;
        const double v = ldcg(vx + k);
        return dk > thr ? __ddiv_rn(v, dk) : v;
    }
};

// numpy.gradient along one axis with host coefficients g = [a|b|c|edges].
__device__ __forceinline__ double grad_at(const double *f, int i, int n, size_t stride,
                                          const double *g, int uniform, double dx) {
    if (i == 0) return __ddiv_rn(__dsub_rn(ldcg(f + stride), ldcg(f)), g[3 * n + 0]);
    if (i == n - 1)
        return __ddiv_rn(__dsub_rn(ldcg(f + (size_t)(n - 1) * stride), ldcg(f + (size_t)(n - 2) * stride)),
                         g[3 * n + 1]);
    const double fm = ldcg(f + (size_t)(i - 1) * stride), f0 = ldcg(f + (size_t)i * stride),
                 fp = ldcg(f + (size_t)(i + 1) * stride);
    if (uniform) return __ddiv_rn(__dsub_rn(fp, fm), __dmul_rn(2.0, dx));
    return __dadd_rn(__dadd_rn(__dmul_rn(g[i], fm), __dmul_rn(g[n + i], f0)), __dmul_rn(g[2 * n + i], fp));
}

struct LoadGrad {     // numpy.gradient of density along x and z, of vx along x
    const double *d, *vx, *gx, *gz;
    int nx, nz, gxu, gzu;
    double gxdx, gzdx;
    __device__ double operator()(int f, int i, int j) const {   // AXIS 0: l = i (x), m = j (z)
        if (f == 0) return grad_at(d + j, i, nx, (size_t)nz, gx, gxu, gxdx);
        if (f == 1) return grad_at(d + (size_t)i * nz, j, nz, 1, gz, gzu, gzdx);
        return grad_at(vx + j, i, nx, (size_t)nz, gx, gxu, gxdx);
    }
};

struct DfArgs {
    dfcsr_df_params p;
    double *density, *vx, *density_x, *density_z, *vx_x, *sc;
    double *T0, *T1, *T2, *col, *tpart, *part0, *part1;
    GridBar *bar;
};

__global__ void __launch_bounds__(DF_THREADS)
df_stage(DfArgs A) {
    extern __shared__ double tile[];
    __shared__ double red[DF_THREADS / 32];
    __shared__ bool last;
    const dfcsr_df_params &p = A.p;
    const int nx = p.nx, nz = p.nz, n = nx * nz, w = p.window;
    const double vth = p.velocity_threshold;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    double *sc = A.sc;

    // max of the raw density (deposit.py:183)
    reduce_part<0>(A.density, nullptr, n, 0.0, A.part0, red);
    grid_sync(A.bar, p);
    // thr = max / vth (every CTA combines the partials); smoothing along x of
    // density and of vx / density where density > thr (deposit.py:183-195)
    {
        double mx, c;
        reduce_combine<0>(A.part0, tile, mx, c);
        const double thr = __ddiv_rn(mx, vth);
        if (gtid == 0) { sc[5] = mx; sc[1] = thr; }
        double *dst[2] = {A.T0, A.T1};
        sg_phase<0>(LoadThrDiv{A.density, A.vx, thr, nz}, dst, 2, nx, nz, w, p.sg_coeff, p.sg_lo,
                    p.sg_hi, tile);
    }
    grid_sync(A.bar, p);
    // ... then along z, into density and vx
    {
        double *dst[2] = {A.density, A.vx};
        sg_phase<1>(LoadPlain<1>{{A.T0, A.T1, nullptr}, nz}, dst, 2, nx, nz, w, p.sg_coeff, p.sg_lo,
                    p.sg_hi, tile);
    }
    grid_sync(A.bar, p);
    // trapz (deposit.py:197-199): col[j] = sum over rows i of
    // (dx_i * (d[i+1][j] + d[i][j])) / 2.0 by a fixed tree.  Virtual block =
    // 32 columns x TRAPZ_ROWS rows: warp w adds its 4 rows as a pair of
    // pairs, the 8 warps are added as a tree -> chunk partial tpart[k][j].
    // The last of these CTAs adds each column's chunks in order into col[j]
    // and sums (dz_j * (col[j+1] + col[j])) / 2.0 over z by a block tree into
    // sc[0].  (a / 2.0 == a * 0.5 exactly: scaling by a power of 2.)
    {
        const int ngroups = (nz + 31) / 32, nchunks = (nx - 1 + TRAPZ_ROWS - 1) / TRAPZ_ROWS;
        const int nvb = ngroups * nchunks;
        if ((int)blockIdx.x < nvb) {
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
            double *wp = tile;   // [8][33]
            for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
                const int g = vb % ngroups, k = vb / ngroups;
                const int j = g * 32 + lane;
                double t[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int i = k * TRAPZ_ROWS + warp * 4 + u;
                    t[u] = (j < nz && i < nx - 1)
                               ? __dmul_rn(__dmul_rn(p.dxg[i], __dadd_rn(ldcg(A.density + (size_t)(i + 1) * nz + j),
                                                                         ldcg(A.density + (size_t)i * nz + j))),
                                           0.5)
                               : 0.0;
                }
                wp[warp * 33 + lane] = __dadd_rn(__dadd_rn(t[0], t[1]), __dadd_rn(t[2], t[3]));
                __syncthreads();
                if (warp == 0 && j < nz) {
                    const double *q = wp + lane;
                    A.tpart[(size_t)k * nz + j] =
                        __dadd_rn(__dadd_rn(__dadd_rn(q[0], q[33]), __dadd_rn(q[66], q[99])),
                                  __dadd_rn(__dadd_rn(q[132], q[165]), __dadd_rn(q[198], q[231])));
                }
                __syncthreads();
            }
            if (threadIdx.x == 0) {
                __threadfence();
                const int parts = (int)gridDim.x < nvb ? (int)gridDim.x : nvb;
                last = atomicAdd(&A.bar->trapz, 1u) == (unsigned)parts - 1;
            }
            __syncthreads();
            if (last) {
                __threadfence();
                for (int jj = threadIdx.x; jj < nz; jj += blockDim.x) {
                    double c = ldcg(A.tpart + jj);
                    for (int k = 1; k < nchunks; ++k) c = __dadd_rn(c, ldcg(A.tpart + (size_t)k * nz + jj));
                    A.col[jj] = c;
                }
                __syncthreads();
                // sum over z of the terms: thread t adds terms t, t + 256, ...
                // in order, then a block tree
                double a = 0.0;
                for (int k = threadIdx.x; k < nz - 1; k += blockDim.x)
                    a = __dadd_rn(a, __dmul_rn(__dmul_rn(p.dzg[k], __dadd_rn(ldcg(A.col + k + 1), ldcg(A.col + k))), 0.5));
                a = block_tree<1>(a, red);
                if (threadIdx.x == 0) sc[0] = a;
            }
        }
    }
    grid_sync(A.bar, p);
    // density /= dsum; vx[density <= thr] = 0 (deposit.py:201-204), and the
    // max of the normalised density (deposit.py:229) over the reduction's
    // element assignment
    {
        const double dsum = ldcg(sc + 0), thr = ldcg(sc + 1);
        for (int vb = blockIdx.x; vb < RED_BLOCKS; vb += gridDim.x) {
            double a = -INFINITY;
#pragma unroll 4
            for (int i = vb * DF_THREADS + threadIdx.x; i < n; i += RED_BLOCKS * DF_THREADS) {
                const double v = __ddiv_rn(ldcg(A.density + i), dsum);
                A.density[i] = v;
                if (v <= thr) A.vx[i] = 0.0;
                a = fmax(a, v);
            }
            a = block_tree<0>(a, red);
            if (threadIdx.x == 0) {
                A.part1[vb * 2 + 0] = a;
                A.part1[vb * 2 + 1] = 0.0;
            }
        }
    }
    grid_sync(A.bar, p);
    // gradients (deposit.py:207-215), formed while staging, smoothed along x ...
    {
        double *dst[3] = {A.T0, A.T1, A.T2};
        sg_phase<0>(LoadGrad{A.density, A.vx, p.gx, p.gz, nx, nz, p.gx_uniform, p.gz_uniform, p.gx_dx,
                             p.gz_dx},
                    dst, 3, nx, nz, w, p.sg_coeff, p.sg_lo, p.sg_hi, tile);
    }
    grid_sync(A.bar, p);
    // ... and along z into density_x, density_z, vx_x
    {
        double *dst[3] = {A.density_x, A.density_z, A.vx_x};
        sg_phase<1>(LoadPlain<1>{{A.T0, A.T1, A.T2}, nz}, dst, 3, nx, nz, w, p.sg_coeff, p.sg_lo, p.sg_hi,
                    tile);
    }
    grid_sync(A.bar, p);
    // thr2 = max(density) / vth * 8; mean of vx_x over density > thr2
    // (deposit.py:229-231)
    double mx2, c2;
    reduce_combine<0>(A.part1, tile, mx2, c2);
    const double thr2 = __dmul_rn(__ddiv_rn(mx2, vth), 8.0);
    reduce_part<1>(A.density, A.vx_x, n, thr2, A.part0, red);
    grid_sync(A.bar, p);
    // vx_x[density < thr2] = fill (deposit.py:232) and the sum of vx_x for
    // its mean, in one pass over the reduction's element assignment
    double fill;
    {
        double s, c;
        reduce_combine<1>(A.part0, tile, s, c);
        fill = s / c;   // NaN when no cell is above thr2, like numpy.mean
    }
    if (gtid == 0) { sc[6] = mx2; sc[2] = thr2; sc[3] = fill; }
    for (int vb = blockIdx.x; vb < RED_BLOCKS; vb += gridDim.x) {
        double a = 0.0;
#pragma unroll 4
        for (int i = vb * DF_THREADS + threadIdx.x; i < n; i += RED_BLOCKS * DF_THREADS) {
            double v = ldcg(A.vx_x + i);
            if (ldcg(A.density + i) < thr2) {
                v = fill;
                A.vx_x[i] = v;
            }
            a += v;
        }
        a = block_tree<1>(a, red);
        if (threadIdx.x == 0) {
            A.part1[vb * 2 + 0] = a;
            A.part1[vb * 2 + 1] = 0.0;
        }
    }
    grid_sync(A.bar, p);
    if (blockIdx.x == 0) {
        double s, c;
        reduce_combine<2>(A.part1, tile, s, c);
        if (threadIdx.x == 0) {
            sc[4] = s / (double)n;
            const bool failed = *(volatile unsigned int *)&A.bar->err != 0u;
            if (failed) {
                for (int k = 0; k < 7; ++k) sc[k] = __longlong_as_double(0x7ff8000000000000ll);
            }
            sc[7] = failed ? 1.0 : 0.0;
        }
    }
}

// dynamic shared memory: the smoothing tile, the trapz warp partials
// (8 x 33), the trapz terms over z (nz - 1), the staged reduction results
static size_t df_smem_bytes(int w, int nz) {
    size_t b = (size_t)(SG_TILE + 2 * w) * (SG_TILE + 1) * sizeof(double);
    if ((size_t)8 * 33 * sizeof(double) > b) b = (size_t)8 * 33 * sizeof(double);
    if ((size_t)nz * sizeof(double) > b) b = (size_t)nz * sizeof(double);
    if (2 * RED_BLOCKS * sizeof(double) > b) b = 2 * RED_BLOCKS * sizeof(double);
    return b;
}

}  // namespace dfcsr

using namespace dfcsr;

extern "C" size_t dfcsr_df_workspace_bytes(int nx, int nz) {
    if (nx <= 0 || nz <= 0) return 0;
    const size_t cells = (size_t)nx * nz;
    // 3 temporary fields, column sums, trapz chunk partials, two sets of
    // reduction partials, the grid barrier
    const size_t nchunks = (size_t)(nx - 1 + TRAPZ_ROWS - 1) / TRAPZ_ROWS;
    return 3 * align_up(cells * sizeof(double), 256) + align_up((size_t)nz * sizeof(double), 256) +
           align_up(nchunks * nz * sizeof(double), 256) + 2 * align_up(2 * RED_BLOCKS * sizeof(double), 256) +
           256 + 512;
}

extern "C" int dfcsr_df_finalize(const dfcsr_df_params *p, double *density, double *vx,
                                 double *density_x, double *density_z, double *vx_x,
                                 double *sc, void *workspace, size_t workspace_bytes, void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(p, "dfcsr_df_finalize: null params");
    DFCSR_CHECK_ARG(density && vx && density_x && density_z && vx_x && sc,
                    "dfcsr_df_finalize: null field pointer");
    const int nx = p->nx, nz = p->nz;
    DFCSR_CHECK_ARG(nx >= 2 && nz >= 2, "dfcsr_df_finalize: grid %d x %d too small", nx, nz);
    DFCSR_CHECK_ARG((int64_t)nx * nz <= (int64_t)INT32_MAX, "dfcsr_df_finalize: grid %d x %d too large",
                    nx, nz);
    DFCSR_CHECK_ARG(p->window % 2 == 1 && p->window >= 1 && p->window <= SG_MAX_WINDOW,
                    "dfcsr_df_finalize: window_length must be odd and <= %d (got %d)",
                    SG_MAX_WINDOW, p->window);
    DFCSR_CHECK_ARG(p->order >= 0 && p->order < p->window,
                    "dfcsr_df_finalize: polyorder must be less than window_length");
    DFCSR_CHECK_ARG(p->window <= nx && p->window <= nz,
                    "dfcsr_df_finalize: If mode is 'interp', window_length must be less than or "
                    "equal to the size of x.");
    DFCSR_CHECK_ARG(p->sg_coeff && p->sg_lo && p->sg_hi && p->gx && p->gz && p->dxg && p->dzg,
                    "dfcsr_df_finalize: null parameter array");
    DFCSR_CHECK_ARG(nz <= 16384, "dfcsr_df_finalize: at most 16384 z bins (got %d)", nz);
    DFCSR_CHECK_ARG(p->barrier_extra == 0 || p->barrier_extra == 1,
                    "dfcsr_df_finalize: barrier_extra must be 0 or 1 (got %d)", p->barrier_extra);
    DFCSR_CHECK_ARG(p->barrier_spins <= kBarSpins,
                    "dfcsr_df_finalize: barrier_spins must be at most %u (got %u)", kBarSpins, p->barrier_spins);
    const size_t need = dfcsr_df_workspace_bytes(nx, nz);
    if (!workspace || workspace_bytes < need) {
        set_error("dfcsr_df_finalize: workspace too small (%zu < %zu)", workspace_bytes, need);
        return DFCSR_OOM;
    }
    cudaStream_t s = as_stream(stream);
    const size_t cells = (size_t)nx * nz;
    Carver c{reinterpret_cast<char *>(workspace), workspace_bytes, 0};
    DfArgs A;
    A.p = *p;
    A.density = density; A.vx = vx; A.density_x = density_x; A.density_z = density_z;
    A.vx_x = vx_x; A.sc = sc;
    A.T0 = c.take<double>(cells); A.T1 = c.take<double>(cells); A.T2 = c.take<double>(cells);
    A.col = c.take<double>(nz);
    A.tpart = c.take<double>((size_t)((nx - 1 + TRAPZ_ROWS - 1) / TRAPZ_ROWS) * nz);
    A.part0 = c.take<double>(2 * RED_BLOCKS);
    A.part1 = c.take<double>(2 * RED_BLOCKS);
    A.bar = c.take<GridBar>(1);

    const int smem = (int)df_smem_bytes(p->window, nz);
    {
        // the dynamic shared-memory limit is a per-device function attribute
        static std::mutex mu;
        static int smem_set[64];
        int dev = 0;
        DFCSR_CUDA_TRY(cudaGetDevice(&dev));
        DFCSR_CHECK_ARG(dev >= 0 && dev < 64, "dfcsr_df_finalize: device ordinal %d out of range", dev);
        std::lock_guard<std::mutex> g(mu);
        if (smem > 48 * 1024 && smem > smem_set[dev]) {
            DFCSR_CUDA_TRY(cudaFuncSetAttribute(df_stage, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
            smem_set[dev] = smem;
        }
    }
    // every CTA must be resident at once: a cooperative launch no larger than
    // the occupancy allows
    int per_sm = 0;
    DFCSR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, df_stage, DF_THREADS, smem));
    DFCSR_CHECK_ARG(per_sm >= 1, "dfcsr_df_finalize: window %d needs too much shared memory", p->window);
    const int blocks = num_sms() * (per_sm < DF_BLOCKS_PER_SM ? per_sm : DF_BLOCKS_PER_SM);

    ScopedTiming tm("df_finalize", s);
    DFCSR_CUDA_TRY(cudaMemsetAsync(A.bar, 0, sizeof(GridBar), s));
    void *args[] = {&A};
    note_launch();
    DFCSR_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)df_stage, dim3(blocks), dim3(DF_THREADS), args,
                                               (size_t)smem, s));
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}

// ------------------------------------------------------ barrier health check
namespace dfcsr {

// One meeting of the stage's grid barrier.  With `arrivals` above the
// launch's CTAs the last arrival never comes: every CTA's wait gives up
// after `max_spins` polls and records the error.
__global__ void gridbar_check(GridBar *b, unsigned int arrivals, unsigned int max_spins) {
    grid_sync(b, arrivals, max_spins);
}

}  // namespace dfcsr

extern "C" int dfcsr_grid_barrier_check(int blocks, int extra_arrivals, unsigned int max_spins,
                                        void *workspace, size_t workspace_bytes, void *stream) {
    using namespace dfcsr;
    clear_error();
    DFCSR_CHECK_ARG(blocks >= 1 && blocks <= num_sms(),
                    "dfcsr_grid_barrier_check: blocks must be in [1, %d] (got %d)", num_sms(), blocks);
    DFCSR_CHECK_ARG(extra_arrivals == 0 || extra_arrivals == 1,
                    "dfcsr_grid_barrier_check: extra_arrivals must be 0 or 1 (got %d)", extra_arrivals);
    DFCSR_CHECK_ARG(max_spins >= 1 && max_spins <= kBarSpins,
                    "dfcsr_grid_barrier_check: max_spins must be in [1, %u] (got %u)", kBarSpins, max_spins);
    DFCSR_CHECK_ARG(workspace && workspace_bytes >= sizeof(GridBar),
                    "dfcsr_grid_barrier_check: workspace needs %zu bytes", sizeof(GridBar));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    GridBar *bar = reinterpret_cast<GridBar *>(workspace);
    DFCSR_CUDA_TRY(cudaMemsetAsync(bar, 0, sizeof(GridBar), s));
    unsigned int arrivals = (unsigned int)(blocks + extra_arrivals);
    void *args[] = {&bar, &arrivals, &max_spins};
    note_launch();
    DFCSR_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)gridbar_check, dim3(blocks), dim3(32), args, 0, s));
    DFCSR_LAUNCH_CHECK();
    unsigned int err = 0;
    DFCSR_CUDA_TRY(cudaMemcpyAsync(&err, &bar->err, sizeof(err), cudaMemcpyDeviceToHost, s));
    DFCSR_CUDA_TRY(cudaStreamSynchronize(s));
    if (err != 0u) {
        set_error("dfcsr_grid_barrier_check: the barrier wait gave up after %u polls", max_spins);
        return DFCSR_TIMEOUT;
    }
    return DFCSR_OK;
}

DFCSR_BOUNDS_READER(dfstage)
