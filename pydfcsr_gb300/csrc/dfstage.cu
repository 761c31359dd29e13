// Distribution-function finalisation on the device: everything
// DF_tracker.get_DF does after the two deposits (pyDFCSR_2D/deposit.py:183-235).
//
// All arithmetic is FP64 and follows the reference's (numpy / scipy) operation
// order: threshold and division, Savitzky-Golay 'interp' smoothing along x then
// z, trapz normalisation (column sums row by row, then numpy pairwise over z),
// numpy.gradient with the host-computed non-uniform coefficients, smoothing of
// the derivatives, and the vx_x fill.  The smoothing is a shared-memory tiled
// stencil: one CTA stages a 32 x (32 + halo) tile and produces 32 x 32 outputs.
#include "dfcsr_common.cuh"

namespace dfcsr {

constexpr int SG_TILE = 32;
constexpr int SG_MAX_WINDOW = 63;

// Two-level deterministic reductions: RED_BLOCKS blocks with a fixed
// element-to-thread assignment, then one block over the partials in order.
constexpr int RED_BLOCKS = 64;

__device__ __forceinline__ double block_max(double v, double *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double r = v;
    if (threadIdx.x == 0) {
        r = red[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = fmax(r, red[w]);
    }
    __syncthreads();
    return r;
}

// OP 0: max(f); OP 1: sum(g) over f > thr2 and count (thr2 = sc[6] / vth * 8);
// OP 2: sum(f).  Final values: OP 0 -> sc[slot] = max; OP 1 -> sc[2] = thr2,
// sc[3] = sum / count (NaN when empty, like numpy.mean of an empty
// selection); OP 2 -> sc[slot] = sum / n.
// One launch: every block writes its partial, and the last block to finish
// (completion counter, reset by that block) combines the partials in block
// order, so the result does not depend on which block finishes last.
template <int OP>
__global__ void __launch_bounds__(256)
reduce_once(const double *__restrict__ f, const double *__restrict__ g, int n,
            double *__restrict__ sc, double vth, double *__restrict__ part, int slot,
            unsigned int *__restrict__ counter) {
    __shared__ double red[8];
    __shared__ bool last;
    double a = (OP == 0) ? -INFINITY : 0.0, c = 0.0;
    double thr2 = 0.0;
    if (OP == 1) thr2 = __dmul_rn(__ddiv_rn(sc[6], vth), 8.0);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (OP == 0) a = fmax(a, f[i]);
        else if (OP == 1) { if (f[i] > thr2) { a += g[i]; c += 1.0; } }
        else a += f[i];
    }
    if (OP == 0) {
        a = block_max(a, red);
    } else {
        a = block_sum(a, red);
        if (OP == 1) c = block_sum(c, red);
    }
    if (threadIdx.x == 0) {
        part[blockIdx.x * 2 + 0] = a;
        part[blockIdx.x * 2 + 1] = c;
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    double A = __ldcg(part), C = __ldcg(part + 1);
    for (int k = 1; k < (int)gridDim.x; ++k) {
        if (OP == 0) A = fmax(A, __ldcg(part + 2 * k));
        else { A += __ldcg(part + 2 * k); C += __ldcg(part + 2 * k + 1); }
    }
    if (OP == 0) sc[slot] = A;
    else if (OP == 1) { sc[2] = thr2; sc[3] = A / C; }
    else sc[slot] = A / (double)n;
    *counter = 0u;
}

// vx[d > thr] /= d[d > thr], thr = max(raw density) / vth  (deposit.py:183-184)
__global__ void threshold_divide(const double *__restrict__ d, double *__restrict__ vx, int n,
                                 double *__restrict__ sc, double vth) {
    const double thr = __ddiv_rn(sc[5], vth);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) sc[1] = thr;
    if (i < n && d[i] > thr) vx[i] = __ddiv_rn(vx[i], d[i]);
}

// Savitzky-Golay along one axis for F fields (blockIdx.z).  AXIS 0 filters
// along x (stride nz), AXIS 1 along z (contiguous).
struct FieldSet {
    const double *src[4];
    double *dst[4];
};

template <int AXIS>
__global__ void __launch_bounds__(256)
sg_axis(FieldSet fs, int nx, int nz, int w, const double *__restrict__ coef,
        const double *__restrict__ elo, const double *__restrict__ ehi) {
    extern __shared__ double tile[];   // [rows][SG_TILE + 1]
    const int L = AXIS == 0 ? nx : nz;     // filter-axis length
    const int M = AXIS == 0 ? nz : nx;     // other-axis length
    const int sL = AXIS == 0 ? nz : 1;
    const int sM = AXIS == 0 ? 1 : nz;
    const int m = w / 2;
    const int l0 = blockIdx.x * SG_TILE, c0 = blockIdx.y * SG_TILE;
    const double *f = fs.src[blockIdx.z];
    double *g = fs.dst[blockIdx.z];
    int lo = l0 - m;
    if (L - w < lo) lo = L - w;
    if (lo < 0) lo = 0;
    int hi = l0 + SG_TILE + m;
    if (hi < w) hi = w;
    if (hi > L) hi = L;
    const int rows = hi - lo;
    const int ld = SG_TILE + 1;
    const int ncol = min(SG_TILE, M - c0);
    for (int idx = threadIdx.x; idx < rows * SG_TILE; idx += blockDim.x) {
        int r, c;
        if (AXIS == 0) { r = idx / SG_TILE; c = idx % SG_TILE; }
        else { c = idx / rows; r = idx % rows; }
        double v = 0.0;
        if (c < ncol) v = f[(size_t)(lo + r) * sL + (size_t)(c0 + c) * sM];
        tile[r * ld + c] = v;
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
        if (l >= m && l < L - m) {
            x = tile + (l - m - lo) * ld + c;
            e = coef;
        } else if (l < m) {
            x = tile + (0 - lo) * ld + c;
            e = elo + (size_t)l * w;
        } else {
            x = tile + (L - w - lo) * ld + c;
            e = ehi + (size_t)(l - (L - m)) * w;
        }
        double a0 = __dmul_rn(x[0], e[0]), a1 = 0.0;
        int k = 1;
        for (; k + 1 < w; k += 2) {
            a1 = __fma_rn(x[k * ld], e[k], a1);
            a0 = __fma_rn(x[(k + 1) * ld], e[k + 1], a0);
        }
        if (k < w) a1 = __fma_rn(x[k * ld], e[k], a1);
        const double acc = __dadd_rn(a0, a1);
        g[(size_t)l * sL + (size_t)(c0 + c) * sM] = acc;
    }
}

// col[j] = sum_i (dx_i * (d[i+1][j] + d[i][j])) / 2.0 (numpy.trapz along
// axis 0): a block covers 32 columns, warp w sums rows w, w + 8, ... of its
// lane's column in order, then the 8 warp partials are added in order; the
// last block to finish then forms the numpy pairwise sum dsum of
// (dz_j * (col[j+1] + col[j])) / 2.0 into sc[0].
__global__ void __launch_bounds__(256)
trapz_once(const double *__restrict__ d, int nx, int nz, const double *__restrict__ dxg,
           const double *__restrict__ dzg, double *__restrict__ col, double *__restrict__ terms,
           double *__restrict__ sc, unsigned int *__restrict__ counter) {
    __shared__ double part[8][33];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = blockIdx.x * 32 + lane;
    double acc = 0.0;
    if (j < nz) {
        for (int i = warp; i < nx - 1; i += 8) {
            const double t = __ddiv_rn(__dmul_rn(dxg[i], __dadd_rn(d[(size_t)(i + 1) * nz + j],
                                                                    d[(size_t)i * nz + j])), 2.0);
            acc = __dadd_rn(acc, t);
        }
    }
    part[warp][lane] = acc;
    __syncthreads();
    if (warp == 0 && j < nz) {
        double s = part[0][lane];
        for (int w = 1; w < 8; ++w) s = __dadd_rn(s, part[w][lane]);
        col[j] = s;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int k = threadIdx.x; k < nz - 1; k += blockDim.x)
        terms[k] = __ddiv_rn(__dmul_rn(dzg[k], __dadd_rn(__ldcg(col + k + 1), __ldcg(col + k))), 2.0);
    __syncthreads();
    if (threadIdx.x == 0) {
        sc[0] = np_pairwise(terms, nz - 1);
        *counter = 0u;
    }
}

// density /= dsum; vx[density <= thr] = 0   (deposit.py:201-204)
__global__ void normalize_fields(double *__restrict__ d, double *__restrict__ vx, int n,
                                 const double *__restrict__ sc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = __ddiv_rn(d[i], sc[0]);
    d[i] = v;
    if (v <= sc[1]) vx[i] = 0.0;
}

// numpy.gradient along one axis with host coefficients g = [a|b|c|edges].
__device__ __forceinline__ double grad_at(const double *f, int i, int n, size_t stride,
                                          const double *g, int uniform, double dx) {
    if (i == 0) return __ddiv_rn(__dsub_rn(f[stride], f[0]), g[3 * n + 0]);
    if (i == n - 1) return __ddiv_rn(__dsub_rn(f[(size_t)(n - 1) * stride], f[(size_t)(n - 2) * stride]),
                                     g[3 * n + 1]);
    const double fm = f[(size_t)(i - 1) * stride], f0 = f[(size_t)i * stride],
                 fp = f[(size_t)(i + 1) * stride];
    if (uniform) return __ddiv_rn(__dsub_rn(fp, fm), __dmul_rn(2.0, dx));
    return __dadd_rn(__dadd_rn(__dmul_rn(g[i], fm), __dmul_rn(g[n + i], f0)), __dmul_rn(g[2 * n + i], fp));
}

__global__ void gradients(const double *__restrict__ d, const double *__restrict__ vx, int nx, int nz,
                          const double *__restrict__ gx, const double *__restrict__ gz,
                          int gxu, double gxdx, int gzu, double gzdx,
                          double *__restrict__ dx_out, double *__restrict__ dz_out,
                          double *__restrict__ vxx_out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nx * nz) return;
    const int i = t / nz, j = t % nz;
    dx_out[t] = grad_at(d + j, i, nx, (size_t)nz, gx, gxu, gxdx);
    dz_out[t] = grad_at(d + (size_t)i * nz, j, nz, 1, gz, gzu, gzdx);
    vxx_out[t] = grad_at(vx + j, i, nx, (size_t)nz, gx, gxu, gxdx);
}

__global__ void fill_vxx(const double *__restrict__ d, double *__restrict__ vxx, int n,
                         const double *__restrict__ sc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && d[i] < sc[2]) vxx[i] = sc[3];
}

static int sg_smem_bytes(int w) {
    const int rows = SG_TILE + 2 * w;
    return rows * (SG_TILE + 1) * (int)sizeof(double);
}

static int launch_sg(int axis, const FieldSet &fs, int nf, int nx, int nz,
                     const dfcsr_df_params *p, cudaStream_t s) {
    const int L = axis == 0 ? nx : nz, M = axis == 0 ? nz : nx;
    dim3 grid((L + SG_TILE - 1) / SG_TILE, (M + SG_TILE - 1) / SG_TILE, nf);
    const int smem = sg_smem_bytes(p->window);
    if (axis == 0)
        sg_axis<0><<<grid, 256, smem, s>>>(fs, nx, nz, p->window, p->sg_coeff, p->sg_lo, p->sg_hi);
    else
        sg_axis<1><<<grid, 256, smem, s>>>(fs, nx, nz, p->window, p->sg_coeff, p->sg_lo, p->sg_hi);
    return 0;
}

}  // namespace dfcsr

using namespace dfcsr;

extern "C" size_t dfcsr_df_workspace_bytes(int nx, int nz) {
    if (nx <= 0 || nz <= 0) return 0;
    const size_t cells = (size_t)nx * nz;
    // 6 temporary fields, column sums, trapz terms, reduction partials
    return 6 * align_up(cells * sizeof(double), 256) + 2 * align_up((size_t)nz * sizeof(double), 256) +
           align_up(2 * RED_BLOCKS * sizeof(double), 256) + 256 + 512;
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
    const size_t need = dfcsr_df_workspace_bytes(nx, nz);
    if (!workspace || workspace_bytes < need) {
        set_error("dfcsr_df_finalize: workspace too small (%zu < %zu)", workspace_bytes, need);
        return DFCSR_OOM;
    }
    cudaStream_t s = as_stream(stream);
    const size_t cells = (size_t)nx * nz;
    Carver c{reinterpret_cast<char *>(workspace), workspace_bytes, 0};
    double *T0 = c.take<double>(cells), *T1 = c.take<double>(cells), *T2 = c.take<double>(cells);
    double *U0 = c.take<double>(cells), *U1 = c.take<double>(cells), *U2 = c.take<double>(cells);
    double *col = c.take<double>(nz), *terms = c.take<double>(nz);
    double *rpart = c.take<double>(2 * RED_BLOCKS);
    unsigned int *counter = c.take<unsigned int>(64);   // completion counters, zero between uses
    const int n = (int)cells;
    const int tb = 256, nb = (n + tb - 1) / tb;
    const double vth = p->velocity_threshold;

    ScopedTiming tm("df_finalize", s);
    DFCSR_CUDA_TRY(cudaMemsetAsync(counter, 0, 64 * sizeof(unsigned int), s));
    reduce_once<0><<<RED_BLOCKS, 256, 0, s>>>(density, nullptr, n, sc, vth, rpart, 5, counter);
    threshold_divide<<<nb, tb, 0, s>>>(density, vx, n, sc, vth);
    launch_sg(0, FieldSet{{density, vx}, {T0, T1}}, 2, nx, nz, p, s);
    launch_sg(1, FieldSet{{T0, T1}, {density, vx}}, 2, nx, nz, p, s);
    trapz_once<<<(nz + 31) / 32, 256, 0, s>>>(density, nx, nz, p->dxg, p->dzg, col, terms, sc,
                                              counter + 16);
    normalize_fields<<<nb, tb, 0, s>>>(density, vx, n, sc);
    gradients<<<nb, tb, 0, s>>>(density, vx, nx, nz, p->gx, p->gz, p->gx_uniform, p->gx_dx,
                                p->gz_uniform, p->gz_dx, U0, U1, U2);
    launch_sg(0, FieldSet{{U0, U1, U2}, {T0, T1, T2}}, 3, nx, nz, p, s);
    launch_sg(1, FieldSet{{T0, T1, T2}, {density_x, density_z, vx_x}}, 3, nx, nz, p, s);
    reduce_once<0><<<RED_BLOCKS, 256, 0, s>>>(density, nullptr, n, sc, vth, rpart, 6, counter);
    reduce_once<1><<<RED_BLOCKS, 256, 0, s>>>(density, vx_x, n, sc, vth, rpart, 3, counter);
    fill_vxx<<<nb, tb, 0, s>>>(density, vx_x, n, sc);
    reduce_once<2><<<RED_BLOCKS, 256, 0, s>>>(vx_x, nullptr, n, sc, vth, rpart, 4, counter);
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}
