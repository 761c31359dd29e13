// Particle-side steps around the wake: linear transport by a 6x6 matrix and
// the wake kick (Beam.apply_wakes, pyDFCSR_2D/beams.py:108-131).
//
// Particles are the [6, ld] row-major FP64 array of the Beam (rows x, px, y,
// py, z, pz; particle i is column i).  Both kernels are one thread per
// particle, read the rows they need with coalesced loads and update in place.
#include "dfcsr_common.cuh"

namespace dfcsr {

struct Matrix6 {
    double m[36];
};

// y_r = sum_k R[r][k] x_k as a fused multiply-add chain in increasing k,
// starting from the first non-zero coefficient; zero coefficients are
// skipped (the branch is uniform: every thread sees the same matrix).
__global__ void __launch_bounds__(256)
transport6(Matrix6 R, double *__restrict__ p, int64_t n, int64_t ld) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) x[k] = p[k * ld + i];
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        double acc = 0.0;
        bool first = true;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const double c = R.m[r * 6 + k];
            if (c != 0.0) {
                acc = first ? __dmul_rn(c, x[k]) : __fma_rn(c, x[k], acc);
                first = false;
            }
        }
        p[r * ld + i] = acc;
    }
}

// Scaled kick tables: kick = ((step * wake) * 1e6) / energy, the order of
// `step_size * dE_dct * 1e6 / self.init_energy` (beams.py:110, 120).
__global__ void scale_kicks(const double *__restrict__ dE, const double *__restrict__ xk, int64_t cells,
                            double step, double energy, double *__restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cells) return;
    out[t] = __ddiv_rn(__dmul_rn(__dmul_rn(step, dE[t]), 1e6), energy);
    if (xk) out[cells + t] = __ddiv_rn(__dmul_rn(__dmul_rn(step, xk[t]), 1e6), energy);
}

// RegularGridInterpolator axis lookup (linear, bounds_error=False): the
// interval i = clip(searchsorted(grid, t, 'right') - 1, 0, n - 2), the
// normalised distance (t - g[i]) / (g[i+1] - g[i]) and the out-of-bounds test
// t < g[0] or t > g[n-1].
__device__ __forceinline__ bool rgi_lookup(const double *g, int n, double t, int &i, double &w) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (g[mid] <= t) lo = mid + 1;
        else hi = mid;
    }
    i = lo - 1;
    if (i < 0) i = 0;
    if (i > n - 2) i = n - 2;
    w = __ddiv_rn(__dsub_rn(t, g[i]), __dsub_rn(g[i + 1], g[i]));
    return !(t < g[0] || t > g[n - 1]);
}

// Bilinear value with the term order of the FP64 history regrid.
__device__ __forceinline__ double rgi_value(const double *__restrict__ f, int nz, int i, int j, double y0,
                                            double y1) {
    const double u0 = __dsub_rn(1.0, y0), u1 = __dsub_rn(1.0, y1);
    const size_t k00 = (size_t)i * nz + j;
    double r = 0.0;
    r = __dadd_rn(r, __dmul_rn(__dmul_rn(f[k00], u0), u1));
    r = __dadd_rn(r, __dmul_rn(__dmul_rn(f[k00 + 1], u0), y1));
    r = __dadd_rn(r, __dmul_rn(__dmul_rn(f[k00 + nz], y0), u1));
    r = __dadd_rn(r, __dmul_rn(__dmul_rn(f[k00 + nz + 1], y0), y1));
    return r;
}

__global__ void __launch_bounds__(256)
apply_kicks(double *__restrict__ p, int64_t n, int64_t ld, const double *__restrict__ tables,
            int64_t cells, int transverse, const double *__restrict__ xrange,
            const double *__restrict__ zrange, int nx, int nz, double slope0, double slope1) {
    extern __shared__ double grids[];
    double *gx = grids, *gz = grids + nx;
    for (int k = threadIdx.x; k < nx; k += blockDim.x) gx[k] = xrange[k];
    for (int k = threadIdx.x; k < nz; k += blockDim.x) gz[k] = zrange[k];
    __syncthreads();
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n) return;
    const double x = p[idx], z = p[4 * ld + idx];
    // x_transform = x - polyval([slope0, slope1], z)  (beams.py:207-211)
    const double xt = __dsub_rn(x, __dadd_rn(__dmul_rn(slope0, z), slope1));
    int i, j;
    double y0, y1;
    const bool in_x = rgi_lookup(gx, nx, xt, i, y0);
    const bool in_z = rgi_lookup(gz, nz, z, j, y1);
    const bool in = in_x && in_z;
    const double dpz = in ? rgi_value(tables, nz, i, j, y0, y1) : 0.0;
    p[5 * ld + idx] = __dadd_rn(p[5 * ld + idx], dpz);
    if (transverse) {
        const double dpx = in ? rgi_value(tables + cells, nz, i, j, y0, y1) : 0.0;
        p[ld + idx] = __dadd_rn(p[ld + idx], dpx);
    }
}

}  // namespace dfcsr

using namespace dfcsr;

extern "C" int dfcsr_transport6(const double *R, double *coords, int64_t n, int64_t ld, void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(n >= 0 && ld >= n, "dfcsr_transport6: need 0 <= n <= ld");
    if (n == 0) return DFCSR_OK;
    DFCSR_CHECK_ARG(R && coords, "dfcsr_transport6: null pointer");
    Matrix6 M;
    for (int k = 0; k < 36; ++k) M.m[k] = R[k];
    ScopedTiming tm("transport6", as_stream(stream));
    note_launch();
    transport6<<<(unsigned)((n + 255) / 256), 256, 0, as_stream(stream)>>>(M, coords, n, ld);
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}

extern "C" size_t dfcsr_apply_wakes_workspace_bytes(int nx, int nz) {
    if (nx < 2 || nz < 2) return 0;
    return (size_t)2 * nx * nz * sizeof(double) + 256;
}

extern "C" int dfcsr_apply_wakes(double *coords, int64_t n, int64_t ld, const double *dE_dct,
                                 const double *x_kick, const double *xrange, const double *zrange,
                                 int nx, int nz, double slope0, double slope1, double step_size,
                                 double init_energy, int transverse_on, void *workspace,
                                 size_t workspace_bytes, void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(n >= 0 && ld >= n, "dfcsr_apply_wakes: need 0 <= n <= ld");
    DFCSR_CHECK_ARG(nx >= 2 && nz >= 2 && nx + nz <= 6144,
                    "dfcsr_apply_wakes: mesh sides must be >= 2 and sum to <= 6144 (got %d, %d)", nx, nz);
    if (n == 0) return DFCSR_OK;
    DFCSR_CHECK_ARG(coords && dE_dct && xrange && zrange, "dfcsr_apply_wakes: null pointer");
    DFCSR_CHECK_ARG(!transverse_on || x_kick, "dfcsr_apply_wakes: transverse_on needs x_kick");
    const int64_t cells = (int64_t)nx * nz;
    if (!workspace || workspace_bytes < (size_t)2 * cells * sizeof(double)) {
        set_error("dfcsr_apply_wakes: workspace too small (%zu < %zu)", workspace_bytes,
                  (size_t)2 * cells * sizeof(double));
        return DFCSR_OOM;
    }
    cudaStream_t st = as_stream(stream);
    double *tables = reinterpret_cast<double *>(workspace);
    ScopedTiming tm("apply_wakes", st);
    note_launch();
    scale_kicks<<<(unsigned)((cells + 255) / 256), 256, 0, st>>>(
        dE_dct, transverse_on ? x_kick : nullptr, cells, step_size, init_energy, tables);
    const size_t smem = (size_t)(nx + nz) * sizeof(double);
    note_launch();
    apply_kicks<<<(unsigned)((n + 255) / 256), 256, smem, st>>>(
        coords, n, ld, tables, cells, transverse_on ? 1 : 0, xrange, zrange, nx, nz, slope0, slope1);
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}
