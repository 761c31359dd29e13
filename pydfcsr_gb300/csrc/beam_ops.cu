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
    unsigned long long nonzero;   // bit 6 r + k set iff m[6 r + k] != 0 (host-computed)
};

// y_r = sum_k R[r][k] x_k as a fused multiply-add chain in increasing k,
// starting from the first non-zero coefficient; zero coefficients are
// skipped.  Which coefficients are zero is an integer mask from the host, so
// the skip costs an integer test instead of an FP64 compare per coefficient
// and thread (GB300's FP64 pipe issues at 1/72 of the FP32 rate, and 36 such
// compares cost twice the chain itself).
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
            if ((R.nonzero >> (r * 6 + k)) & 1ull) {
                const double c = R.m[r * 6 + k];
                acc = first ? __dmul_rn(c, x[k]) : __fma_rn(c, x[k], acc);
                first = false;
            }
        }
        p[r * ld + i] = acc;
    }
}

// Scaled kick tables: kick = ((step * wake) * 1e6) / energy, the order of
// `step_size * dE_dct * 1e6 / self.init_energy` (beams.py:110, 120); and the
// interval tables of both axes: width b[i] = g[i+1] - g[i] (the
// interpolator's denominator) and its correctly rounded reciprocal.
__global__ void scale_kicks(const double *__restrict__ dE, const double *__restrict__ xk, int64_t cells,
                            double step, double energy, const double *__restrict__ xg, int nx,
                            const double *__restrict__ zg, int nz, double *__restrict__ out,
                            double2 *__restrict__ axes) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < cells) {
        out[t] = __ddiv_rn(__dmul_rn(__dmul_rn(step, dE[t]), 1e6), energy);
        if (xk) out[cells + t] = __ddiv_rn(__dmul_rn(__dmul_rn(step, xk[t]), 1e6), energy);
    }
    if (t < (int64_t)(nx - 1) + (nz - 1)) {
        const bool onx = t < nx - 1;
        const double *g = onx ? xg : zg;
        const int i = onx ? (int)t : (int)(t - (nx - 1));
        const double b = __dsub_rn(g[i + 1], g[i]);
        axes[t] = make_double2(b, __drcp_rn(b));
    }
}

// Total-order key of an FP64 value for integer comparisons: for any two
// non-NaN values, key(a) <= key(b) iff a <= b (-0 is mapped to +0, which
// IEEE compares equal).  A positive NaN keys above every number.
__device__ __forceinline__ long long order_key(double v) {
    long long b = __double_as_longlong(v);
    if (b == (long long)0x8000000000000000ull) b = 0;
    return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}

__device__ __forceinline__ bool is_nan_bits(double v) {
    return (__double_as_longlong(v) & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
}

// RegularGridInterpolator axis lookup (linear, bounds_error=False): the
// interval i = clip(searchsorted(grid, t, 'right') - 1, 0, n - 2), the
// normalised distance (t - g[i]) / (g[i+1] - g[i]) and the out-of-bounds test
// t < g[0] or t > g[n-1] (false for NaN, as numpy's comparisons).
//
// The search compares integer order keys (no FP64 compares).  The distance
// is the correctly rounded quotient a / b from the reciprocal y = RN(1/b):
// q0 = RN(a y), r = a - b q0 (exact by FMA), q = RN(q0 + r y).  Markstein's
// theorem (y within half an ulp of 1/b, q0 within one ulp of a/b) makes q
// equal RN(a / b) in round-to-nearest, away from underflow; a is a distance
// within one interval of a grid of normal numbers (or exactly 0), so the
// weight equals the reference's division bit for bit at 4 FP64 operations
// instead of a full division.
__device__ __forceinline__ bool rgi_lookup(const double *g, const double2 *__restrict__ ax, int n,
                                           double t, int &i, double &w) {
    const long long kt = order_key(t);
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (order_key(g[mid]) <= kt) lo = mid + 1;
        else hi = mid;
    }
    i = lo - 1;
    if (i < 0) i = 0;
    if (i > n - 2) i = n - 2;
    const double2 by = __ldg(ax + i);
    const double a = __dsub_rn(t, g[i]);
    const double q0 = __dmul_rn(a, by.y);
    const double r = __fma_rn(-q0, by.x, a);
    w = __fma_rn(r, by.y, q0);
    if (is_nan_bits(t)) return true;
    return !(kt < order_key(g[0]) || kt > order_key(g[n - 1]));
}

// Bilinear value with the term order of the FP64 history regrid.
__device__ __forceinline__ double rgi_value(const double *__restrict__ f, int nz, int i, int j, double u0,
                                            double u1, double y0, double y1) {
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
            const double *__restrict__ zrange, const double2 *__restrict__ axes, int nx, int nz,
            double slope0, double slope1) {
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
    const bool in_x = rgi_lookup(gx, axes, nx, xt, i, y0);
    const bool in_z = rgi_lookup(gz, axes + (nx - 1), nz, z, j, y1);
    const bool in = in_x && in_z && bounds_ok(i, nx - 1, BS_KICK) && bounds_ok(j, nz - 1, BS_KICK);
    const double u0 = __dsub_rn(1.0, y0), u1 = __dsub_rn(1.0, y1);
    const double dpz = in ? rgi_value(tables, nz, i, j, u0, u1, y0, y1) : 0.0;
    p[5 * ld + idx] = __dadd_rn(p[5 * ld + idx], dpz);
    if (transverse) {
        const double dpx = in ? rgi_value(tables + cells, nz, i, j, u0, u1, y0, y1) : 0.0;
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
    M.nonzero = 0;
    for (int k = 0; k < 36; ++k) {
        M.m[k] = R[k];
        if (R[k] != 0.0) M.nonzero |= 1ull << k;
    }
    ScopedTiming tm("transport6", as_stream(stream));
    note_launch();
    transport6<<<(unsigned)((n + 255) / 256), 256, 0, as_stream(stream)>>>(M, coords, n, ld);
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}

// Workspace: the two scaled kick tables, then the interval tables of both
// axes (width and reciprocal per interval).
static size_t kick_tables_bytes(int nx, int nz) { return (size_t)2 * nx * nz * sizeof(double); }
static size_t kick_axes_bytes(int nx, int nz) { return (size_t)(nx - 1 + nz - 1) * sizeof(double2); }

extern "C" size_t dfcsr_apply_wakes_workspace_bytes(int nx, int nz) {
    if (nx < 2 || nz < 2) return 0;
    return kick_tables_bytes(nx, nz) + kick_axes_bytes(nx, nz) + 256;
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
    const size_t need = kick_tables_bytes(nx, nz) + kick_axes_bytes(nx, nz);
    if (!workspace || workspace_bytes < need) {
        set_error("dfcsr_apply_wakes: workspace too small (%zu < %zu)", workspace_bytes, need);
        return DFCSR_OOM;
    }
    DFCSR_CHECK_ARG(((uintptr_t)workspace % 16) == 0, "dfcsr_apply_wakes: workspace must be 16-byte aligned");
    cudaStream_t st = as_stream(stream);
    double *tables = reinterpret_cast<double *>(workspace);
    double2 *axes = reinterpret_cast<double2 *>(static_cast<char *>(workspace) + kick_tables_bytes(nx, nz));
    ScopedTiming tm("apply_wakes", st);
    const int64_t prep = cells > (int64_t)(nx + nz) ? cells : (int64_t)(nx + nz);
    note_launch();
    scale_kicks<<<(unsigned)((prep + 255) / 256), 256, 0, st>>>(
        dE_dct, transverse_on ? x_kick : nullptr, cells, step_size, init_energy, xrange, nx, zrange,
        nz, tables, axes);
    const size_t smem = (size_t)(nx + nz) * sizeof(double);
    note_launch();
    apply_kicks<<<(unsigned)((n + 255) / 256), 256, smem, st>>>(
        coords, n, ld, tables, cells, transverse_on ? 1 : 0, xrange, zrange, axes, nx, nz, slope0,
        slope1);
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}

DFCSR_BOUNDS_READER(beam_ops)
