// Plain FP64 CSR wake: the drop-in for calculate_2D_CSR / get_CSR_wake /
// get_CSR_integrand (pyDFCSR_2D/CSR.py:397-418, 454-782).
//
// This translation unit is compiled with -fmad=false: every a*b+c rounds twice,
// exactly like numpy's element-wise operations, so the integrand of each
// (x', s') point is bit-identical to the reference's given the same history.
// The trapz reduction also follows numpy's order: one thread owns one s'
// column and sums its x' terms row by row (numpy reduces axis 0 of a C array
// sequentially); the column integrals are then added with numpy's pairwise
// summation.  One CTA evaluates one observation point.
#include <mutex>

#include "wake_common.cuh"

namespace dfcsr {

constexpr int F64_THREADS = 128;
// s' columns per region: up to F64_STATIC_COLS in static shared memory (the
// usual case, three CTAs per SM); up to F64_MAX_COLS in dynamic shared
// memory sized to the call's zbins (4 arrays of 8 B per column).
constexpr int F64_STATIC_COLS = 1024;
constexpr int F64_MAX_COLS = 6144;

template <bool DYN>
__global__ void __launch_bounds__(F64_THREADS)
wake_fp64_kernel(const dfcsr_wake_job *__restrict__ jobs, const int32_t *__restrict__ job_of_point,
                 const double *__restrict__ S, const double *__restrict__ X, int64_t n,
                 int cols_cap, double *__restrict__ dE, double *__restrict__ xkick) {
    __shared__ double s_cols[DYN ? 1 : 4 * F64_STATIC_COLS];
    extern __shared__ double d_cols[];
    double *colz = DYN ? d_cols : s_cols;
    double *colx = colz + cols_cap, *tz = colx + cols_cap, *tx = tz + cols_cap;
    __shared__ double red[2];
    for (int64_t pt = blockIdx.x; pt < n; pt += gridDim.x) {
        const dfcsr_wake_job &J = jobs[job_of_point ? job_of_point[pt] : 0];
        ObsConst o;
        o.t = J.position;
        o.s = S[pt];
        o.x = X[pt];
        o.vx = hist_field_fp64(J, 3, o.t, o.x, o.s - o.t);
        double lat_s[6];
        lattice_lerp(J, o.s, lat_s);
        o.X0s = lat_s[0]; o.Y0s = lat_s[1]; o.nsx = lat_s[2]; o.nsy = lat_s[3];
        o.tsx = lat_s[4]; o.tsy = lat_s[5];
        Region reg[WAKE_MAX_REGIONS];
        const int nreg = wake_regions(J, o.s, o.x, reg);
        double sum_e = 0.0, sum_x = 0.0;
        bool bad = false;
        for (int r = 0; r < nreg; ++r) {
            const Region R = reg[r];
            if (R.nsp < 1 || R.nsp > cols_cap || R.nxp < 1) { bad = true; break; }
            for (int j = threadIdx.x; j < R.nsp; j += blockDim.x) {
                const double spj = np_linspace_at(R.sl, R.sr, R.nsp, j);
                double lat_sp[6];
                lattice_lerp(J, spj, lat_sp);
                const double rho_sp = rho_at(J, spj);
                double az = 0.0, ax = 0.0, pz = 0.0, px = 0.0, xprev = 0.0;
                for (int i = 0; i < R.nxp; ++i) {
                    const double xpi = np_linspace_at(R.xl, R.xr, R.nxp, i);
                    double Iz, Ix;
                    integrand_fp64(J, o, lat_sp, rho_sp, spj, xpi, Iz, Ix);
                    if (i > 0) {
                        const double d = xpi - xprev;
                        const double termz = d * (Iz + pz) / 2.0;
                        const double termx = d * (Ix + px) / 2.0;
                        az = (i == 1) ? termz : az + termz;
                        ax = (i == 1) ? termx : ax + termx;
                    }
                    pz = Iz;
                    px = Ix;
                    xprev = xpi;
                }
                colz[j] = az;
                colx[j] = ax;
            }
            __syncthreads();
            for (int j = threadIdx.x; j < R.nsp - 1; j += blockDim.x) {
                const double ds = np_linspace_at(R.sl, R.sr, R.nsp, j + 1) -
                                  np_linspace_at(R.sl, R.sr, R.nsp, j);
                tz[j] = ds * (colz[j + 1] + colz[j]) / 2.0;
                tx[j] = ds * (colx[j + 1] + colx[j]) / 2.0;
            }
            __syncthreads();
            if (threadIdx.x == 0) red[0] = (R.nsp > 1) ? np_pairwise(tz, R.nsp - 1) : 0.0;
            if (threadIdx.x == 32) red[1] = (R.nsp > 1) ? np_pairwise(tx, R.nsp - 1) : 0.0;
            __syncthreads();
            const double e = -J.csr_scaling * red[0];
            const double k = J.csr_scaling * red[1];
            sum_e = (r == 0) ? e : sum_e + e;
            sum_x = (r == 0) ? k : sum_x + k;
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            dE[pt] = bad ? __longlong_as_double(0x7ff8000000000000ll) : sum_e;
            xkick[pt] = bad ? __longlong_as_double(0x7ff8000000000000ll) : sum_x;
        }
    }
}

// get_CSR_integrand at arbitrary (x', s') points: one thread per point.
__global__ void integrand_points(const dfcsr_wake_job *__restrict__ job, double s, double x,
                                 const double *__restrict__ sp, const double *__restrict__ xp,
                                 int64_t m, int ignore_vx, double *__restrict__ Iz,
                                 double *__restrict__ Ix) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    const dfcsr_wake_job &J = *job;
    ObsConst o;
    o.t = J.position;
    o.s = s;
    o.x = x;
    o.vx = hist_field_fp64(J, 3, o.t, o.x, o.s - o.t);
    double lat_s[6];
    lattice_lerp(J, s, lat_s);
    o.X0s = lat_s[0]; o.Y0s = lat_s[1]; o.nsx = lat_s[2]; o.nsy = lat_s[3];
    o.tsx = lat_s[4]; o.tsy = lat_s[5];
    const double spk = sp[k];
    double lat_sp[6];
    lattice_lerp(J, spk, lat_sp);
    double a, b;
    integrand_fp64(J, o, lat_sp, rho_at(J, spk), spk, xp[k], a, b, ignore_vx != 0);
    Iz[k] = a;
    Ix[k] = b;
}

}  // namespace dfcsr

using namespace dfcsr;

extern "C" int dfcsr_wake_integrand(const dfcsr_wake_job *job, double s, double x, const double *sp,
                                    const double *xp, int64_t m, int ignore_vx, double *Iz,
                                    double *Ix, void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(m >= 0, "dfcsr_wake_integrand: negative point count");
    if (m == 0) return DFCSR_OK;
    DFCSR_CHECK_ARG(job && sp && xp && Iz && Ix, "dfcsr_wake_integrand: null pointer");
    note_launch();
    integrand_points<<<(unsigned)((m + 127) / 128), 128, 0, as_stream(stream)>>>(job, s, x, sp, xp, m,
                                                                                  ignore_vx, Iz, Ix);
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}

extern "C" int dfcsr_wake_fp64(const dfcsr_wake_job *jobs, const int32_t *job_of_point,
                               const double *s, const double *x, int64_t n, int zbins_max,
                               double *dE, double *xkick, void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(n >= 0, "dfcsr_wake_fp64: negative point count");
    if (n == 0) return DFCSR_OK;
    DFCSR_CHECK_ARG(jobs && s && x && dE && xkick, "dfcsr_wake_fp64: null pointer");
    DFCSR_CHECK_ARG(zbins_max >= 1 && zbins_max <= F64_MAX_COLS,
                    "dfcsr_wake_fp64: zbins must be in [1, %d] (got %d)", F64_MAX_COLS, zbins_max);
    cudaStream_t st = as_stream(stream);
    const int64_t grid64 = n < (int64_t)(1 << 30) ? n : (int64_t)(1 << 30);
    ScopedTiming tm("wake_fp64", st);
    note_launch();
    if (zbins_max <= F64_STATIC_COLS) {
        wake_fp64_kernel<false><<<(unsigned)grid64, F64_THREADS, 0, st>>>(
            jobs, job_of_point, s, x, n, F64_STATIC_COLS, dE, xkick);
    } else {
        const size_t smem = (size_t)4 * zbins_max * sizeof(double);
        int dev = 0;
        DFCSR_CUDA_TRY(cudaGetDevice(&dev));
        static std::mutex mu;
        static size_t attr_set[64];
        {
            std::lock_guard<std::mutex> g(mu);
            if (dev < 0 || dev >= 64) {
                set_error("dfcsr_wake_fp64: device ordinal %d out of range", dev);
                return DFCSR_BAD_ARG;
            }
            if (attr_set[dev] < smem) {
                DFCSR_CUDA_TRY(cudaFuncSetAttribute(wake_fp64_kernel<true>,
                                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)((size_t)4 * F64_MAX_COLS * sizeof(double))));
                attr_set[dev] = (size_t)4 * F64_MAX_COLS * sizeof(double);
            }
        }
        wake_fp64_kernel<true><<<(unsigned)grid64, F64_THREADS, smem, st>>>(
            jobs, job_of_point, s, x, n, zbins_max, dE, xkick);
    }
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}

DFCSR_BOUNDS_READER(wake_fp64)
