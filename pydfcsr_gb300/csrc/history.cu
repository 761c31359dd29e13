// History ring regrid: the device side of DF_interp / append_interpolant
// (pyDFCSR_2D/deposit.py:296-392).
//
// scipy RegularGridInterpolator (linear, bounds_error=False) evaluated on the
// tensor-product interpolation grid: the host computes, per target x and per
// target z, the source interval l with g[l] <= v < g[l+1] (last interval at
// the right end point), the normalised distance and the out-of-bounds flag;
// the kernel forms the bilinear sum in scipy's term order
//   v[i,j](1-y0)(1-y1) + v[i,j+1](1-y0)y1 + v[i+1,j]y0(1-y1) + v[i+1,j+1]y0 y1
// and writes the five fields interleaved into one ring slot (FP64 and/or
// FP32 copy).  Out-of-bounds targets take the fill value (0, or the mean of
// vx_x for vx_x).
#include "dfcsr_common.cuh"

namespace dfcsr {

// EXACT: RegularGridInterpolator's term order with every product rounded
// (the FP64 ring of the drop-in).  Otherwise (FP32 ring only) the four
// bilinear weights are formed once and each field is one multiply and three
// fused multiply-adds in FP64 - well inside the FP32 cell's resolution, and
// density_x keeps the ~1e-16 relative accuracy its hi + lo pair carries.
template <bool EXACT>
__global__ void regrid5(const double *__restrict__ f0, const double *__restrict__ f1,
                        const double *__restrict__ f2, const double *__restrict__ f3,
                        const double *__restrict__ f4, int snx, int snz,
                        const int32_t *__restrict__ ix, const double *__restrict__ wx,
                        const uint8_t *__restrict__ oobx, int nxi,
                        const int32_t *__restrict__ iz, const double *__restrict__ wz,
                        const uint8_t *__restrict__ oobz, int nzi,
                        const double *__restrict__ fill4, double *__restrict__ out64,
                        float *__restrict__ out32) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nxi * nzi) return;
    const int a = (int)(t / nzi), c = (int)(t % nzi);
    double v[5];
    if (oobx[a] || oobz[c]) {
        v[0] = v[1] = v[2] = v[3] = 0.0;
        v[4] = *fill4;
    } else {
        const int i = ix[a], j = iz[c];
        if (!(bounds_ok(i, snx - 1, BS_REGRID) && bounds_ok(j, snz - 1, BS_REGRID))) return;
        const double y0 = wx[a], y1 = wz[c];
        const double u0 = 1.0 - y0, u1 = 1.0 - y1;
        const size_t k00 = (size_t)i * snz + j, k01 = k00 + 1, k10 = k00 + snz, k11 = k10 + 1;
        const double *F[5] = {f0, f1, f2, f3, f4};
        if (EXACT) {
#pragma unroll
            for (int q = 0; q < 5; ++q) {
                const double *p = F[q];
                double r = 0.0;
                r = __dadd_rn(r, __dmul_rn(__dmul_rn(p[k00], u0), u1));
                r = __dadd_rn(r, __dmul_rn(__dmul_rn(p[k01], u0), y1));
                r = __dadd_rn(r, __dmul_rn(__dmul_rn(p[k10], y0), u1));
                r = __dadd_rn(r, __dmul_rn(__dmul_rn(p[k11], y0), y1));
                v[q] = r;
            }
        } else {
            const double w00 = u0 * u1, w01 = u0 * y1, w10 = y0 * u1, w11 = y0 * y1;
#pragma unroll
            for (int q = 0; q < 5; ++q) {
                const double *p = F[q];
                v[q] = fma(p[k11], w11, fma(p[k10], w10, fma(p[k01], w01, p[k00] * w00)));
            }
        }
    }
    if (out64) {
        double *o = out64 + (size_t)t * 5;
#pragma unroll
        for (int q = 0; q < 5; ++q) o[q] = v[q];
    }
    if (out32) {
        // FP32 cell: density, density_x (high part), density_z, vx (high
        // part) | vx_x, density_x low part (v - (double)hi), vx low part, 0.
        // density_x and vx are carried as float-float pairs: the wake's
        // density_x term sums to ~1/300 of its terms, and vx enters it through
        // b - vx (..), where the two are of similar size after a bend.
        float4 *o = reinterpret_cast<float4 *>(out32 + (size_t)t * 8);
        const float hi = (float)v[1];
        const float lo = (float)(v[1] - (double)hi);
        const float vhi = (float)v[3];
        const float vlo = (float)(v[3] - (double)vhi);
        o[0] = make_float4((float)v[0], hi, (float)v[2], vhi);
        o[1] = make_float4((float)v[4], lo, vlo, 0.f);
    }
}

// RegularGridInterpolator axis tables for a source grid and a target grid
// that are both numpy linspaces: i = clip(searchsorted(src, t, 'right') - 1,
// 0, ns - 2), w = (t - src[i]) / (src[i+1] - src[i]), oob = t < src[0] or
// t > src[ns-1].  Grid values are regenerated with numpy's linspace formula,
// so the tables equal the ones computed from the host arrays.  The interval
// is guessed from (t - src[0]) / step and then corrected by exact
// comparisons with the grid values (two or three steps instead of a binary
// search: every FP64 operation here costs some hundred cycles of latency).
struct Linspace {   // numpy.linspace(start, stop, num) element by element
    double start, stop, delta, step;
    int num;
    __device__ Linspace(double a, double b, int n) : start(a), stop(b), num(n) {
        const int div = n - 1;
        delta = __dsub_rn(b, a);
        step = div > 0 ? __ddiv_rn(delta, (double)div) : 0.0;
    }
    __device__ double at(int i) const {
        if (num == 1) return start;
        if (i == num - 1) return stop;
        if (step == 0.0) return __dadd_rn(__dmul_rn(__ddiv_rn((double)i, (double)(num - 1)), delta), start);
        return __dadd_rn(__dmul_rn((double)i, step), start);
    }
};

__global__ void rgi_axis_linspace(double s0, double s1, int ns, double t0, double t1, int nt,
                                  int32_t *__restrict__ idx, double *__restrict__ w,
                                  uint8_t *__restrict__ oob) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nt) return;
    const Linspace src(s0, s1, ns);
    const double t = Linspace(t0, t1, nt).at(m);
    // g = (number of source values <= t) - 1, from a guess within a step or
    // two of it; NaN -> -1 (no value compares <= NaN)
    int g = -1;
    if (t == t) {
        double gd = floor(__dmul_rn(__dsub_rn(t, s0), __drcp_rn(src.step)));
        if (!(gd >= -1.0)) gd = -1.0;
        if (gd > (double)(ns - 1)) gd = (double)(ns - 1);
        g = (int)gd;
        while (g + 1 < ns && src.at(g + 1) <= t) ++g;
        while (g >= 0 && src.at(g) > t) --g;
    }
    int i = g;
    if (i < 0) i = 0;
    if (i > ns - 2) i = ns - 2;
    const double a = src.at(i), b = src.at(i + 1);
    idx[m] = i;
    w[m] = __ddiv_rn(__dsub_rn(t, a), __dsub_rn(b, a));
    oob[m] = (t < src.at(0) || t > src.at(ns - 1)) ? 1 : 0;
}

// get_DF's per-step axis tables (deposit.py:170-171, 212-213) from the grid
// linspaces: diff(grid) and the coefficients numpy.gradient applies with a
// coordinate array (edge_order 1) - per interior index a = -d2 / (d1 (d1 +
// d2)), b = (d2 - d1) / (d1 d2), c = d1 / (d2 (d1 + d2)) with d1, d2 the
// spacings below and above it; row 3 holds the first and last spacing (the
// first twice when numpy takes its uniform-spacing branch).  Grid values by
// numpy's linspace formula and the operations in numpy's order, so the
// tables equal the host's bit for bit.  Thread t < nx handles x index t,
// the next nz threads the z indices.
__global__ void df_axis_tables(double x0, double x1, int nx, double z0, double z1, int nz,
                               int x_uniform, int z_uniform, double *__restrict__ gx,
                               double *__restrict__ gz, double *__restrict__ dxg,
                               double *__restrict__ dzg) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nx + nz) return;
    const bool onx = t < nx;
    const Linspace L = onx ? Linspace(x0, x1, nx) : Linspace(z0, z1, nz);
    const int n = onx ? nx : nz;
    const int i = onx ? t : t - nx;
    double *g = onx ? gx : gz;
    double *d = onx ? dxg : dzg;
    const int uniform = onx ? x_uniform : z_uniform;
    const double gi = L.at(i);
    if (i + 1 < n) d[i] = __dsub_rn(L.at(i + 1), gi);
    double a = 0.0, b = 0.0, c = 0.0;
    if (i >= 1 && i + 1 < n) {
        const double d1 = __dsub_rn(gi, L.at(i - 1)), d2 = __dsub_rn(L.at(i + 1), gi);
        const double s12 = __dadd_rn(d1, d2);
        a = __ddiv_rn(-d2, __dmul_rn(d1, s12));
        b = __ddiv_rn(__dsub_rn(d2, d1), __dmul_rn(d1, d2));
        c = __ddiv_rn(d1, __dmul_rn(d2, s12));
    }
    g[i] = a;
    g[n + i] = b;
    g[2 * n + i] = c;
    double r3 = 0.0;
    if (n >= 2) {
        const double first = __dsub_rn(L.at(1), L.at(0));
        const double last = __dsub_rn(L.at(n - 1), L.at(n - 2));
        if (i == 0) r3 = first;
        else if (i == 1) r3 = uniform ? first : last;
    }
    g[3 * n + i] = r3;
}

}  // namespace dfcsr

using namespace dfcsr;

// Longest grid axis the table entry points accept (keeps their launch sizes
// in int range; DF and history grids are a few thousand points at most).
static constexpr int kMaxAxisPoints = 1 << 24;

extern "C" int dfcsr_rgi_axis_linspace(double src_start, double src_stop, int nsrc,
                                       double tgt_start, double tgt_stop, int ntgt, int32_t *idx,
                                       double *w, uint8_t *oob, void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(nsrc >= 2 && ntgt >= 1, "dfcsr_rgi_axis_linspace: need nsrc >= 2, ntgt >= 1");
    DFCSR_CHECK_ARG(nsrc <= kMaxAxisPoints && ntgt <= kMaxAxisPoints,
                    "dfcsr_rgi_axis_linspace: axes longer than %d points", kMaxAxisPoints);
    DFCSR_CHECK_ARG(idx && w && oob, "dfcsr_rgi_axis_linspace: null pointer");
    DFCSR_CHECK_ARG(src_stop > src_start, "dfcsr_rgi_axis_linspace: source grid must ascend");
    note_launch();
    rgi_axis_linspace<<<(unsigned)((ntgt + 127) / 128), 128, 0, as_stream(stream)>>>(
        src_start, src_stop, nsrc, tgt_start, tgt_stop, ntgt, idx, w, oob);
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}

extern "C" int dfcsr_history_regrid(const double *density, const double *density_x,
                                    const double *density_z, const double *vx, const double *vx_x,
                                    int snx, int snz, const int32_t *ix, const double *wx,
                                    const uint8_t *oobx, int nxi, const int32_t *iz,
                                    const double *wz, const uint8_t *oobz, int nzi,
                                    const double *vx_x_fill, double *ring64_slot,
                                    float *ring32_slot, void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(density && density_x && density_z && vx && vx_x && vx_x_fill,
                    "dfcsr_history_regrid: null field pointer");
    DFCSR_CHECK_ARG(ix && wx && oobx && iz && wz && oobz, "dfcsr_history_regrid: null index table");
    DFCSR_CHECK_ARG(snx >= 2 && snz >= 2, "dfcsr_history_regrid: source grid %d x %d too small", snx, snz);
    DFCSR_CHECK_ARG(nxi >= 1 && nzi >= 1, "dfcsr_history_regrid: empty target grid");
    DFCSR_CHECK_ARG(ring64_slot || ring32_slot, "dfcsr_history_regrid: no output ring");
    DFCSR_CHECK_ARG(!ring32_slot || ((uintptr_t)ring32_slot % 32) == 0,
                    "dfcsr_history_regrid: ring32 slot must be 32-byte aligned");
    const int64_t cells = (int64_t)nxi * nzi;
    ScopedTiming tm("history_regrid", as_stream(stream));
    const unsigned blocks = (unsigned)((cells + 255) / 256);
    note_launch();
    if (ring64_slot)
        regrid5<true><<<blocks, 256, 0, as_stream(stream)>>>(
            density, density_x, density_z, vx, vx_x, snx, snz, ix, wx, oobx, nxi, iz, wz, oobz, nzi,
            vx_x_fill, ring64_slot, ring32_slot);
    else
        regrid5<false><<<blocks, 256, 0, as_stream(stream)>>>(
            density, density_x, density_z, vx, vx_x, snx, snz, ix, wx, oobx, nxi, iz, wz, oobz, nzi,
            vx_x_fill, ring64_slot, ring32_slot);
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}

extern "C" int dfcsr_df_axis_tables(double x0, double x1, int nx, double z0, double z1, int nz,
                                    int x_uniform, int z_uniform, double *gx, double *gz,
                                    double *dxg, double *dzg, void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(nx >= 2 && nz >= 2, "dfcsr_df_axis_tables: grids need >= 2 points (%d, %d)", nx, nz);
    DFCSR_CHECK_ARG(nx <= kMaxAxisPoints && nz <= kMaxAxisPoints,
                    "dfcsr_df_axis_tables: grids longer than %d points", kMaxAxisPoints);
    DFCSR_CHECK_ARG(gx && gz && dxg && dzg, "dfcsr_df_axis_tables: null pointer");
    note_launch();
    const int total = nx + nz;
    df_axis_tables<<<(unsigned)((total + 127) / 128), 128, 0, as_stream(stream)>>>(
        x0, x1, nx, z0, z1, nz, x_uniform ? 1 : 0, z_uniform ? 1 : 0, gx, gz, dxg, dzg);
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}

DFCSR_BOUNDS_READER(history)
