// Standalone interpolants with the numba functions' semantics:
// interpolate3D (pyDFCSR_2D/interp3D.py:18-66) and interpolate1D
// (pyDFCSR_2D/interp1D.py:13-36).  Same IEEE operation order; int()
// truncation (a query in (-1, 0) extrapolates from the first cell).
#include "dfcsr_common.cuh"

namespace dfcsr {

__global__ void interp3d_kernel(const double *__restrict__ qt, const double *__restrict__ qx,
                                const double *__restrict__ qz, int64_t m,
                                const double *__restrict__ d, int nt, int nx, int nz,
                                double min_t, double min_x, double min_z, double dt, double dx,
                                double dz, double *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    int t0, t1, x0, x1, z0, z1;
    double td, xd, zd;
    if (!axis_index(__ddiv_rn(__dsub_rn(qt[i], min_t), dt), nt, t0, t1, td) ||
        !axis_index(__ddiv_rn(__dsub_rn(qx[i], min_x), dx), nx, x0, x1, xd) ||
        !axis_index(__ddiv_rn(__dsub_rn(qz[i], min_z), dz), nz, z0, z1, zd)) {
        out[i] = 0.0;
        return;
    }
    if (!(bounds_ok(t1, nt, BS_INTERP) && bounds_ok(x1, nx, BS_INTERP) && bounds_ok(z1, nz, BS_INTERP) &&
          bounds_ok(t0, nt, BS_INTERP) && bounds_ok(x0, nx, BS_INTERP) && bounds_ok(z0, nz, BS_INTERP))) {
        out[i] = 0.0;
        return;
    }
    auto D = [&](int a, int b, int c) { return d[((size_t)a * nx + b) * nz + c]; };
    auto L = [](double p, double q, double w) {
        return __dadd_rn(__dmul_rn(p, __dsub_rn(1.0, w)), __dmul_rn(q, w));
    };
    const double c00 = L(D(t0, x0, z0), D(t1, x0, z0), td);
    const double c01 = L(D(t0, x0, z1), D(t1, x0, z1), td);
    const double c10 = L(D(t0, x1, z0), D(t1, x1, z0), td);
    const double c11 = L(D(t0, x1, z1), D(t1, x1, z1), td);
    const double c0 = L(c00, c10, xd);
    const double c1 = L(c01, c11, xd);
    out[i] = L(c0, c1, zd);
}

__global__ void interp1d_kernel(const double *__restrict__ q, int64_t m, const double *__restrict__ tab,
                                int n, double min_x, double delta_x, double *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    int a, b;
    double f;
    if (!axis_index(__ddiv_rn(__dsub_rn(q[i], min_x), delta_x), n, a, b, f)) {
        out[i] = 0.0;
        return;
    }
    if (!(bounds_ok(a, n, BS_INTERP) && bounds_ok(b, n, BS_INTERP))) {
        out[i] = 0.0;
        return;
    }
    out[i] = __dadd_rn(__dmul_rn(tab[a], __dsub_rn(1.0, f)), __dmul_rn(tab[b], f));
}

// Observation mesh of get_CSR_mesh (CSR.py:361-394) as the points that
// calculate_2D_CSR visits (CSR.py:404-415): point k = i * zbins + j,
// s = position + zrange[j], x = xrange[i] + polyval([slope0, slope1], zrange[j]),
// with numpy's linspace and polyval arithmetic.
__global__ void csr_mesh_kernel(double x0, double x1, int xbins, double z0, double z1, int zbins,
                                double slope0, double slope1, double position,
                                double *__restrict__ s, double *__restrict__ x) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (int64_t)xbins * zbins) return;
    const int i = (int)(k / zbins), j = (int)(k % zbins);
    const double z = np_linspace_at(z0, z1, zbins, j);
    const double xt = np_linspace_at(x0, x1, xbins, i);
    s[k] = __dadd_rn(position, z);
    x[k] = __dadd_rn(xt, __dadd_rn(__dmul_rn(slope0, z), slope1));
}

}  // namespace dfcsr

using namespace dfcsr;

extern "C" int dfcsr_csr_mesh(double x0, double x1, int xbins, double z0, double z1, int zbins,
                              double slope0, double slope1, double position, double *s, double *x,
                              void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(xbins >= 1 && zbins >= 1, "dfcsr_csr_mesh: empty mesh (%d x %d)", xbins, zbins);
    DFCSR_CHECK_ARG(s && x, "dfcsr_csr_mesh: null pointer");
    const int64_t n = (int64_t)xbins * zbins;
    note_launch();
    csr_mesh_kernel<<<(unsigned)((n + 255) / 256), 256, 0, as_stream(stream)>>>(
        x0, x1, xbins, z0, z1, zbins, slope0, slope1, position, s, x);
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}

extern "C" int dfcsr_interp3d(const double *qt, const double *qx, const double *qz, int64_t m,
                              const double *data, int nt, int nx, int nz, double min_t, double min_x,
                              double min_z, double delta_t, double delta_x, double delta_z,
                              double *out, void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(m >= 0, "dfcsr_interp3d: negative query count");
    if (m == 0) return DFCSR_OK;
    DFCSR_CHECK_ARG(qt && qx && qz && data && out, "dfcsr_interp3d: null pointer");
    DFCSR_CHECK_ARG(nt >= 1 && nx >= 1 && nz >= 1, "dfcsr_interp3d: empty grid");
    note_launch();
    interp3d_kernel<<<(unsigned)((m + 255) / 256), 256, 0, as_stream(stream)>>>(
        qt, qx, qz, m, data, nt, nx, nz, min_t, min_x, min_z, delta_t, delta_x, delta_z, out);
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}

extern "C" int dfcsr_interp1d(const double *q, int64_t m, const double *table, int n, double min_x,
                              double delta_x, double *out, void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(m >= 0, "dfcsr_interp1d: negative query count");
    if (m == 0) return DFCSR_OK;
    DFCSR_CHECK_ARG(q && table && out, "dfcsr_interp1d: null pointer");
    DFCSR_CHECK_ARG(n >= 1, "dfcsr_interp1d: empty table");
    note_launch();
    interp1d_kernel<<<(unsigned)((m + 255) / 256), 256, 0, as_stream(stream)>>>(q, m, table, n, min_x,
                                                                                delta_x, out);
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}

DFCSR_BOUNDS_READER(interp)
