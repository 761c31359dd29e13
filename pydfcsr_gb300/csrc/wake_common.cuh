// Device helpers shared by the FP64 and mixed-precision CSR wake kernels:
// lattice-table lookups (interpolate1D, pyDFCSR_2D/interp1D.py:13-36), the
// history lookup (interpolate3D, pyDFCSR_2D/interp3D.py:18-66) over the device
// ring, and the integration-region bounds of get_CSR_wake
// (pyDFCSR_2D/CSR.py:454-553).
#pragma once
#include "dfcsr_common.cuh"

namespace dfcsr {

constexpr int WAKE_MAX_REGIONS = 4;

struct Region {
    int nxp, nsp;
    double xl, xr, sl, sr;
};

// np.max((0, v)): NaN propagates, otherwise max(0, v)
__device__ __forceinline__ double np_max0(double v) { return (v != v) ? v : (0.0 >= v ? 0.0 : v); }

// get_CSR_wake region bounds (CSR.py:478-553), same operation order.
__device__ inline int wake_regions(const dfcsr_wake_job &J, double s, double x, Region *reg) {
    const double t = J.position, sz = J.sigma_z, sx = J.sigma_x, tt = J.slope0;
    const double x0 = (s - t) * tt;
    const int zb = J.zbins, xb = J.xbins;
    if (fabs(tt) <= 1.0) {
        const double s2 = s - 500 * sz, s3 = s - 20 * sz, s4 = s + 5 * sz;
        const double s1 = np_max0(s2 - J.n_formation_length * J.formation_length);
        reg[0] = Region{2 * xb, zb, x0 - 20 * sx, x0 + 20 * sx, s1, s2};
        reg[1] = Region{xb, zb, x0 - 10 * sx, x0 + 10 * sx, s2, s3};
        reg[2] = Region{xb, zb, x0 - 10 * sx, x0 + 10 * sx, s3, s4};
        return 3;
    }
    double s2, s3, s4, x1l, x1r, x2l, x2r;
    if (tt > 0) {
        const double ta = -2 * tt / (1 - tt * tt);
        const double d = (10 * sx + J.mean_x - x) / ta;
        s4 = s + 3 * sz;
        s3 = np_max0(s - d);
        s2 = s3 - 200 * sz;
        x1l = x + 0.1 * sx; x1r = x + 10 * sx;
        x2l = x - 3 * sx;   x2r = x1l;
    } else {
        const double ta = 2 * tt / (1 - tt * tt);
        const double d = -(J.mean_x - x - 10 * sx) / ta;
        s4 = s + 3 * sz;
        s3 = np_max0(s - d);
        s2 = s3 - 200 * sz;
        x1l = x - 10 * sx; x1r = x - 1 * sx;
        x2l = x1r;         x2r = x + 3 * sx;
    }
    const double s1 = np_max0(s2 - J.n_formation_length * J.formation_length);
    reg[0] = Region{2 * xb, zb, x0 - 20 * sx, x0 + 20 * sx, s1, s2};
    reg[1] = Region{xb, zb, x0 - 5 * sx, x0 + 5 * sx, s2, s3};
    reg[2] = Region{xb, zb, x1l, x1r, s3, s4};
    reg[3] = Region{xb, zb, x2l, x2r, s3, s4};
    return 4;
}

// Six reference-orbit tables at s (X0, Y0, nX, nY, tauX, tauY): one
// interpolate1D each, sharing the index computation.
__device__ __forceinline__ void lattice_lerp(const dfcsr_wake_job &J, double s, double out[6]) {
    const double u = (s - J.s_min) / J.s_delta;
    int a, b;
    double f;
    if (!axis_index(u, J.nsample, a, b, f)) {
#pragma unroll
        for (int k = 0; k < 6; ++k) out[k] = 0.0;
        return;
    }
    if (!(bounds_ok(a, J.nsample, BS_ORBIT) && bounds_ok(b, J.nsample, BS_ORBIT))) {
#pragma unroll
        for (int k = 0; k < 6; ++k) out[k] = 0.0;
        return;
    }
    const double *pa = J.lattice + (size_t)a * 6, *pb = J.lattice + (size_t)b * 6;
#pragma unroll
    for (int k = 0; k < 6; ++k) out[k] = pa[k] * (1 - f) + pb[k] * f;
}

// Curvature at s' (CSR.py:651-656): rho[e] for distance[e-1] <= s' < distance[e]
// (first element: s' < distance[0]); 0 beyond the last element.
__device__ __forceinline__ double rho_at(const dfcsr_wake_job &J, double sp) {
    double r = 0.0;
    for (int e = 0; e < J.nelement; ++e) {
        if (e == 0) {
            if (sp < J.distance[0]) r = J.rho[0];
        } else if (sp < J.distance[e] && sp >= J.distance[e - 1]) {
            r = J.rho[e];
        }
    }
    return r;
}

// One field of an FP32 ring cell as a double: density_x and vx are stored as
// hi + lo (low parts in slots 5 and 6 of the 8-float cell).
__device__ __forceinline__ double ring32_value(const float *ring32, size_t cell, int field) {
    const float *c = ring32 + cell * 8;
    double v = (double)c[field];
    if (field == 1) v += (double)c[5];
    else if (field == 3) v += (double)c[6];
    return v;
}

__device__ __forceinline__ int ring_slot(const dfcsr_wake_job &J, int t) {
    int s = J.head + t;
    if (s >= J.cap) s -= J.cap;
    return s;
}

// Checked build: the ring coordinates of a trilinear gather inside the ring
// (slots < cap, x < nx, z < nz).
__device__ __forceinline__ bool ring_cells_ok(const dfcsr_wake_job &J, int s0, int s1, int x0, int x1,
                                              int z0, int z1) {
    return bounds_ok(s0, J.cap, BS_FP64_RING) && bounds_ok(s1, J.cap, BS_FP64_RING) &&
           bounds_ok(x0, J.nx, BS_FP64_RING) && bounds_ok(x1, J.nx, BS_FP64_RING) &&
           bounds_ok(z0, J.nz, BS_FP64_RING) && bounds_ok(z1, J.nz, BS_FP64_RING);
}

// interpolate3D of one field of the history at (t, x, z), FP64 arithmetic,
// reading the FP64 ring when present, else the FP32 ring.
__device__ inline double hist_field_fp64(const dfcsr_wake_job &J, int field, double t, double x, double z) {
    int t0, t1, x0, x1, z0, z1;
    double td, xd, zd;
    if (!axis_index((t - J.t_min) / J.t_delta, J.nt, t0, t1, td) ||
        !axis_index((x - J.x_min) / J.x_delta, J.nx, x0, x1, xd) ||
        !axis_index((z - J.z_min) / J.z_delta, J.nz, z0, z1, zd))
        return 0.0;
    const int s0 = ring_slot(J, t0), s1 = ring_slot(J, t1);
    if (!ring_cells_ok(J, s0, s1, x0, x1, z0, z1)) return 0.0;
    auto D = [&](int s, int xi, int zi) -> double {
        const size_t cell = ((size_t)s * J.nx + xi) * J.nz + zi;
        return J.ring64 ? J.ring64[cell * 5 + field] : ring32_value(J.ring32, cell, field);
    };
    const double c00 = D(s0, x0, z0) * (1 - td) + D(s1, x0, z0) * td;
    const double c01 = D(s0, x0, z1) * (1 - td) + D(s1, x0, z1) * td;
    const double c10 = D(s0, x1, z0) * (1 - td) + D(s1, x1, z0) * td;
    const double c11 = D(s0, x1, z1) * (1 - td) + D(s1, x1, z1) * td;
    const double c0 = c00 * (1 - xd) + c10 * xd;
    const double c1 = c01 * (1 - xd) + c11 * xd;
    return c0 * (1 - zd) + c1 * zd;
}

// interpolate3D of all five fields at (t, x, z) in FP64 arithmetic (same
// operation order as the reference), from the FP64 ring when present, else
// from the FP32 ring.  Out of range: all zero.
__device__ __forceinline__ void gather5_fp64(const dfcsr_wake_job &J, double t, double x, double z,
                                             double v[5]) {
    int t0, t1, x0, x1, z0, z1;
    double td, xd, zd;
#pragma unroll
    for (int f = 0; f < 5; ++f) v[f] = 0.0;
    if (!axis_index((t - J.t_min) / J.t_delta, J.nt, t0, t1, td) ||
        !axis_index((x - J.x_min) / J.x_delta, J.nx, x0, x1, xd) ||
        !axis_index((z - J.z_min) / J.z_delta, J.nz, z0, z1, zd))
        return;
    const int s0 = ring_slot(J, t0), s1 = ring_slot(J, t1);
    if (!ring_cells_ok(J, s0, s1, x0, x1, z0, z1)) return;
    const size_t nz = J.nz, nxz = (size_t)J.nx * J.nz;
    const size_t c[8] = {(size_t)s0 * nxz + (size_t)x0 * nz + z0, (size_t)s1 * nxz + (size_t)x0 * nz + z0,
                         (size_t)s0 * nxz + (size_t)x0 * nz + z1, (size_t)s1 * nxz + (size_t)x0 * nz + z1,
                         (size_t)s0 * nxz + (size_t)x1 * nz + z0, (size_t)s1 * nxz + (size_t)x1 * nz + z0,
                         (size_t)s0 * nxz + (size_t)x1 * nz + z1, (size_t)s1 * nxz + (size_t)x1 * nz + z1};
#pragma unroll
    for (int f = 0; f < 5; ++f) {
        double d[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            d[k] = J.ring64 ? J.ring64[c[k] * 5 + f] : ring32_value(J.ring32, c[k], f);
        const double c00 = d[0] * (1 - td) + d[1] * td;
        const double c01 = d[2] * (1 - td) + d[3] * td;
        const double c10 = d[4] * (1 - td) + d[5] * td;
        const double c11 = d[6] * (1 - td) + d[7] * td;
        const double c0 = c00 * (1 - xd) + c10 * xd;
        const double c1 = c01 * (1 - xd) + c11 * xd;
        v[f] = c0 * (1 - zd) + c1 * zd;
    }
}

struct ObsConst {
    double t, s, x, vx, X0s, Y0s, nsx, nsy, tsx, tsy;
};

// get_CSR_integrand (CSR.py:605-782) at one (x', s') point; lat_sp holds
// the six table values at s'.
__device__ __forceinline__ void integrand_fp64(const dfcsr_wake_job &J, const ObsConst &o,
                                               const double lat_sp[6], double rho_sp, double spj,
                                               double xpi, double &Iz, double &Ix,
                                               bool ignore_vx = false) {
    const double X0_sp = lat_sp[0], Y0_sp = lat_sp[1];
    const double npx = lat_sp[2], npy = lat_sp[3], tpx = lat_sp[4], tpy = lat_sp[5];
    const double rx = o.X0s - X0_sp + o.x * o.nsx - xpi * npx;
    const double ry = o.Y0s - Y0_sp + o.x * o.nsy - xpi * npy;
    const double r = sqrt(rx * rx + ry * ry);
    const double t_ret = o.t - r;
    const double zq = spj - t_ret;
    // five fields at (t_ret, x', s' - t_ret)
    double v[5];
    gather5_fp64(J, t_ret, xpi, zq, v);
    const double den = v[0], den_x = v[1], den_z = v[2];
    const double vx_r = ignore_vx ? 0.0 : v[3], vx_x_r = ignore_vx ? 0.0 : v[4];
    const double ovx = ignore_vx ? 0.0 : o.vx;
    const double scale = 1 + xpi * rho_sp;
    const double vel_x = o.tsx + ovx * o.nsx;
    const double vel_y = o.tsy + ovx * o.nsy;
    const double velr_x = tpx + vx_r * npx;
    const double velr_y = tpy + vx_r * npy;
    const double nab_x = den_x * npx + den_z / scale * tpx;
    const double nab_y = den_x * npy + den_z / scale * tpy;
    const double div_v = vx_x_r;
    const double p1 = vel_x * velr_x + vel_y * velr_y;
    const double num1 = scale * ((vel_x - p1 * velr_x) * nab_x + (vel_y - p1 * velr_y) * nab_y);
    const double num2 = -scale * p1 * den * div_v;
    Iz = num1 / r + num2 / r;
    const double nmx = o.nsx - npx, nmy = o.nsy - npy;
    const double q1 = rx * nmx + ry * nmy;
    const double q2 = o.nsx * tpx + o.nsy * tpy;
    const double pd = -(velr_x * nab_x + velr_y * nab_y) - den * div_v;
    const double W1 = scale * q1 / (r * r * r) * den;
    const double W2 = scale * q1 / (r * r) * pd;
    const double W3 = -scale * q2 / r * pd;
    Ix = W1 + W2 + W3;
}

}  // namespace dfcsr
