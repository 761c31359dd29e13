// Mixed-precision CSR wake (FP32 bulk, retarded geometry at ~48 bits or more).
//
// Same integral as get_CSR_wake / get_CSR_integrand (pyDFCSR_2D/CSR.py:454-782),
// restructured so that FP32 is safe and little work is wasted:
//  * set-up kernel (FP64), one small CTA per observation point: regions,
//    record layout, orbit at s, vx at the observer, axes, element
//    thresholds and the double-word per-point constants, written as one
//    record per point.
//  * geometry kernel (double-word FP32 from the job's double-word orbit
//    tables, ~48 bits; FP64 for jobs without them), one CTA per observation
//    point: per s' column the orbit tables at s', the separation R0 = r - r'
//    at a reference x' (the region centre), |R0|, the history coordinates of
//    t_ret and s' - t_ret, and every direction product whose difference would
//    cancel in FP32 (v.tau', v.n', 1 - |tau'|^2, |n'|^2 - 1,
//    (r - r').(n - n'), ...); per x' row the history x cell and the trapz
//    weight, and the range of rows whose x' lies inside the history grid
//    (outside it every field, hence the integrand, is exactly zero, so those
//    rows are skipped).  Records are written for a batch of points (up to
//    1 GiB of records: one batch for a 64^2 mesh).
//  * integral kernel (FP32), a persistent CTA loop over points: per (x', s')
//    only an FP32 correction remains,
//        |r - r'| = r0 + delta,  delta = D / (r0 + sqrt(r0^2 + D)),
//        D = u (|n'|^2 u - 2 R0.n'),  u = x' - x'_ref   (no cancellation);
//    history coordinates are an integer cell plus an FP32 offset, so a grid
//    index near 1000 keeps ~1e-7 cell resolution; the x' axis (index and
//    weight) is resolved once per row; gathers and the integrand are FP32
//    (in the far region density_x, whose x' integral cancels, is read as a
//    stored hi + lo pair and interpolated in offset form so that it is
//    rounded once), Kahan-compensated per-thread sums and a fixed-order
//    block reduction in FP32 double-word.
//  * band kernel (FP64, optional): s' columns with |s' - s| < near_band are
//    skipped by the integral kernel and evaluated with the FP64 integrand.
//  * finalize kernel: adds the regions in the reference's order and scales.
#include <mutex>

#include "dw.cuh"
#include "wake_common.cuh"

namespace dfcsr {

#ifndef MX_INTEGRAL_THREADS
#define MX_INTEGRAL_THREADS 128
#endif
constexpr int MX_THREADS = MX_INTEGRAL_THREADS;
#ifndef MX_INTEGRAL_CHUNK
#define MX_INTEGRAL_CHUNK 128
#endif
constexpr int MX_CHUNK = MX_INTEGRAL_CHUNK;   // s' columns staged in shared memory at once
constexpr int MX_MAX_ROWS = 1024;   // x' rows per region (2 * xbins)
constexpr int MX_MAX_COLS = 4096;   // s' columns per region (zbins)
#ifndef MX_GEO_THREADS
#define MX_GEO_THREADS 128
#endif
constexpr int GEO_THREADS = MX_GEO_THREADS;
constexpr int SETUP_THREADS = 64;
constexpr int GEO_MAXB = 6;

// Column record: 36 words (9 float4; a stride of 144 B keeps 8-lane phases
// of 16-byte shared loads conflict free).  Row record: 8 words (2 float4).
constexpr int CW = 36;
constexpr int RW = 8;
// column record words (float4 groups); "dw" = double-word (hi, lo):
//  0: t cell (int), z cell (int), t offset (dw)        history coordinates at x'_ref
//  1: z offset (dw), r0 = |R0| (dw)                    R0 = r(s) + x n(s) - r(s') - x'_ref n(s')
//  2: u* = R0.n' / g (dw), rmin^2 = (R0 x n')^2 / g (dw)   foot of the perpendicular from
//     the observer to the line x' -> r(s') + x' n(s'): |r - r'|^2 = rmin^2 + g (u - u*)^2;
//     for s' outside the orbit tables (interpolate1D gives n' = tau' = 0, g = 0, as the
//     reference's) u* = 0 and rmin^2 = r0^2, so that |r - r'| = r0 for every x
//  3: g - 1, K0x = b - a e (dw), curvature at s'       g = |n'|^2
//  4: a = v.tau', b = v.n', e = tau'.n', h = |tau'|^2
//  5: K1x - 1 = a g - 1 + b e, K2x = b g, K0z = a (1 - h), K1z = a e + b h
//  6: K2z = b e, Q0 = R0.(n - n'), Q1 = n'.(n - n'), q2 = n.tau'
//  7: M0 = Q0 - q2 r0, trapz weight in s', a - (float)a (a = word 4.x + this), 0
//  8: 0, 0, 0, 0
// row record words: x0 (int), x weight, u = x' - x'_ref (dw) | trapz weight in x',
// x1 - x0 (int), x', x weight - (float)x weight (the row's weight is shared by
// every s' column, so density_x's x step uses it as a double-word)

struct RegionMeta {
    int nxp, nsp, col_off, row_off;   // offsets in words within the point record
};

struct PointMeta {
    int nreg, valid;
    float inv_dt_hi, inv_dt_lo, inv_dz_hi, inv_dz_lo;   // reciprocals of the history t and z steps (dw)
    // per region: the trapz weights in the records are FP32 roundings of the
    // s' and x' steps, the same relative rounding for every weight of the
    // region (end weights are exactly half the inner ones); the region sum
    // is multiplied by 1 + wdelta, the exact ratio of the FP64 steps to them
    float wdelta[WAKE_MAX_REGIONS];
    RegionMeta reg[WAKE_MAX_REGIONS];
};

// Per-point record size (words): 4 regions of zbins columns and at most
// 5 * xbins rows in total.
__host__ __device__ inline size_t point_record_words(int xbins, int zbins) {
    return (size_t)WAKE_MAX_REGIONS * zbins * CW + (size_t)5 * xbins * RW;
}

// Integer cell of a history coordinate u from its floor fl: clamped to
// +-2e9 with integer operations; NaN -> 2e9 (outside every grid).
__device__ __forceinline__ int cell_index(double u, double fl) {
    const int c = __double2int_rz(fl);   // fl is integral; saturates for huge |u|
    const bool nan = (__double_as_longlong(u) & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
    return nan ? 2000000000 : max(min(c, 2000000000), -2000000000);
}

// s' of column j and x' of row i: start + k * step (the reference's
// linspace up to rounding, which the mixed path does not need to reproduce).
struct Axis {
    double start, step;
    int n;
    __device__ double at(int k) const { return fma((double)k, step, start); }
    __device__ double weight(int k) const {   // trapz weight of sample k
        if (n < 2) return 0.0;
        return (k == 0 || k == n - 1) ? 0.5 * step : step;
    }
};

__device__ __forceinline__ Axis make_axis(double a, double b, int n) {
    Axis ax;
    ax.start = a;
    ax.n = n;
    ax.step = (n > 1) ? (b - a) / (double)(n - 1) : 0.0;
    return ax;
}

__device__ __forceinline__ void layout(const Region *reg, int nreg, RegionMeta *rm, bool &ok,
                                       size_t rec_words, int max_rows) {
    int off = 0;
    ok = true;
    for (int k = 0; k < nreg; ++k) {
        rm[k].nxp = reg[k].nxp;
        rm[k].nsp = reg[k].nsp;
        rm[k].col_off = off;
        off += reg[k].nsp * CW;
        rm[k].row_off = off;
        off += reg[k].nxp * RW;
        if (reg[k].nxp < 1 || reg[k].nxp > max_rows || reg[k].nsp < 1 || reg[k].nsp > MX_MAX_COLS)
            ok = false;
    }
    if ((size_t)off > rec_words) ok = false;
}

// The integral's history-cell offsets are 32-bit counts of float4 (two per
// 32-byte cell): the FP32 ring must hold fewer than 2^32 of them (64 GiB).
__host__ __device__ __forceinline__ bool ring32_offsets_fit(long long cap, long long nx, long long nz) {
    return cap >= 0 && nx >= 0 && nz >= 0 && cap * nx * nz * 2 <= 0xFFFFFFFFll;
}

// One history field at (slot, x, z) from the FP64 ring, else the FP32 ring.
__device__ __forceinline__ double hist_cell(const dfcsr_wake_job &J, int field, int slot, int xi, int zi) {
    if (!(bounds_ok(slot, J.cap, BS_MIXED_SETUP) && bounds_ok(xi, J.nx, BS_MIXED_SETUP) &&
          bounds_ok(zi, J.nz, BS_MIXED_SETUP)))
        return 0.0;
    const size_t cell = ((size_t)slot * J.nx + xi) * J.nz + zi;
    return J.ring64 ? J.ring64[cell * 5 + field] : ring32_value(J.ring32, cell, field);
}

struct alignas(16) GeoShared {
    Region reg[WAKE_MAX_REGIONS];
    RegionMeta rm[WAKE_MAX_REGIONS];
    Axis ax_s[WAKE_MAX_REGIONS], ax_x[WAKE_MAX_REGIONS];
    double xref[WAKE_MAX_REGIONS];
    int col_begin[WAKE_MAX_REGIONS + 1], row_begin[WAKE_MAX_REGIONS + 1];
    int lo[WAKE_MAX_REGIONS], hi[WAKE_MAX_REGIONS];
    // curvature per column: element index at the region's first column and
    // the columns where s' crosses the next element ends (GEO_MAXB at most;
    // more -> per-column lookup)
    int e_first[WAKE_MAX_REGIONS], nthr[WAKE_MAX_REGIONS];
    int thr_j[WAKE_MAX_REGIONS][GEO_MAXB];
    double lat_s[6];
    double vx_obs;
    int nreg, ok;
    // double-word forms for the double-word column and row paths
    dw S0[WAKE_MAX_REGIONS], Sst[WAKE_MAX_REGIONS];   // s'(j) = S0 + j Sst
    dw U0[WAKE_MAX_REGIONS], Ust[WAKE_MAX_REGIONS];   // orbit-table coordinate of s'(j)
    dw X0[WAKE_MAX_REGIONS], Xst[WAKE_MAX_REGIONS];   // x'(i) = X0 + i Xst
    dw UX0[WAKE_MAX_REGIONS], UXst[WAKE_MAX_REGIONS]; // history x coordinate of x'(i)
    dw xrefw[WAKE_MAX_REGIONS];
    dw Px, Py, T0, Tz, inv_t, inv_z, nsx, nsy, tsx, tsy, vxw, Sw;
    // FP32 per-region constants: trapz weights (end point, inner point) in
    // s' and x', curvature of the elements e_first + k, near band half-width
    float wsf[WAKE_MAX_REGIONS][2], wxf[WAKE_MAX_REGIONS][2];
    float wdelta[WAKE_MAX_REGIONS];   // (step_s / wsf[r][1]) (step_x / wxf[r][1]) - 1
    float rhof[WAKE_MAX_REGIONS][GEO_MAXB + 1];
    float band_f;
    double inv_s, inv_x;        // reciprocals of the orbit-table and history x steps
};

__device__ __forceinline__ int cell_of(float fl, bool nan) {
    if (nan) return 2000000000;
    const int c = __float2int_rz(fl);   // integral; saturates for huge values
    return max(min(c, 2000000000), -2000000000);
}

__device__ __forceinline__ bool dw_isnan(dw a) { return a.hi != a.hi; }

// One s' column record in double-word FP32: the same quantities as the FP64
// column code in mixed_geometry, from the double-word orbit tables.
__device__ __noinline__ void column_dw(const dfcsr_wake_job &J, const GeoShared &gs, int r, int j,
                                       dw vxo, dw vyo, float4 *o) {
    const float fj = (float)j;
    const dw spj = dw_add(gs.S0[r], dw_mul_f(gs.Sst[r], fj));
    const dw u = dw_add(gs.U0[r], dw_mul_f(gs.Ust[r], fj));
    dw L[6];
    // interpolate1D rule: in range iff -1 < u < n; lower index int(u)
    // (truncation: u in (-1, 0) uses index 0 and extrapolates)
    const float fn = (float)J.nsample;
    const bool gt = u.hi > -1.f || (u.hi == -1.f && u.lo > 0.f);
    const bool lt = u.hi < fn || (u.hi == fn && u.lo < 0.f);
    if (gt && lt) {
        int a0 = (int)dw_floor(u);
        if (a0 < 0) a0 = 0;
        if (a0 > J.nsample - 1) a0 = J.nsample - 1;
        const dw f = dw_add_f(u, -(float)a0);
        if (!bounds_ok(a0, J.nsample, BS_ORBIT)) a0 = 0;
        const float2 *P = reinterpret_cast<const float2 *>(J.lattice_dw) + (size_t)a0 * 6;
        const float2 *D = reinterpret_cast<const float2 *>(J.lattice_delta_dw) + (size_t)a0 * 6;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const float2 p = P[k], d = D[k];
            L[k] = dw_add(dw_make(p.x, p.y), dw_mul(f, dw_make(d.x, d.y)));
        }
    } else {
#pragma unroll
        for (int k = 0; k < 6; ++k) L[k] = dw_make(0.f, 0.f);
    }
    const dw npx = L[2], npy = L[3], tpx = L[4], tpy = L[5];
    const dw xref = gs.xrefw[r];
    const dw rx0 = dw_sub(dw_sub(gs.Px, L[0]), dw_mul(xref, npx));
    const dw ry0 = dw_sub(dw_sub(gs.Py, L[1]), dw_mul(xref, npy));
    const dw r02 = dw_add_abs(dw_mul(rx0, rx0), dw_mul(ry0, ry0));   // both >= 0
    const dw r0 = dw_sqrt(r02);
    const dw ut0 = dw_mul(dw_sub(gs.T0, r0), gs.inv_t);
    const dw uz0 = dw_mul(dw_add(dw_sub(spj, gs.Tz), r0), gs.inv_z);
    const float tfl = dw_floor(ut0), zfl = dw_floor(uz0);
    // dot products of the orbit vectors: sums of two products whose
    // absolute error 2^-48 (|x| + |y|) is far below what the integrand reads
    // from them (unit vectors: a cancellation leaves a small value, not a
    // small relative error that matters); position differences (rx0, ry0
    // above, the history coordinates) keep the accurate double-word sum
    const dw a = dw_add_abs(dw_mul(vxo, tpx), dw_mul(vyo, tpy));
    const dw bb = dw_add_abs(dw_mul(vxo, npx), dw_mul(vyo, npy));
    const dw e = dw_add_abs(dw_mul(tpx, npx), dw_mul(tpy, npy));
    const dw g = dw_add_abs(dw_mul(npx, npx), dw_mul(npy, npy));
    const dw h = dw_add_abs(dw_mul(tpx, tpx), dw_mul(tpy, tpy));
    const dw nmx = dw_sub(gs.nsx, npx), nmy = dw_sub(gs.nsy, npy);
    const dw Q0 = dw_add_abs(dw_mul(rx0, nmx), dw_mul(ry0, nmy));
    const dw q2 = dw_add_abs(dw_mul(gs.nsx, tpx), dw_mul(gs.nsy, tpy));
    const dw ae = dw_mul(a, e);
    float rho_f;
    if (gs.nthr[r] >= 0) {
        int k = 0;
        for (int q = 0; q < gs.nthr[r]; ++q) k += (j >= gs.thr_j[r][q]) ? 1 : 0;
        rho_f = gs.rhof[r][k];
    } else {
        rho_f = (float)rho_at(J, dw_to_double(spj));
    }
    const bool near = gs.band_f > 0.f && fabsf(dw_float(dw_sub(spj, gs.Sw))) < gs.band_f;
    const float ws = (j == 0 || j == gs.ax_s[r].n - 1) ? gs.wsf[r][0] : gs.wsf[r][1];
    const dw R0n = dw_add_abs(dw_mul(rx0, npx), dw_mul(ry0, npy));
    const dw cr = dw_sub_abs(dw_mul(rx0, npy), dw_mul(ry0, npx));
    // s' outside the orbit tables: n' = 0 (g = 0), the distance is r0 for
    // every x' (the integral's g (u - u*)^2 term vanishes with g - 1 = -1)
    const bool no_normal = !(g.hi > 0.f);
    const dw us = no_normal ? dw{0.f, 0.f} : dw_div(R0n, g);
    const dw rmin2 = no_normal ? r02 : dw_div(dw_mul(cr, cr), g);
    const dw toff = dw_add_f(ut0, -tfl), zoff = dw_add_f(uz0, -zfl);
    const dw K0x = dw_sub(bb, ae);
    o[0] = make_float4(__int_as_float(cell_of(tfl, dw_isnan(ut0))),
                       __int_as_float(cell_of(zfl, dw_isnan(uz0))), toff.hi, toff.lo);
    o[1] = make_float4(zoff.hi, zoff.lo, r0.hi, r0.lo);
    o[2] = make_float4(us.hi, us.lo, rmin2.hi, rmin2.lo);
    o[3] = make_float4(dw_float(dw_add_f(g, -1.f)), K0x.hi, K0x.lo, rho_f);
    o[4] = make_float4(dw_float(a), dw_float(bb), dw_float(e), dw_float(h));
    o[5] = make_float4(dw_float(dw_add_abs(dw_add_f(dw_mul(a, g), -1.f), dw_mul(bb, e))),
                       dw_float(dw_mul(bb, g)), dw_float(dw_mul(a, dw_add_f(dw_neg(h), 1.f))),
                       dw_float(dw_add_abs(ae, dw_mul(bb, h))));
    o[6] = make_float4(dw_float(dw_mul(bb, e)), dw_float(Q0),
                       dw_float(dw_add_abs(dw_mul(npx, nmx), dw_mul(npy, nmy))), dw_float(q2));
    o[7] = make_float4(dw_float(dw_sub(Q0, dw_mul(q2, r0))), near ? 0.f : ws,
                       __fsub_rn(a.hi, dw_float(a)) + a.lo, 0.f);   // band columns: FP64 kernel
    o[8] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// One x' row record in double-word FP32: history x cell with the reference's
// rule (in range iff -1 < u < nx, lower index int(u), weight u - int(u)),
// u = x' - x'_ref, x', trapz weight; in-range rows widen the valid range.
__device__ __forceinline__ void row_dw(const dfcsr_wake_job &J, GeoShared &gs, int r, int i,
                                       float4 *rb) {
    const float fi = (float)i;
    const dw ux = dw_add(gs.UX0[r], dw_mul_f(gs.UXst[r], fi));
    const dw xpi = dw_add(gs.X0[r], dw_mul_f(gs.Xst[r], fi));
    const float fnx = (float)J.nx;
    const bool in = (ux.hi > -1.f || (ux.hi == -1.f && ux.lo > 0.f)) &&
                    (ux.hi < fnx || (ux.hi == fnx && ux.lo < 0.f));
    int x0 = 0, x1 = 0;
    dw xw{0.f, 0.f};
    if (in) {
        x0 = max((int)dw_floor(ux), 0);   // int() truncation: u in (-1, 0) -> 0
        x1 = (x0 == J.nx - 1) ? x0 : x0 + 1;
        xw = dw_add_f(ux, -(float)x0);
    }
    const int n = gs.ax_x[r].n;
    const dw u = dw_sub(xpi, gs.xrefw[r]);
    rb[2 * i] = make_float4(__int_as_float(x0), xw.hi, u.hi, u.lo);
    rb[2 * i + 1] = make_float4((i == 0 || i == n - 1) ? gs.wxf[r][0] : gs.wxf[r][1],
                                __int_as_float(x1 - x0), dw_float(xpi), xw.lo);
    if (in) {
        atomicMin(&gs.lo[r], i);   // integer min / max: order independent
        atomicMax(&gs.hi[r], i);
    }
}

// FP64 column and row records (jobs without double-word orbit tables).
__device__ __noinline__ void geometry_fp64(const dfcsr_wake_job &J, GeoShared &gs, double t, double s,
                                           double x, float *prec, int ncols, int nrows) {
    const int nreg = gs.nreg;
    const double X0s = gs.lat_s[0], Y0s = gs.lat_s[1], nsx = gs.lat_s[2], nsy = gs.lat_s[3];
    const double vxo = gs.lat_s[4] + gs.vx_obs * nsx, vyo = gs.lat_s[5] + gs.vx_obs * nsy;
    const double inv_s = 1.0 / J.s_delta, inv_t = 1.0 / J.t_delta, inv_z = 1.0 / J.z_delta;
    const double inv_x = 1.0 / J.x_delta;
    // per-point constants: r(s) + x n(s), t - t_min, t + z_min
    const double Px = fma(x, nsx, X0s), Py = fma(x, nsy, Y0s);
    const double T0 = t - J.t_min, Tz = t + J.z_min;
    const double *dtab = J.lattice_delta;
    for (int c = threadIdx.x; c < ncols; c += blockDim.x) {
        int r = 0;
        while (r + 1 < nreg && c >= gs.col_begin[r + 1]) ++r;
        const int j = c - gs.col_begin[r];
        const Axis ax_s = gs.ax_s[r];
        const double xref = gs.xref[r];
        const double spj = ax_s.at(j);
        // orbit tables at s' (interpolate1D rule: in range iff -1 < u < n,
        // lower index int(u)), one FMA per table column with the differences
        double L[6];
        {
            const double u = fma((double)j, ax_s.step * inv_s, (ax_s.start - J.s_min) * inv_s);
            const int a0 = __double2int_rz(u);   // truncation, saturating
            const bool nan = (__double_as_longlong(u) & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
            // u in (-1, 0) truncates to 0 (extrapolation, like int()); u <= -1
            // truncates below 0
            if (!nan && a0 >= 0 && a0 < J.nsample) {
                const double f = u - (double)a0;
                const double *pa = J.lattice + (size_t)a0 * 6;
                if (dtab) {
                    const double *da = dtab + (size_t)a0 * 6;
#pragma unroll
                    for (int k = 0; k < 6; ++k) L[k] = fma(f, da[k], pa[k]);
                } else {
                    const double *pb = J.lattice + (size_t)(a0 == J.nsample - 1 ? a0 : a0 + 1) * 6;
#pragma unroll
                    for (int k = 0; k < 6; ++k) L[k] = fma(f, pb[k] - pa[k], pa[k]);
                }
            } else {
#pragma unroll
                for (int k = 0; k < 6; ++k) L[k] = 0.0;
            }
        }
        const double npx = L[2], npy = L[3], tpx = L[4], tpy = L[5];
        const double rx0 = fma(-xref, npx, Px - L[0]), ry0 = fma(-xref, npy, Py - L[1]);
        const double r0 = sqrt(fma(rx0, rx0, ry0 * ry0));
        const double ut0 = (T0 - r0) * inv_t;
        const double uz0 = ((spj - Tz) + r0) * inv_z;
        const double tfl = floor(ut0), zfl = floor(uz0);
        float rho_f;
        if (gs.nthr[r] >= 0) {
            int e = gs.e_first[r];
            for (int q = 0; q < gs.nthr[r]; ++q) e += (j >= gs.thr_j[r][q]) ? 1 : 0;
            rho_f = (e < J.nelement) ? (float)J.rho[e] : 0.f;
        } else {
            rho_f = (float)rho_at(J, spj);
        }
        const double a = vxo * tpx + vyo * tpy, bb = vxo * npx + vyo * npy;
        const double e = tpx * npx + tpy * npy, g = npx * npx + npy * npy;
        const double h = tpx * tpx + tpy * tpy;
        const double nmx = nsx - npx, nmy = nsy - npy;
        const double Q0 = rx0 * nmx + ry0 * nmy;
        const double q2 = nsx * tpx + nsy * tpy;
        const bool near = J.near_band > 0.0 && fabs(spj - s) < J.near_band;
        float4 *o = reinterpret_cast<float4 *>(prec + gs.rm[r].col_off) + (size_t)j * (CW / 4);
        const double R0n = rx0 * npx + ry0 * npy, cr = rx0 * npy - ry0 * npx;
        const dw toff = dw_from(ut0 - tfl), zoff = dw_from(uz0 - zfl), r0w = dw_from(r0);
        // s' outside the orbit tables: n' = 0, the distance is r0 for every x'
        const bool no_normal = !(g > 0.0);
        const dw us = no_normal ? dw{0.f, 0.f} : dw_from(R0n / g);
        const dw rmin2 = no_normal ? dw_from(rx0 * rx0 + ry0 * ry0) : dw_from(cr * cr / g);
        const dw K0x = dw_from(bb - a * e);
        o[0] = make_float4(__int_as_float(cell_index(ut0, tfl)), __int_as_float(cell_index(uz0, zfl)),
                           toff.hi, toff.lo);
        o[1] = make_float4(zoff.hi, zoff.lo, r0w.hi, r0w.lo);
        o[2] = make_float4(us.hi, us.lo, rmin2.hi, rmin2.lo);
        o[3] = make_float4((float)(g - 1.0), K0x.hi, K0x.lo, rho_f);
        o[4] = make_float4((float)a, (float)bb, (float)e, (float)h);
        o[5] = make_float4((float)((a * g - 1.0) + bb * e), (float)(bb * g), (float)(a * (1.0 - h)),
                           (float)(a * e + bb * h));
        o[6] = make_float4((float)(bb * e), (float)Q0, (float)(npx * nmx + npy * nmy), (float)q2);
        o[7] = make_float4((float)(Q0 - q2 * r0), near ? 0.f : (float)ax_s.weight(j),
                           (float)(a - (double)(float)a), 0.f);   // band columns: FP64 kernel
        o[8] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    // rows: x cell, offset, u = x' - x'_ref, x', trapz weight; valid row range
    for (int c = threadIdx.x; c < nrows; c += blockDim.x) {
        int r = 0;
        while (r + 1 < nreg && c >= gs.row_begin[r + 1]) ++r;
        const int i = c - gs.row_begin[r];
        const Axis ax_x = gs.ax_x[r];
        const double xpi = ax_x.at(i);
        const double ux = fma((double)i, ax_x.step * inv_x, (gs.reg[r].xl - J.x_min) * inv_x);
        // x axis of the history with the reference's rule (interpolate3D:
        // in range iff -1 < u < nx, lower index int(u), weight u - int(u));
        // rows in range form one contiguous run because u grows with i
        int x0 = 0, x1 = 0;
        double xw = 0.0;
        const bool in = axis_index(ux, J.nx, x0, x1, xw);
        float4 *rb = reinterpret_cast<float4 *>(prec + gs.rm[r].row_off);
        const dw u = dw_from(xpi - gs.xref[r]);
        const dw xwd = dw_from(xw);
        rb[2 * i] = make_float4(__int_as_float(x0), xwd.hi, u.hi, u.lo);
        rb[2 * i + 1] = make_float4((float)ax_x.weight(i), __int_as_float(x1 - x0), (float)xpi, xwd.lo);
        if (in) {
            atomicMin(&gs.lo[r], i);   // integer min / max: order independent
            atomicMax(&gs.hi[r], i);
        }
    }
}

// Per-point set-up of the geometry: regions and record layout, orbit at s,
// vx at the observer, per-region axes, element thresholds and double-word
// constants.  These are chains of dependent FP64 operations (some hundred
// cycles each on this GPU) done by single threads, so they run in a kernel
// of their own: 64-thread CTAs, many per SM, hide one another's latency,
// and the geometry CTAs start from the finished record.  Two warps: warp 0
// finds the regions (lane 0) and sets up one region per lane; in warp 1,
// lane 0 interpolates vx at the observer, lane 1 the orbit at s, lane 2 the
// history constants.
__global__ void __launch_bounds__(SETUP_THREADS)
mixed_setup(const dfcsr_wake_job *__restrict__ jobs, const int32_t *__restrict__ job_of_point,
            const double *__restrict__ S, const double *__restrict__ X, int64_t first, int64_t count,
            size_t rec_words, int max_rows, GeoShared *__restrict__ setup) {
    __shared__ GeoShared gs;
    const int64_t b = blockIdx.x;
    const int64_t pt = first + b;
    if (b >= count) return;
    const dfcsr_wake_job &J = jobs[job_of_point ? job_of_point[pt] : 0];
    const double t = J.position, s = S[pt], x = X[pt];
    const bool use_dw = J.lattice_dw != nullptr && J.lattice_delta_dw != nullptr;
    // the independent per-point set-up tasks run in separate warps
    if (threadIdx.x >= 32) {
        // warp 1: the eight quotients of the set-up in ONE warp-wide FP64
        // division (lane l), instead of eight divisions issued one after
        // another by single threads (an FP64 instruction costs the SM's FP64
        // unit the same time for one active lane as for 32)
        const int l = threadIdx.x - 32;
        double num = 1.0, den = 1.0;
        if (l == 0) { num = t - J.t_min; den = J.t_delta; }
        else if (l == 1) { num = x - J.x_min; den = J.x_delta; }
        else if (l == 2) { num = (s - t) - J.z_min; den = J.z_delta; }
        else if (l == 3) { num = s - J.s_min; den = J.s_delta; }
        else if (l == 4) den = J.t_delta;
        else if (l == 5) den = J.z_delta;
        else if (l == 6) den = J.s_delta;
        else if (l == 7) den = J.x_delta;
        const double q = num / den;
        double qv[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) qv[k] = __shfl_sync(0xffffffffu, q, k);
        // axis indices in one pass: lanes 0..2 the history t, x, z of vx at
        // the observer, lane 3 the orbit-table index of s
        const double uu = q;   // lanes 0..3 hold these quotients themselves
        const int nn = (l == 0) ? J.nt : (l == 1) ? J.nx : (l == 2) ? J.nz : J.nsample;
        int i0 = 0, i1 = 0;
        double fr = 0.0;
        const bool in = l < 4 && axis_index(uu, nn, i0, i1, fr);
        const unsigned inm = __ballot_sync(0xffffffffu, in);
        const bool hist_in = (inm & 7u) == 7u, lat_in = (inm & 8u) != 0u;
        const int t0 = __shfl_sync(0xffffffffu, i0, 0), t1 = __shfl_sync(0xffffffffu, i1, 0);
        const int x0 = __shfl_sync(0xffffffffu, i0, 1), x1 = __shfl_sync(0xffffffffu, i1, 1);
        const int z0 = __shfl_sync(0xffffffffu, i0, 2), z1 = __shfl_sync(0xffffffffu, i1, 2);
        const int a0 = __shfl_sync(0xffffffffu, i0, 3), a1 = __shfl_sync(0xffffffffu, i1, 3);
        const double td = __shfl_sync(0xffffffffu, fr, 0), xd = __shfl_sync(0xffffffffu, fr, 1);
        const double zd = __shfl_sync(0xffffffffu, fr, 2), lf = __shfl_sync(0xffffffffu, fr, 3);
        // one warp-wide lerp: lanes 0..3 the t-lerps of vx at the four (x, z)
        // history corners (lane = 2 xi + zi), lanes 4..9 the six orbit tables
        // at s (interpolate3D / interpolate1D arithmetic)
        double pa = 0.0, pb = 0.0, wgt = 0.0;
        if (l < 4) {
            if (hist_in) {
                const int xi = (l & 2) ? x1 : x0, zi = (l & 1) ? z1 : z0;
                const int s0 = ring_slot(J, t0), s1 = ring_slot(J, t1);
                pa = hist_cell(J, 3, s0, xi, zi);
                pb = hist_cell(J, 3, s1, xi, zi);
                wgt = td;
            }
        } else if (l < 10) {
            if (lat_in && bounds_ok(a0, J.nsample, BS_ORBIT) && bounds_ok(a1, J.nsample, BS_ORBIT)) {
                pa = J.lattice[(size_t)a0 * 6 + (l - 4)];
                pb = J.lattice[(size_t)a1 * 6 + (l - 4)];
                wgt = lf;
            }
        }
        const double lv = pa * (1 - wgt) + pb * wgt;
        // then x (lanes 0, 1: z0 and z1) and z
        const double cx1 = __shfl_sync(0xffffffffu, lv, (l & 1) + 2);
        const double e = lv * (1 - xd) + cx1 * xd;
        const double e1 = __shfl_sync(0xffffffffu, e, 1);
        const double vx_obs = __shfl_sync(0xffffffffu, hist_in ? e * (1 - zd) + e1 * zd : 0.0, 0);
        double lat[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) lat[k] = lat_in ? __shfl_sync(0xffffffffu, lv, 4 + k) : 0.0;
        if (l == 0) gs.vx_obs = vx_obs;
        if (l >= 4 && l < 10) gs.lat_s[l - 4] = lat_in ? lv : 0.0;
        // the per-point double-word constants in one warp-wide conversion
        double dv = 0.0;
        switch (l) {
            case 0: dv = fma(x, lat[2], lat[0]); break;   // r(s) + x n(s)
            case 1: dv = fma(x, lat[3], lat[1]); break;
            case 2: dv = lat[2]; break;
            case 3: dv = lat[3]; break;
            case 4: dv = lat[4]; break;
            case 5: dv = lat[5]; break;
            case 6: dv = t - J.t_min; break;
            case 7: dv = t + J.z_min; break;
            case 8: dv = qv[4]; break;
            case 9: dv = qv[5]; break;
            case 10: dv = s; break;
            case 11: dv = vx_obs; break;
            default: break;
        }
        const dw dd = dw_from(dv);
        if (l == 11) gs.vxw = dd;
        if (l == 8) gs.inv_t = dd;   // the integral needs these for every job
        if (l == 9) gs.inv_z = dd;
        if (use_dw) {
            switch (l) {
                case 0: gs.Px = dd; break;
                case 1: gs.Py = dd; break;
                case 2: gs.nsx = dd; break;
                case 3: gs.nsy = dd; break;
                case 4: gs.tsx = dd; break;
                case 5: gs.tsy = dd; break;
                case 6: gs.T0 = dd; break;
                case 7: gs.Tz = dd; break;
                case 10: gs.Sw = dd; break;
                default: break;
            }
        }
        if (l == 12) {
            gs.inv_s = qv[6];
            gs.inv_x = qv[7];
            gs.band_f = (use_dw && J.near_band > 0.0) ? (float)J.near_band : 0.f;
        }
    } else {
        // warp 0: lane 0 finds the regions and the record layout, then one
        // lane per region sets up that region's axes and element thresholds
        if (threadIdx.x == 0) {
            gs.nreg = wake_regions(J, s, x, gs.reg);
            bool ok;
            layout(gs.reg, gs.nreg, gs.rm, ok, rec_words, max_rows);
            // the integral reads 32-byte cells with one 256-bit load: a ring
            // that is not 32-byte aligned makes the point invalid (NaN result)
            if (((uintptr_t)J.ring32 & 31u) != 0) ok = false;
            // and forms cell offsets in 32-bit float4 units: a ring of more
            // than 2^32 of them (64 GiB) makes the point invalid too
            if (!ring32_offsets_fit(J.cap, J.nx, J.nz)) ok = false;
            gs.ok = ok ? 1 : 0;
            int cb = 0, rb = 0;
            for (int r = 0; r < gs.nreg; ++r) {
                gs.col_begin[r] = cb;
                gs.row_begin[r] = rb;
                cb += gs.reg[r].nsp;
                rb += gs.reg[r].nxp;
            }
            gs.col_begin[gs.nreg] = cb;
            gs.row_begin[gs.nreg] = rb;
        }
        __syncwarp();
        // the regions' axes in one warp-wide division: lanes 0..3 the s'
        // axis of region lane, lanes 4..7 the x' axis of region lane - 4
        {
            const int lane = threadIdx.x, rr = lane & 3;
            const bool mine = lane < 8 && rr < gs.nreg;
            double aa = 0.0, ab = 1.0;
            int an = 2;
            if (mine) {
                const Region &R = gs.reg[rr];
                if (lane < 4) { aa = R.sl; ab = R.sr; an = R.nsp; }
                else { aa = R.xl; ab = R.xr; an = R.nxp; }
            }
            const Axis ax = make_axis(aa, ab, an);
            if (mine) {
                if (lane < 4) gs.ax_s[rr] = ax;
                else { gs.ax_x[rr] = ax; gs.xref[rr] = ax.at(an / 2); }
            }
        }
        __syncwarp();
        const int r = threadIdx.x;
        if (r < gs.nreg) {
            const Region &R = gs.reg[r];
            const Axis A = gs.ax_s[r], AX = gs.ax_x[r];
            gs.lo[r] = R.nxp;
            gs.hi[r] = -1;
            // rho_at over the region's columns s'(j) = start + j step (non-
            // decreasing in j): element index = number of element ends <= s'
            const double s_first = A.at(0), s_last = A.at(R.nsp - 1);
            int ef = 0, nb = (A.step > 0.0) ? 0 : -1;   // descending / flat: per column
            for (int e = 0; e < J.nelement && nb >= 0; ++e) {
                const double d = J.distance[e];
                if (d <= s_first) ++ef;
                else if (d <= s_last) {
                    if (nb == GEO_MAXB) { nb = -1; break; }
                    // first column j with s'(j) >= d
                    int jj = (int)ceil((d - A.start) / A.step);
                    jj = max(0, min(jj, R.nsp - 1));
                    while (jj > 0 && A.at(jj - 1) >= d) --jj;
                    while (jj < R.nsp - 1 && A.at(jj) < d) ++jj;
                    gs.thr_j[r][nb++] = jj;
                }
            }
            gs.e_first[r] = ef;
            gs.nthr[r] = nb;
            for (int k = 0; k <= GEO_MAXB; ++k)
                gs.rhof[r][k] = (k <= nb && ef + k < J.nelement) ? (float)J.rho[ef + k] : 0.f;
            gs.wsf[r][0] = A.n < 2 ? 0.f : (float)(0.5 * A.step);
            gs.wsf[r][1] = A.n < 2 ? 0.f : (float)A.step;
            gs.wxf[r][0] = AX.n < 2 ? 0.f : (float)(0.5 * AX.step);
            gs.wxf[r][1] = AX.n < 2 ? 0.f : (float)AX.step;
            gs.wdelta[r] = (A.n < 2 || AX.n < 2 || gs.wsf[r][1] == 0.f || gs.wxf[r][1] == 0.f)
                               ? 0.f
                               : (float)((A.step / (double)gs.wsf[r][1]) * (AX.step / (double)gs.wxf[r][1]) - 1.0);
        }
    }
    __syncthreads();
    // the regions' double-word constants (nine per region; the orbit-table
    // and history coordinates need warp 1's reciprocals), two warp-wide
    // conversions: value v = 9 r + k
    if (use_dw && threadIdx.x < 32) {
        for (int v = threadIdx.x; v < 9 * WAKE_MAX_REGIONS; v += 32) {
            const int r = v / 9, k = v - 9 * r;
            double val = 0.0;
            if (r < gs.nreg) {
                const Axis A = gs.ax_s[r], AX = gs.ax_x[r];
                switch (k) {
                    case 0: val = A.start; break;
                    case 1: val = A.step; break;
                    case 2: val = AX.start; break;
                    case 3: val = AX.step; break;
                    case 4: val = gs.xref[r]; break;
                    case 5: val = (A.start - J.s_min) * gs.inv_s; break;
                    case 6: val = A.step * gs.inv_s; break;
                    case 7: val = (AX.start - J.x_min) * gs.inv_x; break;
                    default: val = AX.step * gs.inv_x; break;
                }
            }
            const dw d = dw_from(val);
            if (r < gs.nreg) {
                switch (k) {
                    case 0: gs.S0[r] = d; break;
                    case 1: gs.Sst[r] = d; break;
                    case 2: gs.X0[r] = d; break;
                    case 3: gs.Xst[r] = d; break;
                    case 4: gs.xrefw[r] = d; break;
                    case 5: gs.U0[r] = d; break;
                    case 6: gs.Ust[r] = d; break;
                    case 7: gs.UX0[r] = d; break;
                    default: gs.UXst[r] = d; break;
                }
            }
        }
    }
    __syncthreads();
    // the finished record to global memory
    const uint4 *src = reinterpret_cast<const uint4 *>(&gs);
    uint4 *dst = reinterpret_cast<uint4 *>(setup + b);
    for (int k = threadIdx.x; k < (int)(sizeof(GeoShared) / 16); k += blockDim.x) dst[k] = src[k];
}

// One 128-thread CTA per observation point (six per SM): the point's set-up
// record from mixed_setup, then the s' columns of all regions as one flat
// range across the block, then the x' rows likewise.
#ifndef MX_GEO_BLOCKS
#define MX_GEO_BLOCKS 6
#endif
__global__ void __launch_bounds__(GEO_THREADS, MX_GEO_BLOCKS)
mixed_geometry(const dfcsr_wake_job *__restrict__ jobs, const int32_t *__restrict__ job_of_point,
               const double *__restrict__ S, const double *__restrict__ X, int64_t first, int64_t count,
               const GeoShared *__restrict__ setup, size_t rec_words, float *__restrict__ rec,
               PointMeta *__restrict__ meta, int2 *__restrict__ rows_valid, double *__restrict__ obs_vx) {
    __shared__ GeoShared gs;
    const int64_t b = blockIdx.x;
    const int64_t pt = first + b;
    if (b >= count) return;
    const dfcsr_wake_job &J = jobs[job_of_point ? job_of_point[pt] : 0];
    const double t = J.position, s = S[pt], x = X[pt];
    const bool use_dw = J.lattice_dw != nullptr && J.lattice_delta_dw != nullptr;
    {
        const uint4 *src = reinterpret_cast<const uint4 *>(setup + b);
        uint4 *dst = reinterpret_cast<uint4 *>(&gs);
        for (int k = threadIdx.x; k < (int)(sizeof(GeoShared) / 16); k += blockDim.x) dst[k] = src[k];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        PointMeta m;
        m.nreg = gs.nreg;
        m.valid = gs.ok;
        m.inv_dt_hi = gs.inv_t.hi;
        m.inv_dt_lo = gs.inv_t.lo;
        m.inv_dz_hi = gs.inv_z.hi;
        m.inv_dz_lo = gs.inv_z.lo;
        for (int k = 0; k < WAKE_MAX_REGIONS; ++k) {
            m.reg[k] = (k < gs.nreg) ? gs.rm[k] : RegionMeta{0, 0, 0, 0};
            m.wdelta[k] = (k < gs.nreg) ? gs.wdelta[k] : 0.f;
        }
        meta[b] = m;
        obs_vx[b] = gs.vx_obs;
    }
    if (!gs.ok) return;
    const int nreg = gs.nreg;
    float *prec = rec + (size_t)b * rec_words;
    const int ncols = gs.col_begin[nreg];
    const int nrows = gs.row_begin[nreg];
    for (int r = 0; r < nreg; ++r)   // checked build: every record inside the point's words
        if (!(bounds_ok((long long)gs.rm[r].col_off + (long long)gs.rm[r].nsp * CW - 1,
                        (long long)rec_words, BS_GEO_REC) &&
              bounds_ok((long long)gs.rm[r].row_off + (long long)gs.rm[r].nxp * RW - 1,
                        (long long)rec_words, BS_GEO_REC)))
            return;
    if (use_dw) {
        // observer velocity direction v = tau(s) + vx n(s), FP32 double-word
        const dw vxo = dw_add(gs.tsx, dw_mul(gs.vxw, gs.nsx));
        const dw vyo = dw_add(gs.tsy, dw_mul(gs.vxw, gs.nsy));
        for (int c = threadIdx.x; c < ncols; c += blockDim.x) {
            int r = 0;
            while (r + 1 < nreg && c >= gs.col_begin[r + 1]) ++r;
            const int j = c - gs.col_begin[r];
            float4 *o = reinterpret_cast<float4 *>(prec + gs.rm[r].col_off) + (size_t)j * (CW / 4);
            column_dw(J, gs, r, j, vxo, vyo, o);
        }
        for (int c = threadIdx.x; c < nrows; c += blockDim.x) {
            int r = 0;
            while (r + 1 < nreg && c >= gs.row_begin[r + 1]) ++r;
            const int i = c - gs.row_begin[r];
            row_dw(J, gs, r, i, reinterpret_cast<float4 *>(prec + gs.rm[r].row_off));
        }
    } else {
        geometry_fp64(J, gs, t, s, x, prec, ncols, nrows);
    }
    __syncthreads();
    if (threadIdx.x < nreg)
        rows_valid[b * WAKE_MAX_REGIONS + threadIdx.x] = make_int2(gs.lo[threadIdx.x], gs.hi[threadIdx.x] + 1);
}

// Resolve one axis from an integer base and a double-word offset with the
// reference's int() truncation rule (in range iff -1 < u < n, u = base +
// off): the lower index and the FP32 weight.  The range decision uses the
// double-word value, so it agrees with the FP64 decision except within
// ~1e-12 cells of a boundary (at u = -1 the reference's interpolant jumps
// from an extrapolated value to zero).
__device__ __forceinline__ bool axis_split_dw(int base, dw off, int n, int &i0, int &i1, float &w,
                                              float &w_lo) {
    float k = floorf(off.hi);
    dw fr = fast_two_sum(__fsub_rn(off.hi, k), off.lo);   // off.hi - k is exact
    if (fr.hi < 0.f) { k = __fsub_rn(k, 1.f); fr = dw_add_f(fr, 1.f); }
    else if (fr.hi >= 1.f) { k = __fadd_rn(k, 1.f); fr = dw_add_f(fr, -1.f); }
    const int ui = base + (int)k;
    if (!(ui > -1 || (ui == -1 && fr.hi > 0.f)) || ui >= n) return false;
    if (ui == -1) { i0 = 0; fr = dw_add_f(fr, -1.f); }
    else i0 = ui;
    w = fr.hi;
    w_lo = fr.lo;
    i1 = (i0 == n - 1) ? i0 : i0 + 1;
    return true;
}

struct Fields5 {
    float den, dz, vxx;
    dw dx, vx;   // double-word: interpolated in offset form, the t step in double-word
};

// A 32-byte history cell (den, dx_hi, dz, vx_hi | vxx, dx_lo, vx_lo, pad) in
// one 256-bit non-coherent load; the pad word is not kept.
__device__ __forceinline__ void ld_cell(const float4 *p, float4 &a, float4 &b) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

// a + w (b - a) with one rounding for the product-add.
__device__ __forceinline__ float lerp1(float a, float b, float w) { return fmaf(w, b - a, a); }

// Bilinear (x, then z) interpolation of a hi + lo field in one history
// slice, in offset form: the corners enter as (hi_c - h) + lo_c with h the
// high part of the slice's first corner (the subtraction is exact for
// neighbouring values within a factor 2, and neighbouring cells in x and z
// differ by a few %), so the FP32 chain rounds only small numbers.  Returns
// h and the interpolated offset D (value = h + D).
__device__ __forceinline__ void slice_offset(float h00, float l00, float h01, float l01, float h10,
                                             float l10, float h11, float l11, float xd, float zd,
                                             float &h, float &D) {
    h = h00;
    const float o01 = __fadd_rn(__fsub_rn(h01, h), l01);
    const float o10 = __fadd_rn(__fsub_rn(h10, h), l10);
    const float o11 = __fadd_rn(__fsub_rn(h11, h), l11);
    const float e0 = lerp1(l00, o10, xd);
    const float e1 = lerp1(o01, o11, xd);
    D = lerp1(e0, e1, zd);
}

// P0 + td (P1 - P0) with P = h + D per slice, in double-word: consecutive
// history slices differ by up to ~100 % (a beam step apart), so this step is
// the one an FP32 chain would round at the value's own size.
__device__ __forceinline__ dw tlerp_dw(float h0, float D0, float h1, float D1, float td) {
    const dw dh = two_sum(h1, -h0);
    const dw d = fast_two_sum(dh.hi, __fadd_rn(dh.lo, __fsub_rn(D1, D0)));
    const dw p = two_prod(td, d.hi);
    const dw a = two_sum(h0, p.hi);
    return fast_two_sum(a.hi, __fadd_rn(__fadd_rn(a.lo, D0), __fmaf_rn(td, d.lo, p.lo)));
}

// a + w (b - a) for double-words a, b (hi + lo, not renormalised between
// steps) and a double-word weight wh + wl: the difference and the product
// are formed without error (TwoSum, FMA TwoProd), so the result carries
// ~2^-46 of the values' magnitude instead of an FP32 rounding.  Each weight
// of a gather is shared by many terms of the wake's sums (the x weight by
// every s' column of a row), so it must not be rounded to FP32 either.
__device__ __forceinline__ dw lerp_dw2(dw a, dw b, float wh, float wl) {
    const dw s = two_sum(b.hi, -a.hi);
    const float dl = __fadd_rn(s.lo, __fsub_rn(b.lo, a.lo));
    const dw p = two_prod(wh, s.hi);
    const dw r = two_sum(a.hi, p.hi);
    const float pl = __fmaf_rn(wl, s.hi, __fmaf_rn(wh, dl, p.lo));
    return dw{r.hi, __fadd_rn(__fadd_rn(r.lo, a.lo), pl)};
}

// Trilinear gather of the five fields from ring32 [slot][nx][nz][8] at
// (t, x, z): density, density_z and vx_x in FP32 (t, then x, then z, like
// the reference); density_x as a double-word lerp chain and vx in per-slice
// offset form with a double-word t step (the wake's density_x term cancels
// to ~1/300 of its terms, and vx enters it through b - vx (K1x + vx K2x)
// where the two are of similar size after a bend).
// c<x><t>: float4 index of the z0 cell at x0/x1, t0/t1; dzc: float4 step to z1.
template <bool DXDW>
__device__ __forceinline__ Fields5 gather5(const float4 *__restrict__ ring, uint32_t c00, uint32_t c01,
                                           uint32_t c10, uint32_t c11, uint32_t dzc, float td,
                                           float td_lo, float xd, float xd_lo, float zd, float zd_lo) {
    // one 32-byte load per cell (the cells are 32-byte aligned)
    float4 A0, A1, B0, B1, C0, C1, D0, D1;
    float4 a0, a1, b0, b1, c0, c1, d0, d1;
    ld_cell(ring + c00, A0, a0);   // t0 x0 z0
    ld_cell(ring + c00 + dzc, A1, a1);   // t0 x0 z1
    ld_cell(ring + c01, B0, b0);   // t1 x0 z0
    ld_cell(ring + c01 + dzc, B1, b1);   // t1 x0 z1
    ld_cell(ring + c10, C0, c0);   // t0 x1 z0
    ld_cell(ring + c10 + dzc, C1, c1);   // t0 x1 z1
    ld_cell(ring + c11, D0, d0);   // t1 x1 z0
    ld_cell(ring + c11 + dzc, D1, d1);   // t1 x1 z1
    auto tri = [&](float v00a, float v00b, float v01a, float v01b, float v10a, float v10b,
                   float v11a, float v11b) -> float {
        const float c00_ = lerp1(v00a, v00b, td);
        const float c01_ = lerp1(v01a, v01b, td);
        const float c10_ = lerp1(v10a, v10b, td);
        const float c11_ = lerp1(v11a, v11b, td);
        const float e0 = lerp1(c00_, c10_, xd);
        const float e1 = lerp1(c01_, c11_, xd);
        return lerp1(e0, e1, zd);
    };
    Fields5 r;
    r.den = tri(A0.x, B0.x, A1.x, B1.x, C0.x, D0.x, C1.x, D1.x);
    r.dz = tri(A0.z, B0.z, A1.z, B1.z, C0.z, D0.z, C1.z, D1.z);
    r.vxx = tri(a0.x, b0.x, a1.x, b1.x, c0.x, d0.x, c1.x, d1.x);
    float h0, q0, h1, q1;
    // density_x (high parts in .y of the first float4, low parts in .y of
    // the second): the reference's t, x, z lerp chain in double-word where
    // its terms cancel (DXDW: the far and middle regions); near the source
    // they do not, and the corners enter in offset form from the first
    // corner's high part, (hi_c - h) + lo_c, with an FP32 chain
    if (!DXDW) {
        const float h = A0.y;
        const float D = tri(a0.y, __fadd_rn(__fsub_rn(B0.y, h), b0.y), __fadd_rn(__fsub_rn(A1.y, h), a1.y),
                            __fadd_rn(__fsub_rn(B1.y, h), b1.y), __fadd_rn(__fsub_rn(C0.y, h), c0.y),
                            __fadd_rn(__fsub_rn(D0.y, h), d0.y), __fadd_rn(__fsub_rn(C1.y, h), c1.y),
                            __fadd_rn(__fsub_rn(D1.y, h), d1.y));
        r.dx = two_sum(h, D);
    } else {
        const dw c00 = lerp_dw2(dw{A0.y, a0.y}, dw{B0.y, b0.y}, td, td_lo);
        const dw c01 = lerp_dw2(dw{A1.y, a1.y}, dw{B1.y, b1.y}, td, td_lo);
        const dw c10 = lerp_dw2(dw{C0.y, c0.y}, dw{D0.y, d0.y}, td, td_lo);
        const dw c11 = lerp_dw2(dw{C1.y, c1.y}, dw{D1.y, d1.y}, td, td_lo);
        const dw e0 = lerp_dw2(c00, c10, xd, xd_lo);
        const dw e1 = lerp_dw2(c01, c11, xd, xd_lo);
        const dw v = lerp_dw2(e0, e1, zd, zd_lo);
        r.dx = fast_two_sum(v.hi, v.lo);
    }
    // vx: high parts in .w of the first float4, low parts in .z of the second
    slice_offset(A0.w, a0.z, A1.w, a1.z, C0.w, c0.z, C1.w, c1.z, xd, zd, h0, q0);
    slice_offset(B0.w, b0.z, B1.w, b1.z, D0.w, d0.z, D1.w, d1.z, xd, zd, h1, q1);
    r.vx = tlerp_dw(h0, q0, h1, q1, td);
    return r;
}

__device__ __forceinline__ void kahan(float &s, float &c, float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

// Shared memory of the integral kernel: the column records of one chunk, the
// reduction slots and the point index, followed by the row records of one
// region (2 * xbins_max rows, sized at launch so that the rest of the SM's
// unified L1 / shared memory stays cache for the history gathers).
struct IntegralSmem {
    float4 col[MX_CHUNK * CW / 4];
    float4 red[MX_THREADS / 32];
    long long pt[2];   // the current work unit and the next one (fetched during the current)
};
constexpr size_t kIntegralRowOff = (sizeof(IntegralSmem) + 15) & ~(size_t)15;

__host__ __device__ inline size_t integral_smem_bytes(int max_rows) {
    return kIntegralRowOff + (size_t)max_rows * RW * sizeof(float);
}

// Deterministic block sum of two double-word values (fixed shuffle tree,
// warps added in order by thread 0; result valid in thread 0).  FP32
// double-word additions instead of FP64: GB300's FP64 rate is 1/72 of FP32.
__device__ __forceinline__ void block_sum2_dw(dw &z, dw &x, float4 *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const dw oz{__shfl_down_sync(0xffffffffu, z.hi, o), __shfl_down_sync(0xffffffffu, z.lo, o)};
        const dw ox{__shfl_down_sync(0xffffffffu, x.hi, o), __shfl_down_sync(0xffffffffu, x.lo, o)};
        z = dw_add(z, oz);
        x = dw_add(x, ox);
    }
    if (lane == 0) red[warp] = make_float4(z.hi, z.lo, x.hi, x.lo);
    __syncthreads();
    if (threadIdx.x == 0) {
        float4 r = red[0];
        z = dw{r.x, r.y};
        x = dw{r.z, r.w};
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            r = red[w];
            z = dw_add(z, dw{r.x, r.y});
            x = dw_add(x, dw{r.z, r.w});
        }
    }
}

struct RingView {
    const float4 *ring;
    int nt, nx, nz, head, cap;
    dw inv_dt, inv_dz;
};

// Per-thread sums of one chunk: the density_x term of the longitudinal
// integrand in double-word (it cancels: its terms sum to ~1/300 of their
// magnitude, so each term must be accurate well beyond FP32), the rest of
// the longitudinal integrand and the transverse one as Kahan-compensated
// FP32 sums.
struct ChunkSums {
    dw zx;
    float sz, cz, sx, cx;
};

// Integrand contribution of rows [i_lo, i_hi) x columns [0, C) of a chunk.
// Work unit = one s' column x MX_ROWBLK consecutive x' rows: a warp covers
// consecutive columns of one row block, so its gathers stay close in the
// history (neighbouring s' -> neighbouring cells) and the row records it
// reads are the same for all lanes (shared-memory broadcast).
//
// Per integrand point, in double-word: the distance from the perpendicular
// foot, |r - r'|^2 = rmin^2 + g (u - u*)^2 (no cancellation, unlike
// r0^2 + D near the source), its change from the column's reference row,
// delta = |r - r'| - r0, and the history coordinates t = t0 - delta / dt,
// z = z0 + delta / dz (a z shift reaches ~100 cells near the source, so an
// FP32 product would misplace the gather by ~1e-5 cell); then the density_x
// product chain w scale brx dx / |r - r'|.  The other terms are FP32.
#ifndef MX_INTEGRAL_ROWBLK
#define MX_INTEGRAL_ROWBLK 4
#endif
constexpr int MX_ROWBLK = MX_INTEGRAL_ROWBLK;
#ifndef MX_DXDW_REGIONS
#define MX_DXDW_REGIONS 2
#endif

template <bool DXDW>
__device__ __forceinline__ void chunk_points(const IntegralSmem &sm, const float4 *__restrict__ rows,
                                             const RingView &V, int i_lo, int i_hi, int C, ChunkSums &acc) {
    const int nblk = (i_hi - i_lo + MX_ROWBLK - 1) / MX_ROWBLK;
    const int units = nblk * C;
    const int tid = threadIdx.x;
    // (row block, column) of u = tid + k * MX_THREADS, advanced without division
    int rb = tid / C, jl = tid - (tid / C) * C;
    const int drb = MX_THREADS / C, dj = MX_THREADS - (MX_THREADS / C) * C;
    const uint32_t nzc = (uint32_t)V.nz * 2u;   // float4 per x row of a slot
    for (int u0 = tid; u0 < units; u0 += MX_THREADS) {
        const float4 *cr = sm.col + jl * (CW / 4);
        const int i0 = i_lo + rb * MX_ROWBLK;
        rb += drb;
        jl += dj;
        if (jl >= C) { jl -= C; rb += 1; }
        const float4 q7 = cr[7];
        const float ws = q7.y;
        if (ws == 0.f) continue;
        const float4 q0 = cr[0], q1 = cr[1], q2 = cr[2], q3 = cr[3];
        const int tcell = __float_as_int(q0.x), zcell = __float_as_int(q0.y);
        const dw toff{q0.z, q0.w}, zoff{q1.x, q1.y}, r0{q1.z, q1.w};
        const dw us{q2.x, q2.y}, rmin2{q2.z, q2.w};
        const float gm1 = q3.x, rho = q3.w;
        const dw K0x{q3.y, q3.z};
        const int iend = min(i0 + MX_ROWBLK, i_hi);
        for (int i = i0; i < iend; ++i) {
            const float4 *rr = rows + i * (RW / 4);
            const float4 ra = rr[0];
            const float4 rw = rr[1];
            const float wx = rw.x;
            if (wx == 0.f) continue;
            // |r - r'| and delta (double-word)
            const dw uu{ra.z, ra.w};
            const dw v = dw_sub_abs(uu, us);
            dw v2 = two_prod(v.hi, v.hi);
            v2.lo = __fmaf_rn(2.f * v.hi, v.lo, v2.lo);
            v2.lo = __fmaf_rn(gm1, v2.hi, v2.lo);            // g v^2, g = 1 + (g - 1)
            const dw r2 = dw_add_abs(rmin2, v2);             // both non-negative
            float inv_r;
            const dw rd = dw_sqrt_rsq(r2, &inv_r);
            const dw del = dw_sub_abs(rd, r0);
            // history coordinates: t shifts by ~1e-3 cell at most (FP32 product),
            // z by up to ~100 cells (double-word product)
            const float delf = dw_float(del);
            const dw ot = dw_add_f(toff, -__fmul_rn(delf, V.inv_dt.hi));
            const dw oz = dw_add_abs(zoff, dw_mul(del, V.inv_dz));
            int t0, t1, z0, z1;
            float td, zd, td_lo, zd_lo;
            if (!axis_split_dw(tcell, ot, V.nt, t0, t1, td, td_lo) ||
                !axis_split_dw(zcell, oz, V.nz, z0, z1, zd, zd_lo))
                continue;   // every field is zero outside the history grid
            // x: rows outside the history grid are not in [i_lo, i_hi)
            const int x0 = __float_as_int(ra.x);
            const float xd = ra.y;
            int s0 = V.head + t0, s1 = V.head + t1;
            if (s0 >= V.cap) s0 -= V.cap;
            if (s1 >= V.cap) s1 -= V.cap;
            if (!(bounds_ok(s0, V.cap, BS_MIXED_RING) && bounds_ok(s1, V.cap, BS_MIXED_RING) &&
                  bounds_ok(x0, V.nx, BS_MIXED_RING) &&
                  bounds_ok(x0 + __float_as_int(rw.y), V.nx, BS_MIXED_RING) &&
                  bounds_ok(z0, V.nz, BS_MIXED_RING) && bounds_ok(z1, V.nz, BS_MIXED_RING)))
                continue;
            const uint32_t c0x0 = ((uint32_t)s0 * (uint32_t)V.nx + (uint32_t)x0) * nzc + 2u * (uint32_t)z0;
            const uint32_t c1x0 = ((uint32_t)s1 * (uint32_t)V.nx + (uint32_t)x0) * nzc + 2u * (uint32_t)z0;
            const uint32_t dxc = (uint32_t)__float_as_int(rw.y) * nzc;
            const Fields5 F = gather5<DXDW>(V.ring, c0x0, c1x0, c0x0 + dxc, c1x0 + dxc,
                                      2u * (uint32_t)(z1 - z0), td, td_lo, xd, rw.w, zd, zd_lo);
            const float vr = F.vx.hi;
            const float4 q4 = cr[4], q5 = cr[5];
            // longitudinal double-word part: w scale (brx dx - (a + vx b) den
            // vx_x) / |r - r'|, with brx = K0x - vx (K1x + vx K2x) and
            // scale = 1 + x' rho applied once to the sum of the two terms
            const float dsc = __fmul_rn(rw.z, rho);
            const dw A = dw_sub_abs(K0x, dw_mul_f(F.vx, fmaf(vr, q5.y, q5.x + 1.f)));
            const dw w = two_prod(wx, ws);
            const dw wr = dw_mul(w, dw_recip_from(rd, inv_r));     // w / |r - r'|
            const float4 q6 = cr[6];
            const float scale = 1.f + dsc;
            const dw p1w = dw_add_f(dw{q4.x, q7.z}, __fmul_rn(vr, q4.y));
            const dw Dn = dw_neg(dw_mul(two_prod(F.den, F.vxx), p1w));
            // the two terms, the scale, one product with w / |r - r'| and one
            // accumulation (the sum's error is ~2^-48 of its terms)
            dw T = dw_add_abs(dw_mul(A, F.dx), Dn);
            T = dw_add_f(T, __fmul_rn(dsc, T.hi));
            acc.zx = dw_add_abs(acc.zx, dw_mul(T, wr));
            // density_z term (FP32)
            const float wf = wx * ws;
            const float brz = q5.z - vr * fmaf(vr, q6.x, q5.w);
            kahan(acc.sz, acc.cz, wf * (F.dz * brz * inv_r));
            // transverse integrand (FP32)
            const float uf = uu.hi;
            const float dxf = dw_float(F.dx);
            const float q1x = q6.y - uf * q6.z;
            const float M = q7.x - uf * q6.z - q6.w * delf;
            const float e = q4.z;
            const float pd = -(dxf * fmaf(vr, 1.f + gm1, e) + F.dz * __fdividef(fmaf(vr, e, q4.w), scale)) -
                             F.den * F.vxx;
            const float Ix = scale * inv_r * inv_r * (q1x * inv_r * F.den + pd * M);
            kahan(acc.sx, acc.cx, wf * Ix);
        }
    }
}

// Persistent: CTAs take points of the batch from a work counter.  Writes the
// FP64 region sums part[b][r][2].
//
// Launch shape: 128-thread CTAs capped at MX_INTEGRAL_MAXREG (120) registers
// per thread.  The kernel needs ~125 registers without spills and has none
// at 120; four CTAs then fit on an SM (16 warps) and leave 4096 of its 65,536
// registers to one 128-thread, 32-register CTA of the beam-moments kernel,
// which runs on a second stream beside the wake in a pipelined step loop.
// Measured per 4-region step of the chicane benchmark (integral, ms): three
// 256-thread CTAs at 80 registers (~240 bytes of spills per thread, a third
// of the kernel's L2 traffic) 2.09; two 256-thread CTAs at 120 registers
// 1.92; four 128-thread CTAs 1.76 (fewer warps wait at each unit-end
// barrier and four work units per SM stage their records independently);
// 96- or 64-thread CTAs 1.87 / 1.93; five 128-thread CTAs at 96 registers
// (136 bytes of spills; the same 4096 registers left over) 1.79.  128
// registers leave no room for the moments CTA, which then waits for the
// whole integral.  Defining
// MX_INTEGRAL_MAXREG as 0 selects __launch_bounds__ with
// MX_INTEGRAL_BLOCKS CTAs per SM instead.
#ifndef MX_INTEGRAL_MAXREG
#define MX_INTEGRAL_MAXREG 120
#endif
#ifndef MX_INTEGRAL_BLOCKS
#define MX_INTEGRAL_BLOCKS 3
#endif
#if MX_INTEGRAL_MAXREG > 0
__global__ void __maxnreg__(MX_INTEGRAL_MAXREG)
#else
__global__ void __launch_bounds__(MX_THREADS, MX_INTEGRAL_BLOCKS)
#endif
mixed_integral(const dfcsr_wake_job *__restrict__ jobs, const int32_t *__restrict__ job_of_point,
               int64_t first, int64_t count, size_t rec_words, const float *__restrict__ rec,
               const PointMeta *__restrict__ meta, const int2 *__restrict__ rows_valid,
               double *__restrict__ part, unsigned long long *__restrict__ counter) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    IntegralSmem &sm = *reinterpret_cast<IntegralSmem *>(smem_raw);
    float4 *rows = reinterpret_cast<float4 *>(smem_raw + kIntegralRowOff);
    const int tid = threadIdx.x;
    // work unit = one integration region of one point (unit u: point
    // u / WAKE_MAX_REGIONS, region u % WAKE_MAX_REGIONS), so that the CTAs
    // finish a batch together (a region is a quarter to a half of a point).
    // Region-major order instead (all far regions first, so that the last
    // units of a launch are the small ones) measured 2 % slower per 4-region
    // step (1.747 vs 1.715 ms).
    // The next unit's index is taken while the current one runs, so the
    // atomic's latency is off the CTA's critical path: slot par holds the
    // current unit, slot par ^ 1 receives the next before the unit-end
    // barrier, and every thread has read slot par before thread 0 reuses it
    // one unit later.
    if (tid == 0) sm.pt[0] = (long long)atomicAdd(counter, 1ull);
    __syncthreads();
    for (int par = 0;; par ^= 1) {
        const int64_t u = sm.pt[par];
        if (u >= count * WAKE_MAX_REGIONS) break;
        if (tid == 0) sm.pt[par ^ 1] = (long long)atomicAdd(counter, 1ull);
        const int64_t b = u / WAKE_MAX_REGIONS;
        const int r = (int)(u - b * WAKE_MAX_REGIONS);
        // PointMeta is read field by field: a local copy indexed by r would
        // live in local memory
        const PointMeta *m = meta + b;
        const int nreg = m->valid ? m->nreg : 0;
        if (r < nreg) {
            const dfcsr_wake_job &J = jobs[job_of_point ? job_of_point[first + b] : 0];
            const float *base = rec + (size_t)b * rec_words;
            RingView V;
            V.ring = reinterpret_cast<const float4 *>(J.ring32);
            V.nt = J.nt; V.nx = J.nx; V.nz = J.nz; V.head = J.head; V.cap = J.cap;
            V.inv_dt = dw{m->inv_dt_hi, m->inv_dt_lo};
            V.inv_dz = dw{m->inv_dz_hi, m->inv_dz_lo};
            const RegionMeta R = m->reg[r];
            int2 rv = rows_valid[b * WAKE_MAX_REGIONS + r];
            if (rv.y > rv.x &&
                !(bounds_ok(rv.x, R.nxp, BS_MIXED_ROWS) && bounds_ok(rv.y - 1, R.nxp, BS_MIXED_ROWS) &&
                  bounds_ok((long long)R.row_off + (long long)R.nxp * RW - 1, (long long)rec_words, BS_MIXED_REC) &&
                  bounds_ok((long long)R.col_off + (long long)R.nsp * CW - 1, (long long)rec_words, BS_MIXED_REC)))
                rv.y = rv.x;   // checked build: skip the region
            dw reg_z{0.f, 0.f}, reg_x{0.f, 0.f};
            if (rv.y > rv.x) {
                const float4 *rb = reinterpret_cast<const float4 *>(base + R.row_off);
                for (int k = tid; k < R.nxp * (RW / 4); k += blockDim.x) rows[k] = rb[k];
                for (int j0 = 0; j0 < R.nsp; j0 += MX_CHUNK) {
                    const int C = min(MX_CHUNK, R.nsp - j0);
                    const float4 *cb = reinterpret_cast<const float4 *>(base + R.col_off) + (size_t)j0 * (CW / 4);
                    for (int k = tid; k < C * (CW / 4); k += blockDim.x) sm.col[k] = cb[k];
                    __syncthreads();
                    ChunkSums acc{dw{0.f, 0.f}, 0.f, 0.f, 0.f, 0.f};
                    // regions below MX_DXDW_REGIONS (0 far, 1 middle):
                    // density_x's terms cancel to ~1/300 of their size there
                    if (r < MX_DXDW_REGIONS)
                        chunk_points<true>(sm, rows, V, rv.x, rv.y, C, acc);
                    else
                        chunk_points<false>(sm, rows, V, rv.x, rv.y, C, acc);
                    // Kahan state s - c exactly as a double-word
                    dw bz = dw_add(acc.zx, two_sum(acc.sz, -acc.cz)), bx = two_sum(acc.sx, -acc.cx);
                    block_sum2_dw(bz, bx, sm.red);
                    if (tid == 0) { reg_z = dw_add(reg_z, bz); reg_x = dw_add(reg_x, bx); }
                    __syncthreads();
                }
            }
            if (tid == 0) {
                const double wd = (double)m->wdelta[r];
                const double vz = dw_to_double(reg_z), vx = dw_to_double(reg_x);
                part[((size_t)b * WAKE_MAX_REGIONS + r) * 2 + 0] = fma(vz, wd, vz);
                part[((size_t)b * WAKE_MAX_REGIONS + r) * 2 + 1] = fma(vx, wd, vx);
            }
        }
        __syncthreads();
    }
}

// FP64 near-source band: one CTA per (point, region), threads over band columns.
__global__ void __launch_bounds__(128)
mixed_band(const dfcsr_wake_job *__restrict__ jobs, const int32_t *__restrict__ job_of_point,
           const double *__restrict__ S, const double *__restrict__ X, int64_t first, int64_t count,
           const PointMeta *__restrict__ meta, const double *__restrict__ obs_vx,
           double *__restrict__ band) {
    __shared__ double red[4];
    const int64_t b = blockIdx.x;
    const int r = blockIdx.y;
    if (b >= count) return;
    const PointMeta *m = meta + b;
    double az = 0.0, ax = 0.0;
    if (m->valid && r < m->nreg) {
        const int64_t pt = first + b;
        const dfcsr_wake_job &J = jobs[job_of_point ? job_of_point[pt] : 0];
        if (J.near_band > 0.0) {
            ObsConst o;
            o.t = J.position; o.s = S[pt]; o.x = X[pt]; o.vx = obs_vx[b];
            double lat_s[6];
            lattice_lerp(J, o.s, lat_s);
            o.X0s = lat_s[0]; o.Y0s = lat_s[1]; o.nsx = lat_s[2]; o.nsy = lat_s[3];
            o.tsx = lat_s[4]; o.tsy = lat_s[5];
            Region reg[WAKE_MAX_REGIONS];
            wake_regions(J, o.s, o.x, reg);
            const Region R = reg[r];
            const Axis ax_s = make_axis(R.sl, R.sr, R.nsp);
            const Axis ax_x = make_axis(R.xl, R.xr, R.nxp);
            for (int j = threadIdx.x; j < R.nsp; j += blockDim.x) {
                const double spj = ax_s.at(j);   // same s' as the geometry kernel
                if (!(fabs(spj - o.s) < J.near_band)) continue;
                const double ws = ax_s.weight(j);
                double L[6];
                lattice_lerp(J, spj, L);
                const double rho_sp = rho_at(J, spj);
                for (int i = 0; i < R.nxp; ++i) {
                    const double xpi = ax_x.at(i);
                    double Iz, Ix;
                    integrand_fp64(J, o, L, rho_sp, spj, xpi, Iz, Ix);
                    const double w = ax_x.weight(i) * ws;
                    az += w * Iz;
                    ax += w * Ix;
                }
            }
        }
    }
    az = block_sum(az, red);
    ax = block_sum(ax, red);
    if (threadIdx.x == 0) {
        band[((size_t)b * WAKE_MAX_REGIONS + r) * 2 + 0] = az;
        band[((size_t)b * WAKE_MAX_REGIONS + r) * 2 + 1] = ax;
    }
}

__global__ void mixed_finalize(const dfcsr_wake_job *__restrict__ jobs, const int32_t *__restrict__ job_of_point,
                               int64_t first, int64_t count, const PointMeta *__restrict__ meta,
                               const double *__restrict__ part, const double *__restrict__ band,
                               double *__restrict__ dE, double *__restrict__ xkick) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= count) return;
    const int64_t pt = first + b;
    const dfcsr_wake_job &J = jobs[job_of_point ? job_of_point[pt] : 0];
    const PointMeta *m = meta + b;
    if (!m->valid) {
        dE[pt] = __longlong_as_double(0x7ff8000000000000ll);
        xkick[pt] = __longlong_as_double(0x7ff8000000000000ll);
        return;
    }
    double se = 0.0, sx = 0.0;
    for (int r = 0; r < m->nreg; ++r) {
        const size_t k = ((size_t)b * WAKE_MAX_REGIONS + r) * 2;
        const double vz = part[k] + (band ? band[k] : 0.0);
        const double vx = part[k + 1] + (band ? band[k + 1] : 0.0);
        const double e = -J.csr_scaling * vz, q = J.csr_scaling * vx;
        se = (r == 0) ? e : se + e;
        sx = (r == 0) ? q : sx + q;
    }
    dE[pt] = se;
    xkick[pt] = sx;
}

struct MixedLayout {
    size_t rec_words;
    int64_t batch;
    int64_t setup_pts;   // points per set-up launch (a whole number of batches)
};

constexpr int SETUP_BATCHES = 4;

// Records of a batch: large batches (one for a 64^2 mesh) leave fewer
// end-of-batch tails of the persistent integral than L2-sized ones (96 MiB:
// three batches, 0.81 vs 0.70 ms for the integral of a step); the records
// are read once from HBM, which the integral's few-% DRAM use absorbs.
static const size_t kMixedScratchTarget = (size_t)1 << 30;

static MixedLayout mixed_layout(int xbins_max, int zbins_max, int64_t n) {
    MixedLayout L;
    L.rec_words = point_record_words(xbins_max, zbins_max);
    const int64_t per = (int64_t)(L.rec_words * sizeof(float) + sizeof(PointMeta) +
                                  2 * 2 * WAKE_MAX_REGIONS * sizeof(double) +
                                  WAKE_MAX_REGIONS * sizeof(int2) + sizeof(double) + 64);
    int64_t batch = (int64_t)(kMixedScratchTarget / per);
    if (batch < 1) batch = 1;
    if (batch > n) batch = n;
    L.batch = batch;
    L.setup_pts = (n < SETUP_BATCHES * batch) ? n : SETUP_BATCHES * batch;
    return L;
}

static size_t mixed_carve(Carver &c, const MixedLayout &L, unsigned long long **counter, float **rec,
                          PointMeta **meta, int2 **rows, double **part, double **band,
                          double **obs_vx, GeoShared **setup, dfcsr_wake_job **jobslot) {
    *counter = c.take<unsigned long long>(4);
    *jobslot = c.take<dfcsr_wake_job>(1);
    *setup = c.take<GeoShared>((size_t)L.setup_pts);
    *rec = c.take<float>((size_t)L.batch * L.rec_words);
    *meta = c.take<PointMeta>((size_t)L.batch);
    *rows = c.take<int2>((size_t)L.batch * WAKE_MAX_REGIONS);
    *part = c.take<double>((size_t)L.batch * WAKE_MAX_REGIONS * 2);
    *band = c.take<double>((size_t)L.batch * WAKE_MAX_REGIONS * 2);
    *obs_vx = c.take<double>((size_t)L.batch);
    return c.used;
}

// Launch set-up of the integral kernel, per device (the shared-memory
// attribute is a per-device setting, the occupancy depends on the device):
// one entry per device ordinal, filled on the device's first call.
struct IntegralDevState {
    bool attr;
    size_t smem;
    int blocks;
};
constexpr int kMaxDevices = 64;
static std::mutex g_integral_mu;
static IntegralDevState g_integral_dev[kMaxDevices];

static int integral_setup(size_t smem, int *blocks) {
    int dev = 0;
    DFCSR_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("dfcsr_wake_mixed: device ordinal %d out of range", dev);
        return DFCSR_BAD_ARG;
    }
    std::lock_guard<std::mutex> g(g_integral_mu);
    IntegralDevState &d = g_integral_dev[dev];
    if (!d.attr) {
        DFCSR_CUDA_TRY(cudaFuncSetAttribute(mixed_integral, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)integral_smem_bytes(MX_MAX_ROWS)));
        d.attr = true;
    }
    if (d.blocks == 0 || d.smem != smem) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mixed_integral, MX_THREADS, smem) !=
                cudaSuccess || per_sm < 1)
            per_sm = 1;
        d.blocks = per_sm * num_sms();
        d.smem = smem;
    }
    *blocks = d.blocks;
    return DFCSR_OK;
}

}  // namespace dfcsr

using namespace dfcsr;

extern "C" size_t dfcsr_wake_workspace_bytes(int xbins_max, int zbins_max, int64_t n) {
    if (xbins_max < 1 || zbins_max < 1 || n < 0) return 0;
    const MixedLayout L = mixed_layout(xbins_max, zbins_max, n > 0 ? n : 1);
    Carver c{nullptr, 0, 0};
    unsigned long long *a;
    float *b;
    PointMeta *m;
    int2 *rw;
    double *p, *q, *v;
    GeoShared *g;
    dfcsr_wake_job *j;
    return mixed_carve(c, L, &a, &b, &m, &rw, &p, &q, &v, &g, &j) + 256;
}

namespace dfcsr {
// One job passed by value (a kernel parameter) into its workspace slot.
__global__ void store_job(dfcsr_wake_job job, dfcsr_wake_job *__restrict__ out) {
    if (threadIdx.x == 0) *out = job;
}
}  // namespace dfcsr

// The mixed wake over n points: jobs in device memory (`jobs`, with
// `job_of_point`), or one job from host memory (`job_host`), stored into the
// workspace by the first kernel of the stream.
static int wake_mixed_run(const dfcsr_wake_job *jobs, const dfcsr_wake_job *job_host,
                          const int32_t *job_of_point, const double *s, const double *x, int64_t n,
                          int xbins_max, int zbins_max, int use_band, double *dE, double *xkick,
                          void *workspace, size_t workspace_bytes, void *stream) {
    DFCSR_CHECK_ARG(n >= 0, "dfcsr_wake_mixed: negative point count");
    if (n == 0) return DFCSR_OK;
    DFCSR_CHECK_ARG((jobs || job_host) && s && x && dE && xkick, "dfcsr_wake_mixed: null pointer");
    DFCSR_CHECK_ARG(xbins_max >= 1 && 2 * xbins_max <= MX_MAX_ROWS,
                    "dfcsr_wake_mixed: xbins must be in [1, %d] (got %d)", MX_MAX_ROWS / 2, xbins_max);
    DFCSR_CHECK_ARG(zbins_max >= 1 && zbins_max <= MX_MAX_COLS,
                    "dfcsr_wake_mixed: zbins must be in [1, %d] (got %d)", MX_MAX_COLS, zbins_max);
    const MixedLayout L = mixed_layout(xbins_max, zbins_max, n);
    Carver c{reinterpret_cast<char *>(workspace), workspace_bytes, 0};
    unsigned long long *counter;
    float *rec;
    PointMeta *meta;
    int2 *rows;
    double *part, *band, *obs_vx;
    GeoShared *setup;
    dfcsr_wake_job *jobslot;
    mixed_carve(c, L, &counter, &rec, &meta, &rows, &part, &band, &obs_vx, &setup, &jobslot);
    if (!workspace || !c.ok()) {
        set_error("dfcsr_wake_mixed: workspace too small (%zu < %zu)", workspace_bytes, c.used);
        return DFCSR_OOM;
    }
    cudaStream_t st = as_stream(stream);
    if (job_host) {
        note_launch();
        store_job<<<1, 32, 0, st>>>(*job_host, jobslot);
        jobs = jobslot;
        job_of_point = nullptr;
    }
    const int max_rows = 2 * xbins_max;
    const size_t smem = integral_smem_bytes(max_rows);
    int blocks_max = 0;
    {
        const int rc = integral_setup(smem, &blocks_max);
        if (rc != DFCSR_OK) return rc;
    }
    int64_t setup_first = 0, setup_count = 0;
    for (int64_t first = 0; first < n; first += L.batch) {
        const int64_t count = (n - first < L.batch) ? n - first : L.batch;
        DFCSR_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st));
        {
            ScopedTiming tm("wake_mixed_geometry", st);
            if (first + count > setup_first + setup_count) {   // next set-up chunk
                setup_first = first;
                setup_count = (n - first < L.setup_pts) ? n - first : L.setup_pts;
                note_launch();
                mixed_setup<<<(unsigned)setup_count, SETUP_THREADS, 0, st>>>(
                    jobs, job_of_point, s, x, setup_first, setup_count, L.rec_words, max_rows, setup);
            }
            note_launch();
            mixed_geometry<<<(unsigned)count, GEO_THREADS, 0, st>>>(
                jobs, job_of_point, s, x, first, count, setup + (first - setup_first), L.rec_words, rec,
                meta, rows, obs_vx);
        }
        const int blocks = (int)((int64_t)blocks_max < count ? blocks_max : count);
        {
            ScopedTiming tm("wake_mixed_integral", st);
            note_launch();
            mixed_integral<<<blocks, MX_THREADS, smem, st>>>(
                jobs, job_of_point, first, count, L.rec_words, rec, meta, rows, part, counter);
        }
        if (use_band) {
            ScopedTiming tm("wake_mixed_band", st);
            note_launch();
            mixed_band<<<dim3((unsigned)count, WAKE_MAX_REGIONS), 128, 0, st>>>(
                jobs, job_of_point, s, x, first, count, meta, obs_vx, band);
        }
        note_launch();
        mixed_finalize<<<(unsigned)((count + 127) / 128), 128, 0, st>>>(
            jobs, job_of_point, first, count, meta, part, use_band ? band : nullptr, dE, xkick);
    }
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}

extern "C" int dfcsr_wake_mixed(const dfcsr_wake_job *jobs, const int32_t *job_of_point,
                                const double *s, const double *x, int64_t n, int xbins_max,
                                int zbins_max, int use_band, double *dE, double *xkick,
                                void *workspace, size_t workspace_bytes, void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(n == 0 || jobs, "dfcsr_wake_mixed: null pointer");
    return wake_mixed_run(jobs, nullptr, job_of_point, s, x, n, xbins_max, zbins_max, use_band, dE,
                          xkick, workspace, workspace_bytes, stream);
}

extern "C" int dfcsr_wake_mixed_job(const dfcsr_wake_job *job, const double *s, const double *x,
                                    int64_t n, int xbins_max, int zbins_max, int use_band, double *dE,
                                    double *xkick, void *workspace, size_t workspace_bytes,
                                    void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(n == 0 || job, "dfcsr_wake_mixed_job: null job");
    DFCSR_CHECK_ARG(n == 0 || ring32_offsets_fit(job->cap, job->nx, job->nz),
                    "dfcsr_wake_mixed_job: the FP32 history ring (%d slots of %d x %d cells) exceeds "
                    "the 64 GiB its 32-bit cell offsets address", job->cap, job->nx, job->nz);
    return wake_mixed_run(nullptr, job, nullptr, s, x, n, xbins_max, zbins_max, use_band, dE, xkick,
                          workspace, workspace_bytes, stream);
}

DFCSR_BOUNDS_READER(wake_mixed)
