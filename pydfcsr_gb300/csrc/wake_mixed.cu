// Mixed-precision CSR wake (FP32 bulk, FP64 retarded geometry).
//
// Same integral as get_CSR_wake / get_CSR_integrand (pyDFCSR_2D/CSR.py:454-782),
// restructured so that FP32 is safe:
//  * geometry kernel (FP64), one thread per (observation point, region, s'
//    column): orbit tables at s', separation R0 = r - r' at a reference x'
//    (the region centre), |R0|, the history coordinates of t_ret and
//    s' - t_ret, and every direction product whose difference would cancel in
//    FP32 (v.tau', v.n', 1 - |tau'|^2, (r - r').(n - n'), ...).  Records are
//    written for a batch of points small enough to stay resident in L2.
//  * integral kernel (FP32), one persistent CTA loop over points: per
//    (x', s') only an FP32 correction remains,
//        |r - r'| = r0 + delta,  delta = D / (r0 + sqrt(r0^2 + D)),
//        D = u (|n'|^2 u - 2 R0.n'),  u = x' - x'_ref   (no cancellation);
//    history coordinates are an integer cell (from FP64) plus an FP32
//    offset, so a grid index near 1000 keeps ~1e-7 cell resolution; gathers
//    and the integrand are FP32 with Kahan-compensated per-thread sums and a
//    fixed-order FP64 block reduction.
//  * band kernel (FP64, optional): s' columns with |s' - s| < near_band are
//    skipped by the integral kernel and evaluated with the FP64 integrand.
//  * finalize kernel: adds the regions in the reference's order and scales.
#include "wake_common.cuh"

namespace dfcsr {

constexpr int MX_THREADS = 256;
constexpr int MX_CHUNK = 128;       // s' columns staged in shared memory at once
constexpr int MX_MAX_ROWS = 1024;   // x' rows per region (2 * xbins)
constexpr int MX_MAX_COLS = 4096;   // s' columns per region (zbins)
constexpr int GEO_THREADS = 128;

// column record: 24 words (SoA within a region)
enum ColField {
    C_TB, C_ZB, C_TF, C_ZF, C_R0, C_BG, C_CG, C_A, C_B, C_E, C_G, C_H,
    C_K0X, C_K1X, C_K2X, C_K0Z, C_K1Z, C_K2Z, C_Q0, C_Q1, C_Q2, C_M0, C_RHO, C_WS, C_NF
};
// row record: 5 words
enum RowField { R_XB, R_XF, R_U, R_XP, R_WX, R_NF };

struct RegionMeta {
    int nxp, nsp, col_off, row_off;   // offsets in words within the point record
};

struct PointMeta {
    int nreg, valid;
    RegionMeta reg[WAKE_MAX_REGIONS];
};

// Per-point record size (words) for a job: 4 regions of zbins columns and at
// most 5 * xbins rows in total.
__host__ __device__ inline size_t point_record_words(int xbins, int zbins) {
    return (size_t)WAKE_MAX_REGIONS * zbins * C_NF + (size_t)5 * xbins * R_NF;
}

__device__ __forceinline__ void put_i(float *base, int field, int stride, int idx, int v) {
    base[(size_t)field * stride + idx] = __int_as_float(v);
}
__device__ __forceinline__ void put_f(float *base, int field, int stride, int idx, double v) {
    base[(size_t)field * stride + idx] = (float)v;
}
__device__ __forceinline__ int clamp_int(double v) { return (int)fmax(fmin(v, 2.0e9), -2.0e9); }

// grid (points in batch, regions); block GEO_THREADS over columns then rows.
__global__ void __launch_bounds__(GEO_THREADS)
mixed_geometry(const dfcsr_wake_job *__restrict__ jobs, const int32_t *__restrict__ job_of_point,
               const double *__restrict__ S, const double *__restrict__ X, int64_t first, int64_t count,
               size_t rec_words, float *__restrict__ rec, PointMeta *__restrict__ meta,
               double *__restrict__ obs_vx) {
    const int64_t b = blockIdx.x;
    const int64_t pt = first + b;
    const int r = blockIdx.y;
    if (b >= count) return;
    const dfcsr_wake_job &J = jobs[job_of_point ? job_of_point[pt] : 0];
    const double t = J.position, s = S[pt], x = X[pt];
    Region reg[WAKE_MAX_REGIONS];
    const int nreg = wake_regions(J, s, x, reg);
    float *base = rec + (size_t)b * rec_words;
    // layout offsets (same computation in every block of this point)
    int off = 0;
    RegionMeta rm[WAKE_MAX_REGIONS];
    bool ok = true;
    for (int k = 0; k < nreg; ++k) {
        rm[k].nxp = reg[k].nxp;
        rm[k].nsp = reg[k].nsp;
        rm[k].col_off = off;
        off += reg[k].nsp * C_NF;
        rm[k].row_off = off;
        off += reg[k].nxp * R_NF;
        if (reg[k].nxp < 1 || reg[k].nxp > MX_MAX_ROWS || reg[k].nsp < 1 || reg[k].nsp > MX_MAX_COLS)
            ok = false;
    }
    if ((size_t)off > rec_words) ok = false;
    if (r == 0 && threadIdx.x == 0) {
        PointMeta m;
        m.nreg = nreg;
        m.valid = ok ? 1 : 0;
        for (int k = 0; k < WAKE_MAX_REGIONS; ++k) m.reg[k] = (k < nreg) ? rm[k] : RegionMeta{0, 0, 0, 0};
        meta[b] = m;
    }
    if (!ok || r >= nreg) return;
    const Region R = reg[r];
    const double vx_obs = hist_field_fp64(J, 3, t, x, s - t);
    if (r == 0 && threadIdx.x == 0) obs_vx[b] = vx_obs;
    double lat_s[6];
    lattice_lerp(J, s, lat_s);
    const double X0s = lat_s[0], Y0s = lat_s[1], nsx = lat_s[2], nsy = lat_s[3];
    const double vxo = lat_s[4] + vx_obs * nsx, vyo = lat_s[5] + vx_obs * nsy;
    const double xref = np_linspace_at(R.xl, R.xr, R.nxp, R.nxp / 2);
    float *cb = base + rm[r].col_off;
    const int cs = R.nsp;
    for (int j = threadIdx.x; j < R.nsp; j += blockDim.x) {
        const double spj = np_linspace_at(R.sl, R.sr, R.nsp, j);
        double L[6];
        lattice_lerp(J, spj, L);
        const double npx = L[2], npy = L[3], tpx = L[4], tpy = L[5];
        const double Ax = X0s - L[0] + x * nsx, Ay = Y0s - L[1] + x * nsy;
        const double rx0 = Ax - xref * npx, ry0 = Ay - xref * npy;
        const double r0 = sqrt(rx0 * rx0 + ry0 * ry0);
        const double ut0 = (t - r0 - J.t_min) / J.t_delta;
        const double uz0 = (spj - (t - r0) - J.z_min) / J.z_delta;
        const double tfl = floor(ut0), zfl = floor(uz0);
        put_i(cb, C_TB, cs, j, clamp_int(tfl));
        put_i(cb, C_ZB, cs, j, clamp_int(zfl));
        put_f(cb, C_TF, cs, j, ut0 - tfl);
        put_f(cb, C_ZF, cs, j, uz0 - zfl);
        put_f(cb, C_R0, cs, j, r0);
        put_f(cb, C_BG, cs, j, rx0 * npx + ry0 * npy);
        put_f(cb, C_CG, cs, j, npx * npx + npy * npy);
        const double a = vxo * tpx + vyo * tpy, bb = vxo * npx + vyo * npy;
        const double e = tpx * npx + tpy * npy, g = npx * npx + npy * npy;
        const double h = tpx * tpx + tpy * tpy;
        put_f(cb, C_A, cs, j, a);
        put_f(cb, C_B, cs, j, bb);
        put_f(cb, C_E, cs, j, e);
        put_f(cb, C_G, cs, j, g);
        put_f(cb, C_H, cs, j, h);
        put_f(cb, C_K0X, cs, j, bb - a * e);
        put_f(cb, C_K1X, cs, j, (a * g - 1.0) + bb * e);   // K1x - 1 (K1x ~ 1)
        put_f(cb, C_K2X, cs, j, bb * g);
        put_f(cb, C_K0Z, cs, j, a * (1.0 - h));
        put_f(cb, C_K1Z, cs, j, a * e + bb * h);
        put_f(cb, C_K2Z, cs, j, bb * e);
        const double nmx = nsx - npx, nmy = nsy - npy;
        const double Q0 = rx0 * nmx + ry0 * nmy;
        const double q2 = nsx * tpx + nsy * tpy;
        put_f(cb, C_Q0, cs, j, Q0);
        put_f(cb, C_Q1, cs, j, npx * nmx + npy * nmy);
        put_f(cb, C_Q2, cs, j, q2);
        put_f(cb, C_M0, cs, j, Q0 - q2 * r0);
        put_f(cb, C_RHO, cs, j, rho_at(J, spj));
        const double dl = (j > 0) ? spj - np_linspace_at(R.sl, R.sr, R.nsp, j - 1) : 0.0;
        const double dr = (j < R.nsp - 1) ? np_linspace_at(R.sl, R.sr, R.nsp, j + 1) - spj : 0.0;
        const bool near = J.near_band > 0.0 && fabs(spj - s) < J.near_band;
        put_f(cb, C_WS, cs, j, near ? 0.0 : 0.5 * (dl + dr));   // band columns: FP64 kernel
    }
    float *rb = base + rm[r].row_off;
    const int rs = R.nxp;
    for (int i = threadIdx.x; i < R.nxp; i += blockDim.x) {
        const double xpi = np_linspace_at(R.xl, R.xr, R.nxp, i);
        const double ux = (xpi - J.x_min) / J.x_delta;
        const double fb = floor(ux);
        put_i(rb, R_XB, rs, i, clamp_int(fb));
        put_f(rb, R_XF, rs, i, ux - fb);
        put_f(rb, R_U, rs, i, xpi - xref);
        put_f(rb, R_XP, rs, i, xpi);
        const double dl = (i > 0) ? xpi - np_linspace_at(R.xl, R.xr, R.nxp, i - 1) : 0.0;
        const double dr = (i < R.nxp - 1) ? np_linspace_at(R.xl, R.xr, R.nxp, i + 1) - xpi : 0.0;
        put_f(rb, R_WX, rs, i, 0.5 * (dl + dr));
    }
}

// Resolve one axis from an integer base and an FP32 offset with the
// reference's int() truncation rule (in range iff -1 < u < n).
__device__ __forceinline__ bool axis_split(int base, float off, int n, int &i0, int &i1, float &w) {
    const float k = floorf(off);
    const int ui = base + (int)k;
    const float fr = off - k;
    if (!(ui > -1 || (ui == -1 && fr > 0.f)) || ui >= n) return false;
    if (ui == -1) { i0 = 0; w = fr - 1.f; }
    else { i0 = ui; w = fr; }
    i1 = (i0 == n - 1) ? i0 : i0 + 1;
    return true;
}

struct Fields5 {
    float den, dx, dz, vx, vxx;
};

// Error-free transformations (round-to-nearest intrinsics: never contracted).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Linear interpolation a + w (b - a) of float-float values (hi, lo).
__device__ __forceinline__ float2 lerp_ff(float2 A, float2 B, float w) {
    float dh, de;
    two_sum(B.x, -A.x, dh, de);
    const float dl = __fadd_rn(de, __fsub_rn(B.y, A.y));
    const float ph = __fmul_rn(w, dh);
    const float pe = __fmaf_rn(w, dh, -ph);
    const float pl = __fmaf_rn(w, dl, pe);
    float rh, re;
    two_sum(A.x, ph, rh, re);
    const float rl = __fadd_rn(re, __fadd_rn(A.y, pl));
    const float s = __fadd_rn(rh, rl);
    return make_float2(s, __fsub_rn(rl, __fsub_rn(s, rh)));
}

// a + w (b - a) with one rounding for the product-add.
__device__ __forceinline__ float lerp1(float a, float b, float w) { return fmaf(w, b - a, a); }

// Trilinear FP32 gather of the five fields from ring32 [slot][nx][nz][8]
// (cell: den, dx_hi, dz, vx | vxx, dx_lo, 0, 0), interpolating t, then x,
// then z like the reference; density_x in float-float.
__device__ __forceinline__ Fields5 gather5(const float *__restrict__ ring, int nx, int nz, int s0, int s1,
                                           float td, int x0, int x1, float xd, int z0, int z1, float zd) {
    const size_t nxz = (size_t)nx * nz;
    const size_t dz8 = (size_t)(z1 - z0) * 8;
    const float4 *p00 = reinterpret_cast<const float4 *>(ring + ((size_t)s0 * nxz + (size_t)x0 * nz + z0) * 8);
    const float4 *q00 = reinterpret_cast<const float4 *>(ring + ((size_t)s1 * nxz + (size_t)x0 * nz + z0) * 8);
    const float4 *p10 = reinterpret_cast<const float4 *>(ring + ((size_t)s0 * nxz + (size_t)x1 * nz + z0) * 8);
    const float4 *q10 = reinterpret_cast<const float4 *>(ring + ((size_t)s1 * nxz + (size_t)x1 * nz + z0) * 8);
    const size_t dz4 = dz8 / 4;
    // corner order: [x][z][t]
    const float4 A0 = __ldg(p00), a0 = __ldg(p00 + 1), A1 = __ldg(p00 + dz4), a1 = __ldg(p00 + dz4 + 1);
    const float4 B0 = __ldg(q00), b0 = __ldg(q00 + 1), B1 = __ldg(q00 + dz4), b1 = __ldg(q00 + dz4 + 1);
    const float4 C0 = __ldg(p10), c0 = __ldg(p10 + 1), C1 = __ldg(p10 + dz4), c1 = __ldg(p10 + dz4 + 1);
    const float4 D0 = __ldg(q10), d0 = __ldg(q10 + 1), D1 = __ldg(q10 + dz4), d1 = __ldg(q10 + dz4 + 1);
    auto tri = [&](float v00a, float v00b, float v01a, float v01b, float v10a, float v10b,
                   float v11a, float v11b) -> float {
        const float c00 = lerp1(v00a, v00b, td);
        const float c01 = lerp1(v01a, v01b, td);
        const float c10 = lerp1(v10a, v10b, td);
        const float c11 = lerp1(v11a, v11b, td);
        const float e0 = lerp1(c00, c10, xd);
        const float e1 = lerp1(c01, c11, xd);
        return lerp1(e0, e1, zd);
    };
    Fields5 r;
    r.den = tri(A0.x, B0.x, A1.x, B1.x, C0.x, D0.x, C1.x, D1.x);
    r.dz = tri(A0.z, B0.z, A1.z, B1.z, C0.z, D0.z, C1.z, D1.z);
    r.vx = tri(A0.w, B0.w, A1.w, B1.w, C0.w, D0.w, C1.w, D1.w);
    r.vxx = tri(a0.x, b0.x, a1.x, b1.x, c0.x, d0.x, c1.x, d1.x);
    {
        const float2 c00 = lerp_ff(make_float2(A0.y, a0.y), make_float2(B0.y, b0.y), td);
        const float2 c01 = lerp_ff(make_float2(A1.y, a1.y), make_float2(B1.y, b1.y), td);
        const float2 c10 = lerp_ff(make_float2(C0.y, c0.y), make_float2(D0.y, d0.y), td);
        const float2 c11 = lerp_ff(make_float2(C1.y, c1.y), make_float2(D1.y, d1.y), td);
        const float2 e0 = lerp_ff(c00, c10, xd);
        const float2 e1 = lerp_ff(c01, c11, xd);
        const float2 f = lerp_ff(e0, e1, zd);
        r.dx = __fadd_rn(f.x, f.y);
    }
    return r;
}

__device__ __forceinline__ void kahan(float &s, float &c, float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

struct IntegralSmem {
    float col[C_NF][MX_CHUNK];
    float row[R_NF][MX_MAX_ROWS];
    double red[MX_THREADS / 32];
    long long pt;
};

// Persistent: CTAs take points of the batch from a work counter.  Writes the
// FP64 region sums part[b][r][2].
__global__ void __launch_bounds__(MX_THREADS, 3)
mixed_integral(const dfcsr_wake_job *__restrict__ jobs, const int32_t *__restrict__ job_of_point,
               int64_t first, int64_t count, size_t rec_words, const float *__restrict__ rec,
               const PointMeta *__restrict__ meta, double *__restrict__ part,
               unsigned long long *__restrict__ counter) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    IntegralSmem &sm = *reinterpret_cast<IntegralSmem *>(smem_raw);
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) sm.pt = (long long)atomicAdd(counter, 1ull);
        __syncthreads();
        const int64_t b = sm.pt;
        if (b >= count) break;
        const dfcsr_wake_job &J = jobs[job_of_point ? job_of_point[first + b] : 0];
        const PointMeta m = meta[b];
        const float *base = rec + (size_t)b * rec_words;
        const float inv_dt = (float)(1.0 / J.t_delta), inv_dz = (float)(1.0 / J.z_delta);
        const float *ring = J.ring32;
        const int nt = J.nt, nx = J.nx, nz = J.nz, head = J.head, cap = J.cap;
        for (int r = 0; r < m.nreg && m.valid; ++r) {
            const RegionMeta R = m.reg[r];
            const float *rb = base + R.row_off;
            for (int k = tid; k < R.nxp * R_NF; k += blockDim.x) {
                const int f = k / R.nxp, i = k - f * R.nxp;
                sm.row[f][i] = rb[k];
            }
            double reg_z = 0.0, reg_x = 0.0;
            for (int j0 = 0; j0 < R.nsp; j0 += MX_CHUNK) {
                const int C = min(MX_CHUNK, R.nsp - j0);
                const float *cb = base + R.col_off;
                for (int k = tid; k < C_NF * C; k += blockDim.x) {
                    const int f = k / C, jl = k - f * C;
                    sm.col[f][jl] = cb[(size_t)f * R.nsp + j0 + jl];
                }
                __syncthreads();
                float sz = 0.f, cz = 0.f, sx = 0.f, cx = 0.f;
                const int total = R.nxp * C;
                for (int p = tid; p < total; p += blockDim.x) {
                    const int i = p / C, jl = p - i * C;
                    const float ws = sm.col[C_WS][jl];
                    if (ws == 0.f) continue;
                    const float w = sm.row[R_WX][i] * ws;
                    const float u = sm.row[R_U][i];
                    const float r0 = sm.col[C_R0][jl];
                    const float Dd = u * (sm.col[C_CG][jl] * u - 2.f * sm.col[C_BG][jl]);
                    const float delta = Dd / (r0 + sqrtf(fmaf(r0, r0, Dd)));
                    const float rr = r0 + delta;
                    int t0, t1, x0, x1, z0, z1;
                    float td, xd, zd;
                    Fields5 F = {0.f, 0.f, 0.f, 0.f, 0.f};
                    if (axis_split(__float_as_int(sm.col[C_TB][jl]), sm.col[C_TF][jl] - delta * inv_dt, nt, t0, t1, td) &&
                        axis_split(__float_as_int(sm.row[R_XB][i]), sm.row[R_XF][i], nx, x0, x1, xd) &&
                        axis_split(__float_as_int(sm.col[C_ZB][jl]), sm.col[C_ZF][jl] + delta * inv_dz, nz, z0, z1, zd)) {
                        int s0 = head + t0, s1 = head + t1;
                        if (s0 >= cap) s0 -= cap;
                        if (s1 >= cap) s1 -= cap;
                        F = gather5(ring, nx, nz, s0, s1, td, x0, x1, xd, z0, z1, zd);
                    }
                    const float scale = 1.f + sm.row[R_XP][i] * sm.col[C_RHO][jl];
                    const float vr = F.vx;
                    // K1x ~ 1 is stored as K1x - 1 so that K0x - vx' (nearly equal
                    // transverse velocities) is formed exactly
                    const float brx = (sm.col[C_K0X][jl] - vr) - vr * (sm.col[C_K1X][jl] + vr * sm.col[C_K2X][jl]);
                    const float brz = sm.col[C_K0Z][jl] - vr * (sm.col[C_K1Z][jl] + vr * sm.col[C_K2Z][jl]);
                    const float p1 = sm.col[C_A][jl] + vr * sm.col[C_B][jl];
                    const float num = scale * F.dx * brx + F.dz * brz - scale * p1 * F.den * F.vxx;
                    const float inv_r = 1.f / rr;
                    const float Iz = num * inv_r;
                    const float Q1 = sm.col[C_Q1][jl];
                    const float q1 = sm.col[C_Q0][jl] - u * Q1;
                    const float M = sm.col[C_M0][jl] - u * Q1 - sm.col[C_Q2][jl] * delta;
                    const float e = sm.col[C_E][jl];
                    const float pd = -(F.dx * (e + vr * sm.col[C_G][jl]) +
                                       F.dz / scale * (sm.col[C_H][jl] + vr * e)) - F.den * F.vxx;
                    const float Ix = scale * inv_r * inv_r * (q1 * inv_r * F.den + pd * M);
                    kahan(sz, cz, w * Iz);
                    kahan(sx, cx, w * Ix);
                }
                const double bz = block_sum((double)sz - (double)cz, sm.red);
                const double bx = block_sum((double)sx - (double)cx, sm.red);
                if (tid == 0) { reg_z += bz; reg_x += bx; }
                __syncthreads();
            }
            if (tid == 0) {
                part[((size_t)b * WAKE_MAX_REGIONS + r) * 2 + 0] = reg_z;
                part[((size_t)b * WAKE_MAX_REGIONS + r) * 2 + 1] = reg_x;
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
    const PointMeta m = meta[b];
    double az = 0.0, ax = 0.0;
    if (m.valid && r < m.nreg) {
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
            for (int j = threadIdx.x; j < R.nsp; j += blockDim.x) {
                const double spj = np_linspace_at(R.sl, R.sr, R.nsp, j);
                if (!(fabs(spj - o.s) < J.near_band)) continue;
                const double dl = (j > 0) ? spj - np_linspace_at(R.sl, R.sr, R.nsp, j - 1) : 0.0;
                const double dr = (j < R.nsp - 1) ? np_linspace_at(R.sl, R.sr, R.nsp, j + 1) - spj : 0.0;
                const double ws = 0.5 * (dl + dr);
                double L[6];
                lattice_lerp(J, spj, L);
                const double rho_sp = rho_at(J, spj);
                for (int i = 0; i < R.nxp; ++i) {
                    const double xpi = np_linspace_at(R.xl, R.xr, R.nxp, i);
                    const double xl = (i > 0) ? xpi - np_linspace_at(R.xl, R.xr, R.nxp, i - 1) : 0.0;
                    const double xr = (i < R.nxp - 1) ? np_linspace_at(R.xl, R.xr, R.nxp, i + 1) - xpi : 0.0;
                    double Iz, Ix;
                    integrand_fp64(J, o, L, rho_sp, spj, xpi, Iz, Ix);
                    const double w = 0.5 * (xl + xr) * ws;
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
    const PointMeta m = meta[b];
    if (!m.valid) {
        dE[pt] = __longlong_as_double(0x7ff8000000000000ll);
        xkick[pt] = __longlong_as_double(0x7ff8000000000000ll);
        return;
    }
    double se = 0.0, sx = 0.0;
    for (int r = 0; r < m.nreg; ++r) {
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
};

static const size_t kMixedScratchTarget = (size_t)96 << 20;   // keep batches L2-sized

static MixedLayout mixed_layout(int xbins_max, int zbins_max, int64_t n) {
    MixedLayout L;
    L.rec_words = point_record_words(xbins_max, zbins_max);
    int64_t per = (int64_t)(L.rec_words * sizeof(float) + sizeof(PointMeta) + 2 * 8 * WAKE_MAX_REGIONS * 8 + 8 + 64);
    int64_t batch = (int64_t)(kMixedScratchTarget / per);
    if (batch < 1) batch = 1;
    if (batch > n) batch = n;
    L.batch = batch;
    return L;
}

static size_t mixed_carve(Carver &c, const MixedLayout &L, unsigned long long **counter, float **rec,
                          PointMeta **meta, double **part, double **band, double **obs_vx) {
    *counter = c.take<unsigned long long>(4);
    *rec = c.take<float>((size_t)L.batch * L.rec_words);
    *meta = c.take<PointMeta>((size_t)L.batch);
    *part = c.take<double>((size_t)L.batch * WAKE_MAX_REGIONS * 2);
    *band = c.take<double>((size_t)L.batch * WAKE_MAX_REGIONS * 2);
    *obs_vx = c.take<double>((size_t)L.batch);
    return c.used;
}

static int integral_blocks() {
    static int cached = 0;
    if (cached) return cached;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mixed_integral, MX_THREADS,
                                                      sizeof(IntegralSmem)) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    cached = per_sm * num_sms();
    return cached;
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
    double *p, *q, *v;
    return mixed_carve(c, L, &a, &b, &m, &p, &q, &v) + 256;
}

extern "C" int dfcsr_wake_mixed(const dfcsr_wake_job *jobs, const int32_t *job_of_point,
                                const double *s, const double *x, int64_t n, int xbins_max,
                                int zbins_max, int use_band, double *dE, double *xkick,
                                void *workspace, size_t workspace_bytes, void *stream) {
    clear_error();
    DFCSR_CHECK_ARG(n >= 0, "dfcsr_wake_mixed: negative point count");
    if (n == 0) return DFCSR_OK;
    DFCSR_CHECK_ARG(jobs && s && x && dE && xkick, "dfcsr_wake_mixed: null pointer");
    DFCSR_CHECK_ARG(xbins_max >= 1 && 2 * xbins_max <= MX_MAX_ROWS,
                    "dfcsr_wake_mixed: xbins must be in [1, %d] (got %d)", MX_MAX_ROWS / 2, xbins_max);
    DFCSR_CHECK_ARG(zbins_max >= 1 && zbins_max <= MX_MAX_COLS,
                    "dfcsr_wake_mixed: zbins must be in [1, %d] (got %d)", MX_MAX_COLS, zbins_max);
    const MixedLayout L = mixed_layout(xbins_max, zbins_max, n);
    Carver c{reinterpret_cast<char *>(workspace), workspace_bytes, 0};
    unsigned long long *counter;
    float *rec;
    PointMeta *meta;
    double *part, *band, *obs_vx;
    mixed_carve(c, L, &counter, &rec, &meta, &part, &band, &obs_vx);
    if (!workspace || !c.ok()) {
        set_error("dfcsr_wake_mixed: workspace too small (%zu < %zu)", workspace_bytes, c.used);
        return DFCSR_OOM;
    }
    cudaStream_t st = as_stream(stream);
    static bool attr_set = false;
    if (!attr_set) {
        DFCSR_CUDA_TRY(cudaFuncSetAttribute(mixed_integral, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)sizeof(IntegralSmem)));
        attr_set = true;
    }
    const int blocks_max = integral_blocks();
    for (int64_t first = 0; first < n; first += L.batch) {
        const int64_t count = (n - first < L.batch) ? n - first : L.batch;
        DFCSR_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st));
        {
            ScopedTiming tm("wake_mixed_geometry", st);
            mixed_geometry<<<dim3((unsigned)count, WAKE_MAX_REGIONS), GEO_THREADS, 0, st>>>(
                jobs, job_of_point, s, x, first, count, L.rec_words, rec, meta, obs_vx);
        }
        const int blocks = (int)((int64_t)blocks_max < count ? blocks_max : count);
        {
            ScopedTiming tm("wake_mixed_integral", st);
            mixed_integral<<<blocks, MX_THREADS, sizeof(IntegralSmem), st>>>(
                jobs, job_of_point, first, count, L.rec_words, rec, meta, part, counter);
        }
        if (use_band) {
            ScopedTiming tm("wake_mixed_band", st);
            mixed_band<<<dim3((unsigned)count, WAKE_MAX_REGIONS), 128, 0, st>>>(
                jobs, job_of_point, s, x, first, count, meta, obs_vx, band);
        }
        mixed_finalize<<<(unsigned)((count + 127) / 128), 128, 0, st>>>(
            jobs, job_of_point, first, count, meta, part, use_band ? band : nullptr, dE, xkick);
    }
    DFCSR_LAUNCH_CHECK();
    return DFCSR_OK;
}
