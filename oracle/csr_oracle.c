/*
 * CPU oracle for the pyDFCSR_2D wake path - TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, the reference's numba loops and its CSR
 * integral so that the CUDA path can be checked against it.  It is the
 * checker, never the product: only tests, the smoke check and the CPU
 * baseline leg of the benchmark may load it.
 *
 * Every routine reproduces the reference's IEEE double arithmetic in the same
 * operation order (compile WITHOUT -ffast-math and with -ffp-contract=off so
 * that a*b+c is never fused):
 *   oracle_cic2d        pyDFCSR_2D/deposit.py:43-87       (histogram_cic_2d)
 *   oracle_interp3d     pyDFCSR_2D/interp3D.py:18-66      (interpolate3D)
 *   oracle_interp1d     pyDFCSR_2D/interp1D.py:13-36      (interpolate1D)
 *   oracle_wake_point   pyDFCSR_2D/CSR.py:454-602         (get_CSR_wake)
 *   integrand()         pyDFCSR_2D/CSR.py:605-782         (get_CSR_integrand)
 * numpy semantics restated: linspace (y_i = i*step + start, last = stop),
 * trapz (d*(y[i+1]+y[i])/2.0; axis-0 sums run sequentially over rows, 1-D
 * sums use numpy's pairwise summation with 8 partial accumulators).
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- CIC ---- */
void oracle_cic2d(const double *q1, const double *q2, const double *w, long n,
                  int nb1, double start1, double end1,
                  int nb2, double start2, double end2, double *hist)
{
    double sp1 = (end1 - start1) / nb1, inv1 = 1. / sp1;
    double sp2 = (end2 - start2) / nb2, inv2 = 1. / sp2;
    memset(hist, 0, sizeof(double) * (size_t)nb1 * nb2);
    for (long i = 0; i < n; ++i) {
        double c1 = (q1[i] - start1) * inv1;
        double c2 = (q2[i] - start2) * inv2;
        double f1 = floor(c1), f2 = floor(c2);
        if (!(f1 > -2.0 && f1 < (double)nb1) || !(f2 > -2.0 && f2 < (double)nb2))
            continue;               /* no corner can land inside the grid */
        long i1 = (long)f1, i2 = (long)f2;
        double s1 = 1. - (c1 - i1);
        double s2 = 1. - (c2 - i2);
        if (i1 >= 0 && i1 < nb1) {
            if (i2 >= 0 && i2 < nb2) hist[i1 * nb2 + i2] += w[i] * s1 * s2;
            if (i2 + 1 >= 0 && i2 + 1 < nb2) hist[i1 * nb2 + i2 + 1] += w[i] * s1 * (1. - s2);
        }
        if (i1 + 1 >= 0 && i1 + 1 < nb1) {
            if (i2 >= 0 && i2 < nb2) hist[(i1 + 1) * nb2 + i2] += w[i] * (1. - s1) * s2;
            if (i2 + 1 >= 0 && i2 + 1 < nb2) hist[(i1 + 1) * nb2 + i2 + 1] += w[i] * (1. - s1) * (1. - s2);
        }
    }
}

/* ------------------------------------------------------- interpolation ---- */
/* int(u) truncates toward zero: for -1 < u < 0 the lower index is 0 and the
 * weight u is negative (linear extrapolation).  In range iff -1 < u < n. */
static inline int axis_index(double u, int n, int *i0, int *i1, double *frac)
{
    if (!(u > -1.0 && u < (double)n)) return 0;
    int a = (int)u;                 /* C cast truncates like Python int() */
    *i0 = a;
    *i1 = (a == n - 1) ? a : a + 1;
    *frac = u - (double)a;
    return 1;
}

static inline double interp3(const double *d, int nt, int nx, int nz,
                             double ut, double ux, double uz)
{
    int t0, t1, x0, x1, z0, z1;
    double td, xd, zd;
    if (!axis_index(ut, nt, &t0, &t1, &td) || !axis_index(ux, nx, &x0, &x1, &xd) ||
        !axis_index(uz, nz, &z0, &z1, &zd))
        return 0.0;
    size_t sx = (size_t)nz, st = (size_t)nx * nz;
#define D(a, b, c) d[(size_t)(a) * st + (size_t)(b) * sx + (size_t)(c)]
    double c00 = D(t0, x0, z0) * (1 - td) + D(t1, x0, z0) * td;
    double c01 = D(t0, x0, z1) * (1 - td) + D(t1, x0, z1) * td;
    double c10 = D(t0, x1, z0) * (1 - td) + D(t1, x1, z0) * td;
    double c11 = D(t0, x1, z1) * (1 - td) + D(t1, x1, z1) * td;
#undef D
    double c0 = c00 * (1 - xd) + c10 * xd;
    double c1 = c01 * (1 - xd) + c11 * xd;
    return c0 * (1 - zd) + c1 * zd;
}

void oracle_interp3d(const double *qt, const double *qx, const double *qz, long m,
                     const double *data, int nt, int nx, int nz,
                     double min_t, double min_x, double min_z,
                     double dt, double dx, double dz, double *out)
{
    for (long i = 0; i < m; ++i)
        out[i] = interp3(data, nt, nx, nz, (qt[i] - min_t) / dt, (qx[i] - min_x) / dx,
                         (qz[i] - min_z) / dz);
}

static inline double interp1(const double *v, int n, double u)
{
    int a, b;
    double f;
    if (!axis_index(u, n, &a, &b, &f)) return 0.0;
    return v[a] * (1 - f) + v[b] * f;
}

void oracle_interp1d(const double *q, long m, const double *tab, int n,
                     double min_x, double delta_x, double *out)
{
    for (long i = 0; i < m; ++i) out[i] = interp1(tab, n, (q[i] - min_x) / delta_x);
}

/* -------------------------------------------------------- numpy helpers ---- */
static void np_linspace(double start, double stop, int num, double *y)
{
    if (num <= 0) return;
    if (num == 1) { y[0] = start; return; }
    int div = num - 1;
    double delta = stop - start;
    double step = delta / div;
    if (step == 0.0) {
        for (int i = 0; i < num; ++i) y[i] = ((double)i / div) * delta + start;
    } else {
        for (int i = 0; i < num; ++i) y[i] = (double)i * step + start;
    }
    y[num - 1] = stop;
}

/* numpy pairwise summation (PW_BLOCKSIZE 128, 8 partial sums) */
static double np_pairwise(const double *a, long n)
{
    if (n < 8) {
        double r = 0.0;
        if (n > 0) r = a[0];
        for (long i = 1; i < n; ++i) r += a[i];
        /* numpy starts from -0.0 for empty; n==0 never happens here */
        return r;
    }
    if (n <= 128) {
        double r[8];
        for (int k = 0; k < 8; ++k) r[k] = a[k];
        long i;
        for (i = 8; i < n - (n % 8); i += 8)
            for (int k = 0; k < 8; ++k) r[k] += a[i + k];
        double res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
        for (; i < n; ++i) res += a[i];
        return res;
    }
    long n2 = n / 2;
    n2 -= n2 % 8;
    return np_pairwise(a, n2) + np_pairwise(a + n2, n - n2);
}

/* ---------------------------------------------------------- wake context -- */
typedef struct {
    /* history interpolant: five fields, each [nt][nx][nz] C-order */
    const double *density, *density_x, *density_z, *vx, *vx_x;
    int nt, nx, nz;
    double t_min, x_min, z_min, t_delta, x_delta, z_delta;
    /* reference-orbit tables, each [nsample] */
    const double *X0, *Y0, *nX, *nY, *tX, *tY;
    int nsample;
    double s_min, s_delta;
    /* per-element curvature and cumulative end positions */
    const double *rho, *distance;
    int nelement;
    /* beam and integration parameters */
    double position, sigma_z, sigma_x, slope0, mean_x;
    double formation_length, n_formation_length, csr_scaling;
    int zbins, xbins;
} oracle_wake_ctx;

static inline double lat_interp(const oracle_wake_ctx *c, const double *tab, double s)
{
    return interp1(tab, c->nsample, (s - c->s_min) / c->s_delta);
}

static inline double hist_interp(const oracle_wake_ctx *c, const double *d,
                                 double t, double x, double z)
{
    return interp3(d, c->nt, c->nx, c->nz, (t - c->t_min) / c->t_delta,
                   (x - c->x_min) / c->x_delta, (z - c->z_min) / c->z_delta);
}

/* get_CSR_integrand for the mesh xp[i] (rows) x sp[j] (columns).  Writes
 * Iz[i*nsp + j], Ix[i*nsp + j]. */
static void integrand(const oracle_wake_ctx *c, double s, double x,
                      const double *xp, int nxp, const double *sp, int nsp,
                      double *Iz, double *Ix)
{
    const double t = c->position;
    const double vx = hist_interp(c, c->vx, t, x, s - t);
    const double X0_s = lat_interp(c, c->X0, s), Y0_s = lat_interp(c, c->Y0, s);
    const double nsx = lat_interp(c, c->nX, s), nsy = lat_interp(c, c->nY, s);
    const double tsx = lat_interp(c, c->tX, s), tsy = lat_interp(c, c->tY, s);
    for (int j = 0; j < nsp; ++j) {
        const double spj = sp[j];
        const double X0_sp = lat_interp(c, c->X0, spj), Y0_sp = lat_interp(c, c->Y0, spj);
        const double npx = lat_interp(c, c->nX, spj), npy = lat_interp(c, c->nY, spj);
        const double tpx = lat_interp(c, c->tX, spj), tpy = lat_interp(c, c->tY, spj);
        double rho_sp = 0.0;
        for (int e = 0; e < c->nelement; ++e) {
            if (e == 0) {
                if (spj < c->distance[0]) rho_sp = c->rho[0];
            } else if (spj < c->distance[e] && spj >= c->distance[e - 1]) {
                rho_sp = c->rho[e];
            }
        }
        for (int i = 0; i < nxp; ++i) {
            const double xpi = xp[i];
            const double rx = X0_s - X0_sp + x * nsx - xpi * npx;
            const double ry = Y0_s - Y0_sp + x * nsy - xpi * npy;
            const double r = sqrt(rx * rx + ry * ry);
            const double t_ret = t - r;
            const double zq = spj - t_ret;
            const double den = hist_interp(c, c->density, t_ret, xpi, zq);
            const double den_x = hist_interp(c, c->density_x, t_ret, xpi, zq);
            const double den_z = hist_interp(c, c->density_z, t_ret, xpi, zq);
            const double vx_r = hist_interp(c, c->vx, t_ret, xpi, zq);
            const double vx_x_r = hist_interp(c, c->vx_x, t_ret, xpi, zq);
            const double scale = 1 + xpi * rho_sp;
            const double vel_x = tsx + vx * nsx;
            const double vel_y = tsy + vx * nsy;
            const double velr_x = tpx + vx_r * npx;
            const double velr_y = tpy + vx_r * npy;
            const double nab_x = den_x * npx + den_z / scale * tpx;
            const double nab_y = den_x * npy + den_z / scale * tpy;
            const double div_v = vx_x_r;
            const double p1 = vel_x * velr_x + vel_y * velr_y;
            const double num1 = scale * ((vel_x - p1 * velr_x) * nab_x + (vel_y - p1 * velr_y) * nab_y);
            const double num2 = -scale * p1 * den * div_v;
            Iz[i * nsp + j] = num1 / r + num2 / r;
            const double nmx = nsx - npx, nmy = nsy - npy;
            const double q1 = rx * nmx + ry * nmy;
            const double q2 = nsx * tpx + nsy * tpy;
            const double pd = -(velr_x * nab_x + velr_y * nab_y) - den * div_v;
            const double W1 = scale * q1 / (r * r * r) * den;
            const double W2 = scale * q1 / (r * r) * pd;
            const double W3 = -scale * q2 / r * pd;
            Ix[i * nsp + j] = W1 + W2 + W3;
        }
    }
}

/* trapz(trapz(I, xp, axis=0), sp) in numpy's order */
static double trapz2(const double *I, const double *xp, int nxp, const double *sp, int nsp,
                     double *colbuf, double *termbuf)
{
    for (int j = 0; j < nsp; ++j) colbuf[j] = 0.0;
    for (int i = 0; i < nxp - 1; ++i) {
        const double d = xp[i + 1] - xp[i];
        for (int j = 0; j < nsp; ++j) {
            const double term = d * (I[(i + 1) * nsp + j] + I[i * nsp + j]) / 2.0;
            colbuf[j] = (i == 0) ? term : colbuf[j] + term;
        }
    }
    for (int j = 0; j < nsp - 1; ++j)
        termbuf[j] = (sp[j + 1] - sp[j]) * (colbuf[j + 1] + colbuf[j]) / 2.0;
    return np_pairwise(termbuf, nsp - 1);
}

typedef struct {
    int nxp, nsp;
    double xl, xr, sl, sr;
} region_t;

/* Region bounds of get_CSR_wake; returns the number of regions (3 or 4). */
static int wake_regions(const oracle_wake_ctx *c, double s, double x, region_t *reg)
{
    const double t = c->position;
    const double sz = c->sigma_z, sx = c->sigma_x, tt = c->slope0;
    const double x0 = (s - t) * c->slope0;
    const double xmean = c->mean_x;
    const int zb = c->zbins, xb = c->xbins;
    if (fabs(tt) <= 1) {
        const double s2 = s - 500 * sz, s3 = s - 20 * sz, s4 = s + 5 * sz;
        const double x1w = x0 - 20 * sx, x2w = x0 + 20 * sx;
        const double x1n = x0 - 10 * sx, x2n = x0 + 10 * sx;
        double s1 = s2 - c->n_formation_length * c->formation_length;
        s1 = (0 >= s1 || s1 != s1) ? ((s1 != s1) ? s1 : 0.0) : s1;
        reg[0] = (region_t){2 * xb, zb, x1w, x2w, s1, s2};
        reg[1] = (region_t){xb, zb, x1n, x2n, s2, s3};
        reg[2] = (region_t){xb, zb, x1n, x2n, s3, s4};
        return 3;
    }
    double s2, s3, s4, x1l, x1r, x2l, x2r, x3l, x3r, x4l, x4r;
    if (tt > 0) {
        const double ta = -2 * tt / (1 - tt * tt);
        const double d = (10 * sx + xmean - x) / ta;
        s4 = s + 3 * sz;
        s3 = s - d;
        s3 = (s3 != s3) ? s3 : (0 >= s3 ? 0.0 : s3);
        s2 = s3 - 200 * sz;
        x1l = x + 0.1 * sx; x1r = x + 10 * sx;
        x2l = x - 3 * sx;   x2r = x1l;
    } else {
        const double ta = 2 * tt / (1 - tt * tt);
        const double d = -(xmean - x - 10 * sx) / ta;
        s4 = s + 3 * sz;
        s3 = s - d;
        s3 = (s3 != s3) ? s3 : (0 >= s3 ? 0.0 : s3);
        s2 = s3 - 200 * sz;
        x1l = x - 10 * sx; x1r = x - 1 * sx;
        x2l = x1r;         x2r = x + 3 * sx;
    }
    x3l = x0 - 5 * sx;  x3r = x0 + 5 * sx;
    x4l = x0 - 20 * sx; x4r = x0 + 20 * sx;
    double s1 = s2 - c->n_formation_length * c->formation_length;
    s1 = (s1 != s1) ? s1 : (0 >= s1 ? 0.0 : s1);
    reg[0] = (region_t){2 * xb, zb, x4l, x4r, s1, s2};
    reg[1] = (region_t){xb, zb, x3l, x3r, s2, s3};
    reg[2] = (region_t){xb, zb, x1l, x1r, s3, s4};
    reg[3] = (region_t){xb, zb, x2l, x2r, s3, s4};
    return 4;
}

/* get_CSR_wake(s, x): returns dE/dct and x-kick.  When dbg is non-NULL the
 * per-region xp, sp, Iz, Ix arrays are copied there region after region
 * (xp[nxp], sp[nsp], Iz[nxp*nsp], Ix[nxp*nsp]) and the return value of the
 * function is the number of doubles written. */
long oracle_wake_point(const oracle_wake_ctx *c, double s, double x,
                       double *dE, double *xkick, double *dbg)
{
    region_t reg[4];
    const int nreg = wake_regions(c, s, x, reg);
    int maxx = 2 * c->xbins, maxs = c->zbins;
    double *xp = malloc(sizeof(double) * maxx);
    double *sp = malloc(sizeof(double) * maxs);
    double *Iz = malloc(sizeof(double) * (size_t)maxx * maxs);
    double *Ix = malloc(sizeof(double) * (size_t)maxx * maxs);
    double *col = malloc(sizeof(double) * maxs);
    double *term = malloc(sizeof(double) * maxs);
    double sum_e = 0.0, sum_x = 0.0;
    long written = 0;
    for (int r = 0; r < nreg; ++r) {
        np_linspace(reg[r].xl, reg[r].xr, reg[r].nxp, xp);
        np_linspace(reg[r].sl, reg[r].sr, reg[r].nsp, sp);
        integrand(c, s, x, xp, reg[r].nxp, sp, reg[r].nsp, Iz, Ix);
        const double e = -c->csr_scaling * trapz2(Iz, xp, reg[r].nxp, sp, reg[r].nsp, col, term);
        const double k = c->csr_scaling * trapz2(Ix, xp, reg[r].nxp, sp, reg[r].nsp, col, term);
        sum_e = (r == 0) ? e : sum_e + e;
        sum_x = (r == 0) ? k : sum_x + k;
        if (dbg) {
            size_t m = (size_t)reg[r].nxp * reg[r].nsp;
            memcpy(dbg + written, xp, sizeof(double) * reg[r].nxp); written += reg[r].nxp;
            memcpy(dbg + written, sp, sizeof(double) * reg[r].nsp); written += reg[r].nsp;
            memcpy(dbg + written, Iz, sizeof(double) * m); written += (long)m;
            memcpy(dbg + written, Ix, sizeof(double) * m); written += (long)m;
        }
    }
    *dE = sum_e;
    *xkick = sum_x;
    free(xp); free(sp); free(Iz); free(Ix); free(col); free(term);
    return written;
}

/* ------------------------------------------------ threaded point batches -- */
typedef struct {
    const oracle_wake_ctx *c;
    const double *s, *x;
    double *dE, *xk;
    long begin, end;
} job_t;

static void *worker(void *arg)
{
    job_t *j = (job_t *)arg;
    for (long i = j->begin; i < j->end; ++i)
        oracle_wake_point(j->c, j->s[i], j->x[i], &j->dE[i], &j->xk[i], NULL);
    return NULL;
}

/* Block partition of points over threads, like the reference's divmod split
 * of the observation mesh over MPI ranks (pyDFCSR_2D/CSR.py:121-125). */
void oracle_wake_points(const oracle_wake_ctx *c, long n, const double *s, const double *x,
                        double *dE, double *xk, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    job_t jobs[256];
    long ave = n / nthreads, res = n % nthreads, start = 0;
    for (int p = 0; p < nthreads; ++p) {
        long cnt = ave + (p < res ? 1 : 0);
        jobs[p] = (job_t){c, s, x, dE, xk, start, start + cnt};
        start += cnt;
        pthread_create(&th[p], NULL, worker, &jobs[p]);
    }
    for (int p = 0; p < nthreads; ++p) pthread_join(th[p], NULL);
}

long oracle_ctx_size(void) { return (long)sizeof(oracle_wake_ctx); }
