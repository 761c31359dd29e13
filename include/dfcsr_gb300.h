/*
 * dfcsr_gb300.h - C ABI of the GB300 (sm_103a) CSR wake path.
 *
 * The wake path of pyDFCSR_2D (deposit -> smoothing/derivatives -> history
 * -> retarded-geometry CSR integral) as plain `extern "C"` entry points over
 * device pointers and sizes.  No torch, numpy or CUDA types appear here:
 * every `stream` is a `cudaStream_t` passed as `void *`, every array is a
 * device pointer unless the comment says host.
 *
 * The reference has no FFI layer: its boundary is the Python method surface
 * of DF_tracker / CSR2D and the numba functions.  Each entry point below
 * names the reference function it replaces (file:line within pyDFCSR_2D/).
 *
 * Every call returns a dfcsr_status; on failure dfcsr_last_error() gives a
 * message for the calling host thread.  Calls are asynchronous on `stream`
 * unless stated otherwise; a call never synchronises the device.
 */
#ifndef DFCSR_GB300_H
#define DFCSR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    DFCSR_OK = 0,
    DFCSR_BAD_ARG = 1,          /* invalid size, null pointer, bad parameter */
    DFCSR_OOM = 2,              /* workspace too small / allocation refused   */
    DFCSR_TIMEOUT = 3,          /* a bounded device wait gave up              */
    DFCSR_KERNEL_ERROR = 4,     /* a kernel reported an error status word     */
    DFCSR_CUDA_ERROR = 5,       /* CUDA runtime error (launch, copy)          */
    DFCSR_ADMISSION_REFUSED = 6 /* request does not fit the HBM budget        */
} dfcsr_status;

/* Library version (major*10000 + minor*100 + patch). */
int dfcsr_version(void);
/* Message of the last failing call on this host thread ("" if none). */
const char *dfcsr_last_error(void);
/* Short name of a status code. */
const char *dfcsr_status_name(int status);
/* Number of kernel launches this library has issued in this process (all
 * entry points, all devices; launches recorded into a CUDA graph count once,
 * at capture).  Host-side counter, no device synchronisation. */
long long dfcsr_kernel_launches(void);
/* sizeof of the ABI structs: 0 dfcsr_df_params, 1 dfcsr_wake_job (for
 * bindings that lay the structs out themselves); 0 for other values. */
size_t dfcsr_abi_sizeof(int which);

/* Bounds-checked build (no reference counterpart; stands in for
 * compute-sanitizer).  libdfcsr_gb300_checked.so is this library built with
 * -DDFCSR_BOUNDS_CHECK=1: every kernel tests its computed global-memory
 * indices (history cells, per-point records, sort positions, particle
 * indices, table cells) against their buffers; the first failing test
 * records bit 63 | site << 48 | (index & 0xffffffffffff) in a device
 * status word and the access is skipped (nothing traps).  Sites: 1 probe,
 * 10-13 mixed integral / set-up, 20 mixed geometry, 30 FP64 history
 * gathers, 31 orbit tables, 40-43
 * deposit, 50 history regrid, 60 apply_wakes, 70 DF stage, 80 interp3d /
 * interp1d.  dfcsr_bounds_checked: 1 in the checked library, 0 otherwise.
 * dfcsr_bounds_status: synchronises the current device and gives the first
 * failure recorded on it (0: none; the status words are per device),
 * clearing them when `reset`; in the release library
 * it gives 0 without touching the device.  dfcsr_bounds_probe: one thread
 * tests `index` against [0, size) at `site` (1..32767) through the same
 * check, without accessing memory (a test of the mechanism itself). */
int dfcsr_bounds_checked(void);
int dfcsr_bounds_status(unsigned long long *first_failure, int reset);
int dfcsr_bounds_probe(long long index, long long size, int site, void *stream);

/* Optional kernel timing (off by default).  When enabled, the entry points
 * record CUDA events around their main kernels on the launch stream;
 * dfcsr_timing_collect() waits for the recorded events and adds their
 * durations to per-kernel totals, read with dfcsr_timing_get(name, ...).
 * Names: beam_moments, deposit_cic2d, df_finalize, history_regrid,
 * wake_fp64, wake_mixed_geometry, wake_mixed_integral, wake_mixed_band,
 * transport6, apply_wakes. */
void dfcsr_timing_enable(int on);
int dfcsr_timing_collect(void);
int dfcsr_timing_get(const char *name, double *total_ms, long long *launches);
void dfcsr_timing_reset(void);

/* ------------------------------------------------------------------------
 * Beam moments.  Replaces the numpy statistics used by DF_tracker.get_DF
 * (deposit.py:147-159: std/mean of x and z, slice std of x where
 * |z| < 0.1 sigma_z) and by Beam (beams.py:137-215: mean/std, polyfit
 * slope of x on z, std/mean of the chirp-removed x_transform).
 *
 * out[16] (device, double): 0 n, 1 mean_x, 2 mean_z, 3 sigma_x, 4 sigma_z,
 * 5 slope (dx/dz), 6 intercept, 7 n_slice, 8 sigma_x_slice, 9 mean_xt,
 * 10 sigma_xt, 11 cov_xz, 12..15 reserved.  Deterministic (fixed reduction
 * order).  Needs dfcsr_moments_workspace_bytes(n) bytes of device scratch.
 */
size_t dfcsr_moments_workspace_bytes(int64_t n);
int dfcsr_beam_moments(const double *x, const double *z, int64_t n, double *out,
                       void *workspace, size_t workspace_bytes, void *stream);

/* ------------------------------------------------------------------------
 * Cloud-in-cell deposit.  Replaces histogram_cic_2d (deposit.py:43-87),
 * called twice per step by get_DF (deposit.py:172-182) with w = 1 and
 * w = px.  Both weight channels are deposited from one sort:
 *   out0 = CIC(q1, q2, w0 or 1 if w0 == NULL)   [nb1][nb2] row-major
 *   out1 = CIC(q1, q2, w1)                       (skipped if out1 == NULL;
 *                                                 w1 required when n > 0)
 * Bin spacing (end - start) / nbins, lower bin floor(cell), weights
 * 1 - frac, bounds-checked corners - exactly the reference's rule.
 * Deterministic: particles are sorted by lower cell (stable LSD radix sort);
 * fixed-size chunks of the sorted particles are summed per cell and the
 * parts of cells that cross chunks are added in a fixed order (four
 * interleaved partial sums over the chunks).  No float atomics; the order
 * of additions depends only on the input order.
 * Needs dfcsr_deposit_workspace_bytes(n, nb1, nb2) bytes of scratch.
 */
size_t dfcsr_deposit_workspace_bytes(int64_t n, int nb1, int nb2);
int dfcsr_deposit_cic2d(const double *q1, const double *q2, const double *w0,
                        const double *w1, int64_t n,
                        int nb1, double start1, double end1,
                        int nb2, double start2, double end2,
                        double *out0, double *out1,
                        void *workspace, size_t workspace_bytes, void *stream);

/* The same deposit on the grid of get_DF (deposit.py:147-159) taken from the
 * beam moments in DEVICE memory (`moments`: the 16 values of
 * dfcsr_beam_moments; [1], [2] the means of q1 and q2, [3], [4] their
 * standard deviations): start = mean - lim sigma, end = mean + lim sigma per
 * axis, computed by a kernel on `stream` in the host's operation order, so
 * the result equals dfcsr_deposit_cic2d with the grid computed on the host
 * from the same moments.  Lets a caller enqueue the deposit right behind the
 * moments, before it has their host copy (a kick-feedback step loop waits
 * for that copy).  A zero standard deviation (empty bin range) cannot be
 * reported from the device: every particle then falls outside the grid; the
 * caller checks its host copy of the moments.  Same workspace as
 * dfcsr_deposit_cic2d. */
int dfcsr_deposit_cic2d_moments(const double *q1, const double *q2, const double *w0,
                                const double *w1, int64_t n, int nb1, int nb2,
                                const double *moments, double lim1, double lim2,
                                double *out0, double *out1,
                                void *workspace, size_t workspace_bytes, void *stream);

/* Deposit that allocates nothing.  No counterpart in the reference.  For
 * callers that cannot allocate device memory when they deposit (a host code
 * that plans its device buffers up front and forbids allocation inside its
 * step loop, a plugin host whose memory belongs to its own pool): the
 * scratch is one fixed device array inside the library (24 MiB, reserved on
 * every GPU that loads this entry point, held until exit).  Same arguments
 * and results as dfcsr_deposit_cic2d without the workspace.  Limits: at most
 * 1,048,576 particles and (nb1 + 1) * (nb2 + 1) <= 257 * 257 (a 256 x 256
 * grid); larger requests return DFCSR_BAD_ARG.  A call resolves the array's
 * device address (cudaGetSymbolAddress) on the current device, again on every
 * call made outside a stream capture (an address from before a
 * cudaDeviceReset would be stale); a call on a capturing stream uses the
 * address of the device's last call outside a capture, so the first call on
 * a device must come before any stream capture (else DFCSR_BAD_ARG).  All
 * calls share the array: calls that overlap on the GPU race and must be
 * serialised by the caller. */
size_t dfcsr_deposit_noalloc_max_bytes(void);
int dfcsr_deposit_cic2d_noalloc(const double *q1, const double *q2, const double *w0,
                                const double *w1, int64_t n,
                                int nb1, double start1, double end1,
                                int nb2, double start2, double end2,
                                double *out0, double *out1, void *stream);

/* ------------------------------------------------------------------------
 * Distribution-function finalisation: everything get_DF does after the two
 * deposits (deposit.py:183-235), in place on device arrays [nx][nz]:
 * threshold and vx = vxsum / density, Savitzky-Golay smoothing along x then
 * z (scipy savgol_filter, mode 'interp'), trapz normalisation, numpy.gradient
 * derivatives, smoothing of the derivatives, vx_x fill.
 *
 * Host-side parameter block (all pointers in `p` are DEVICE pointers):
 */
typedef struct {
    int nx, nz;                 /* grid size                                  */
    int window, order;          /* SG window (odd) and polynomial order       */
    double velocity_threshold;  /* DF_tracker.velocity_threhold               */
    const double *sg_coeff;     /* [window] interior coefficients             */
    const double *sg_lo;        /* [window/2][window] left edge map           */
    const double *sg_hi;        /* [window/2][window] right edge map          */
    const double *gx;           /* [4][nx]: a,b,c (interior), edge 1/dx info  */
    const double *gz;           /* [4][nz]                                    */
    const double *dxg;          /* [nx-1] diff(x_grids)                       */
    const double *dzg;          /* [nz-1] diff(z_grids)                       */
    int gx_uniform, gz_uniform; /* numpy.gradient uniform-spacing path taken  */
    double gx_dx, gz_dx;        /* the uniform spacing when taken             */
    unsigned int barrier_spins; /* polls before a grid-barrier wait gives up  */
                                /* (0: 2^24, about a second; at most 2^24)    */
    int barrier_extra;          /* 0; 1 expects one arrival more than the     */
                                /* launch has CTAs, so that every wait runs   */
                                /* out (exercises the timeout path)           */
} dfcsr_df_params;

/* density, vx: in = raw deposits, out = final fields.  density_x,
 * density_z, vx_x: outputs.  scalars_out[8] (device): 0 dsum, 1 thr,
 * 2 thr2, 3 vx_x fill, 4 mean(vx_x), 5 max raw density, 6 max density,
 * 7 status: 0.0, or 1.0 if a grid-barrier wait of the launch gave up - the
 * fields are then invalid and scalars 0..6 are NaN.  The call returns before
 * the launch ends, so the caller reads scalars_out[7] once the stream has
 * passed it (DF_tracker raises DfcsrTimeout from it).  nz <= 16384.
 * One cooperative launch (one CTA per SM, all resident) on `stream`.
 * Scratch: dfcsr_df_workspace_bytes(nx, nz). */
size_t dfcsr_df_workspace_bytes(int nx, int nz);

/* The per-step grid tables of dfcsr_df_params from get_DF's two grids,
 * x_grids = linspace(x0, x1, nx), z_grids = linspace(z0, z1, nz)
 * (deposit.py:170-171), on the device: gx [4][nx], gz [4][nz] (the
 * numpy.gradient coefficients, deposit.py:212-213, edge_order 1) and dxg
 * [nx-1], dzg [nz-1] (diff of each grid), equal to the host's numpy values
 * bit for bit.  x_uniform / z_uniform: whether numpy takes its
 * uniform-spacing branch (all differences equal; the caller decides it
 * from its host grid).  2 <= nx, nz <= 2^24.  One launch on `stream`,
 * device pointers out. */
int dfcsr_df_axis_tables(double x0, double x1, int nx, double z0, double z1, int nz,
                         int x_uniform, int z_uniform, double *gx, double *gz,
                         double *dxg, double *dzg, void *stream);
int dfcsr_df_finalize(const dfcsr_df_params *p, double *density, double *vx,
                      double *density_x, double *density_z, double *vx_x,
                      double *scalars_out, void *workspace, size_t workspace_bytes,
                      void *stream);

/* Health check of the bounded grid barrier that dfcsr_df_finalize's
 * cooperative launch uses between its phases (no reference counterpart:
 * the reference's get_DF runs on one CPU thread).  One cooperative launch
 * of `blocks` CTAs (1..SM count) meets at the barrier once, expecting
 * blocks + extra_arrivals arrivals (extra_arrivals 0 or 1).  With 1 the
 * last arrival never comes: each CTA's wait gives up after max_spins polls
 * (1..2^24; df_finalize uses 2^24, about a second) and the call returns
 * DFCSR_TIMEOUT with the CUDA context intact.  Synchronises `stream`;
 * workspace >= 16 bytes of device memory. */
int dfcsr_grid_barrier_check(int blocks, int extra_arrivals, unsigned int max_spins,
                             void *workspace, size_t workspace_bytes, void *stream);

/* ------------------------------------------------------------------------
 * History regrid.  Replaces DF_interp (deposit.py:296-309: scipy
 * RegularGridInterpolator, linear, bounds_error False) for the five fields
 * appended by append_interpolant (deposit.py:321-337, 379-390).
 *
 * The source fields are five device arrays [snx][snz]; the target is one
 * slot of the device history ring.  The per-axis interval indices and
 * normalised distances (tensor-product grids) are device tables computed
 * beforehand (dfcsr_rgi_axis_linspace, or by the host): ix[nxi], wx[nxi],
 * oobx[nxi] (1 = outside), iz[nzi], wz[nzi], oobz[nzi].
 * vx_x_fill is a DEVICE pointer to the fill value of vx_x (its mean).
 * ring64: [slot][nxi][nzi][5] doubles (or NULL); ring32: [slot][nxi][nzi][8]
 * floats (or NULL): fields 0..4, then in slot 5 the low part of density_x
 * (density_x - (double)(float)density_x), in slot 6 the low part of vx,
 * slot 7 zero.  Field order:
 * density, density_x, density_z, vx, vx_x.  With ring64 the values follow
 * RegularGridInterpolator's term order exactly; with ring32 only, the
 * bilinear weights are applied as fused multiply-adds (the FP32 cells are
 * unchanged to within their rounding). */

/* The axis tables of dfcsr_history_regrid when the source grid and the
 * target grid are numpy linspaces (get_DF's x_grids / z_grids and
 * append_interpolant's x_grid_interp / z_grid_interp, deposit.py:170-171,
 * 347-350): idx[ntgt], w[ntgt], oob[ntgt] computed on the device with the
 * RegularGridInterpolator rule above, equal to the host computation from the
 * numpy arrays.  2 <= nsrc <= 2^24, 1 <= ntgt <= 2^24. */
int dfcsr_rgi_axis_linspace(double src_start, double src_stop, int nsrc,
                            double tgt_start, double tgt_stop, int ntgt, int32_t *idx,
                            double *w, uint8_t *oob, void *stream);

int dfcsr_history_regrid(const double *density, const double *density_x,
                         const double *density_z, const double *vx,
                         const double *vx_x, int snx, int snz,
                         const int32_t *ix, const double *wx, const uint8_t *oobx, int nxi,
                         const int32_t *iz, const double *wz, const uint8_t *oobz, int nzi,
                         const double *vx_x_fill,
                         double *ring64_slot, float *ring32_slot, void *stream);

/* ------------------------------------------------------------------------
 * Standalone interpolants (API parity with the numba functions).
 * interpolate3D (interp3D.py:18-66) on a C-order [nt][nx][nz] double grid;
 * interpolate1D (interp1D.py:13-36).  int() truncation semantics: a query
 * with -1 < u < 0 extrapolates from the first cell; u <= -1 or u >= n -> 0.
 */
int dfcsr_interp3d(const double *qt, const double *qx, const double *qz, int64_t m,
                   const double *data, int nt, int nx, int nz,
                   double min_t, double min_x, double min_z,
                   double delta_t, double delta_x, double delta_z,
                   double *out, void *stream);
int dfcsr_interp1d(const double *q, int64_t m, const double *table, int n,
                   double min_x, double delta_x, double *out, void *stream);

/* ------------------------------------------------------------------------
 * CSR wake.  Replaces calculate_2D_CSR / get_CSR_wake / get_CSR_integrand
 * (CSR.py:397-418, 454-602, 605-782) for a batch of observation points.
 *
 * A job describes one beam's history, lattice and parameters; observation
 * point k uses job job_of_point[k] (NULL: all use job 0).  The job array
 * lives in DEVICE memory.
 */
typedef struct {
    const double *ring64;       /* [cap][nx][nz][5] or NULL                   */
    const float *ring32;        /* [cap][nx][nz][8] or NULL (see regrid);     */
                                /* 32-byte aligned (else the mixed wake       */
                                /* returns NaN for the job's points)          */
    int cap, head, nt, nx, nz;  /* ring capacity, oldest slot, slices, grid   */
    int pad0;
    double t_min, x_min, z_min; /* build_interpolant (deposit.py:416-421)     */
    double t_delta, x_delta, z_delta;
    const double *lattice;      /* [nsample][6]: X0, Y0, nX, nY, tauX, tauY   */
    int nsample, nelement;
    double s_min, s_delta;      /* Lattice.build_interpolant (lattice.py:141) */
    const double *rho;          /* [nelement] curvature angle/L               */
    const double *distance;     /* [nelement] cumulative element ends         */
    double position;            /* beam.position = t                          */
    double sigma_z, sigma_x;    /* beam._sigma_z, beam._sigma_x               */
    double slope0, mean_x;      /* beam._slope[0], beam._mean_x               */
    double formation_length, n_formation_length;
    double csr_scaling;         /* 8.98755e3 * charge (CSR.py:80)             */
    int zbins, xbins;           /* Integration_params                         */
    double near_band;           /* mixed only: |s' - s| below which the       */
                                /* integrand runs in FP64 (0 = none)          */
    const double *lattice_delta;/* mixed only, optional: [nsample][6] row     */
                                /* differences lattice[k+1] - lattice[k]      */
                                /* (last row 0), or NULL                      */
    const float *lattice_dw;    /* mixed only, optional: [nsample][6][2] the  */
                                /* table as double-word FP32 pairs (hi, lo =  */
                                /* value - hi), with lattice_delta_dw: the    */
                                /* geometry then runs in double-word FP32;    */
    const float *lattice_delta_dw; /* NULL: FP64                               */
} dfcsr_wake_job;

/* Plain FP64 drop-in: reproduces the reference's IEEE operation order
 * (trapz over x' summed row by row, then numpy pairwise over s').  Needs
 * ring64.  zbins_max: the largest integration zbins (s' columns per
 * region) of the jobs in the call, 1..6144 (up to 1024 the column sums sit
 * in static shared memory; above, in dynamic shared memory sized to
 * zbins_max).  A job whose zbins exceeds zbins_max gets NaN.  Outputs
 * dE[n], xkick[n] (MeV/m). */
int dfcsr_wake_fp64(const dfcsr_wake_job *jobs, const int32_t *job_of_point,
                    const double *s, const double *x, int64_t n, int zbins_max,
                    double *dE, double *xkick, void *stream);

/* Observation points of get_CSR_mesh + calculate_2D_CSR (CSR.py:361-418):
 * zrange = linspace(z0, z1, zbins), xrange = linspace(x0, x1, xbins) (numpy's
 * formula), point k = i * zbins + j: s[k] = position + zrange[j],
 * x[k] = xrange[i] + (slope0 * zrange[j] + slope1).  s, x: [xbins * zbins]. */
int dfcsr_csr_mesh(double x0, double x1, int xbins, double z0, double z1, int zbins,
                   double slope0, double slope1, double position, double *s, double *x,
                   void *stream);

/* get_CSR_integrand (CSR.py:605-782) at m arbitrary points (sp[k], xp[k])
 * for one observation point (s, x) of *job (device pointer), plain FP64.
 * ignore_vx != 0 zeroes vx, vx_ret and vx_x_ret like the reference flag.
 * Outputs Iz[m] (longitudinal) and Ix[m] (transverse) integrands. */
int dfcsr_wake_integrand(const dfcsr_wake_job *job, double s, double x,
                         const double *sp, const double *xp, int64_t m, int ignore_vx,
                         double *Iz, double *Ix, void *stream);

/* Mixed precision: the per-(point, s') retarded geometry (FP64, or
 * double-word FP32 from the job's double-word orbit tables) written as
 * per-column records; per integrand point the distance, the retarded shift
 * and the history coordinates in double-word FP32; FP32 gathers from ring32
 * with density_x and vx (stored hi + lo) interpolated in double-word; the
 * density_x and density terms of the longitudinal integrand summed in
 * double-word, the rest Kahan-compensated FP32; fixed-order block sums,
 * region sums in FP64.  Max, rms and pointwise error vs the FP64 kernel on
 * the same history <= 2e-5 of the peak on the benchmark workloads.  Needs
 * ring32 in every job, below 64 GiB (cap * nx * nz * 2 <= 2^32 - 1: cells
 * are addressed with 32-bit float4 offsets; a larger ring makes the job's
 * points NaN, and dfcsr_wake_mixed_job refuses it with DFCSR_BAD_ARG).
 * xbins_max / zbins_max
 * bound the integration bins of all jobs in the call.  use_band != 0 runs
 * the s' columns with |s' - s| < job.near_band through the FP64 integrand.
 * Scratch: dfcsr_wake_workspace_bytes(xbins_max, zbins_max, n); points are
 * processed in batches of up to 1 GiB of per-point records (~74 KB per
 * point at 100 x 100 bins: a 64^2 mesh is one batch). */
size_t dfcsr_wake_workspace_bytes(int xbins_max, int zbins_max, int64_t n);
int dfcsr_wake_mixed(const dfcsr_wake_job *jobs, const int32_t *job_of_point,
                     const double *s, const double *x, int64_t n,
                     int xbins_max, int zbins_max, int use_band,
                     double *dE, double *xkick,
                     void *workspace, size_t workspace_bytes, void *stream);

/* The same wake for one job in HOST memory (a caller's dfcsr_wake_job
 * struct, read during the call and passed to the device as a kernel
 * parameter): no device copy of the job to stage, no copy on the stream.
 * Same results, workspace and limits as dfcsr_wake_mixed with that job for
 * every point.  No reference counterpart as a separate call: it is
 * calculate_2D_CSR (CSR.py:397-418) for one beam. */
int dfcsr_wake_mixed_job(const dfcsr_wake_job *job, const double *s, const double *x,
                         int64_t n, int xbins_max, int zbins_max, int use_band,
                         double *dE, double *xkick, void *workspace,
                         size_t workspace_bytes, void *stream);

/* ------------------------------------------------------------------------
 * Particle steps on either side of the wake.  `coords` is the beam's
 * [6, ld] row-major FP64 array (rows x, px, y, py, z, pz; particle i is
 * column i), updated in place. */

/* Linear transport coords <- R coords by a 6x6 matrix (R: HOST pointer, 36
 * doubles, row-major; copied into the launch, so it may be reused at once).
 * No counterpart on the reference's run path: there Beam.track
 * (beams.py:101-106) calls bmadx's track_element (third party); the linear
 * matrices come from r_gen6 (r_gen6.py:4-122).  Each output row is a fused
 * multiply-add chain over the non-zero coefficients in increasing column. */
int dfcsr_transport6(const double *R, double *coords, int64_t n, int64_t ld, void *stream);

/* Beam.apply_wakes (beams.py:108-131): tables step * wake * 1e6 / energy,
 * RegularGridInterpolator (linear, fill 0) at (x_transform, z) with
 * x_transform = x - (slope0 * z + slope1), pz += dE term, and px += x-kick
 * term when transverse_on.  dE_dct / x_kick: [nx, nz] row-major; xrange
 * [nx], zrange [nz] strictly ascending (as the interpolator requires).
 * Scratch (16-byte aligned): dfcsr_apply_wakes_workspace_bytes - the scaled
 * tables and, per axis interval, its width and reciprocal (the weights are
 * then the reference's divisions, correctly rounded, without a division per
 * particle). */
size_t dfcsr_apply_wakes_workspace_bytes(int nx, int nz);
int dfcsr_apply_wakes(double *coords, int64_t n, int64_t ld, const double *dE_dct,
                      const double *x_kick, const double *xrange, const double *zrange,
                      int nx, int nz, double slope0, double slope1, double step_size,
                      double init_energy, int transverse_on, void *workspace,
                      size_t workspace_bytes, void *stream);

/* ------------------------------------------------------------------------
 * Arithmetic-rate probe (measurement only; no counterpart in the
 * reference).  Launches a kernel of independent fused multiply-add chains in
 * FP64 (fp64 != 0) or FP32 with `iters` iterations per thread and stores its
 * floating-point operation count in *flops (host); time it with events on
 * `stream` to get the FMA throughput.  `sink`: 8 bytes of device memory
 * (never written in practice). */
int dfcsr_probe_fma(int fp64, int64_t iters, void *sink, double *flops, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* DFCSR_GB300_H */
