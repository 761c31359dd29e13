"""A C host drives the library on the GPU through the C ABI alone (no
Python, no torch): it allocates device buffers with the CUDA runtime, runs
dfcsr_beam_moments and dfcsr_deposit_cic2d, and checks the results against
what it computes itself:
* the moments' mean and standard deviation of x and z against two-pass sums
  on the host (1e-12 relative; the means against the mean magnitude);
* the deposit's conservation laws for particles well inside the grid: the
  unit-weight grid sums to the particle count and the weighted grid to the
  sum of the weights, and the grids' first moments (sum of node position x
  weight) reproduce the particles' coordinate sums - cloud-in-cell
  distributes each particle over the nodes of its cell with weights 1 - f,
  f, so these hold exactly up to rounding (1e-12 of the sums of magnitudes,
  since the coordinate sums themselves nearly cancel)."""
import os
import shutil
import subprocess

import pytest
import torch

from pydfcsr_gb300 import build

pytestmark = pytest.mark.gpu
cuda = pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")

HOST_C = r"""
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <cuda_runtime.h>
#include "dfcsr_gb300.h"

#define TRY(x) do { int s_ = (x); if (s_) { printf("FAIL %s: %d %s\n", #x, s_, dfcsr_last_error()); return 1; } } while (0)
#define CU(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { printf("FAIL %s: %s\n", #x, cudaGetErrorString(e_)); return 1; } } while (0)

static double rel(double a, double b) { return fabs(a - b) / (fabs(b) > 0 ? fabs(b) : 1.0); }

int main(void) {
    const int n = 200000, nb1 = 64, nb2 = 48;
    const double s1 = -4.0, e1 = 4.0, s2 = -3.0, e2 = 3.0;
    double *x = malloc(n * sizeof(double)), *z = malloc(n * sizeof(double)), *w = malloc(n * sizeof(double));
    unsigned long long r = 12345;
    for (int i = 0; i < n; ++i) {   /* uniform in [-2, 2) x [-1.5, 1.5): well inside the grid */
        r = r * 6364136223846793005ull + 1442695040888963407ull;
        x[i] = -2.0 + 4.0 * (double)(r >> 11) / 9007199254740992.0;
        r = r * 6364136223846793005ull + 1442695040888963407ull;
        z[i] = -1.5 + 3.0 * (double)(r >> 11) / 9007199254740992.0;
        r = r * 6364136223846793005ull + 1442695040888963407ull;
        w[i] = 0.5 + (double)(r >> 11) / 9007199254740992.0;
    }
    double *dx, *dz, *dw, *g0, *g1, *mom;
    void *ws, *mws;
    CU(cudaMalloc((void **)&dx, n * sizeof(double)));
    CU(cudaMalloc((void **)&dz, n * sizeof(double)));
    CU(cudaMalloc((void **)&dw, n * sizeof(double)));
    CU(cudaMalloc((void **)&g0, (size_t)nb1 * nb2 * sizeof(double)));
    CU(cudaMalloc((void **)&g1, (size_t)nb1 * nb2 * sizeof(double)));
    CU(cudaMalloc((void **)&mom, 16 * sizeof(double)));
    CU(cudaMemcpy(dx, x, n * sizeof(double), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(dz, z, n * sizeof(double), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(dw, w, n * sizeof(double), cudaMemcpyHostToDevice));
    const size_t mb = dfcsr_moments_workspace_bytes(n), wb = dfcsr_deposit_workspace_bytes(n, nb1, nb2);
    CU(cudaMalloc(&mws, mb));
    CU(cudaMalloc(&ws, wb));
    TRY(dfcsr_beam_moments(dx, dz, n, mom, mws, mb, NULL));
    TRY(dfcsr_deposit_cic2d(dx, dz, NULL, dw, n, nb1, s1, e1, nb2, s2, e2, g0, g1, ws, wb, NULL));
    CU(cudaDeviceSynchronize());
    double m[16], *h0 = malloc((size_t)nb1 * nb2 * sizeof(double)), *h1 = malloc((size_t)nb1 * nb2 * sizeof(double));
    CU(cudaMemcpy(m, mom, sizeof(m), cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(h0, g0, (size_t)nb1 * nb2 * sizeof(double), cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(h1, g1, (size_t)nb1 * nb2 * sizeof(double), cudaMemcpyDeviceToHost));
    /* host: two-pass mean and standard deviation, coordinate and weight sums */
    double sx = 0, sz = 0, sw = 0, swx = 0, swz = 0, ax = 0, az = 0, awx = 0, awz = 0;
    for (int i = 0; i < n; ++i) {
        sx += x[i]; sz += z[i]; sw += w[i]; swx += w[i] * x[i]; swz += w[i] * z[i];
        ax += fabs(x[i]); az += fabs(z[i]); awx += fabs(w[i] * x[i]); awz += fabs(w[i] * z[i]);
    }
    const double mx = sx / n, mz = sz / n;
    double vx = 0, vz = 0;
    for (int i = 0; i < n; ++i) { vx += (x[i] - mx) * (x[i] - mx); vz += (z[i] - mz) * (z[i] - mz); }
    int fails = 0;
#define CHECK(c) do { if (!(c)) { printf("FAIL line %d: %s\n", __LINE__, #c); ++fails; } } while (0)
    CHECK(m[0] == (double)n);
    CHECK(fabs(m[1] - mx) <= 1e-12 * ax / n);   /* means near 0: against the mean magnitude */
    CHECK(fabs(m[2] - mz) <= 1e-12 * az / n);
    CHECK(rel(m[3], sqrt(vx / n)) < 1e-12);
    CHECK(rel(m[4], sqrt(vz / n)) < 1e-12);
    /* deposit: node i of axis 1 at s1 + i (e1 - s1) / nb1 */
    const double d1 = (e1 - s1) / nb1, d2 = (e2 - s2) / nb2;
    double t0 = 0, t1 = 0, fx = 0, fz = 0, fwx = 0, fwz = 0;
    for (int i = 0; i < nb1; ++i)
        for (int j = 0; j < nb2; ++j) {
            const double a = h0[i * nb2 + j], b = h1[i * nb2 + j];
            const double xi = s1 + i * d1, zj = s2 + j * d2;
            t0 += a; t1 += b; fx += a * xi; fz += a * zj; fwx += b * xi; fwz += b * zj;
        }
    CHECK(rel(t0, (double)n) < 1e-12);
    CHECK(rel(t1, sw) < 1e-12);
    /* the sums nearly cancel (coordinates centred on 0): compare against the
       sums of magnitudes, which bound the rounding */
    CHECK(fabs(fx - sx) <= 1e-12 * ax);
    CHECK(fabs(fz - sz) <= 1e-12 * az);
    CHECK(fabs(fwx - swx) <= 1e-12 * awx);
    CHECK(fabs(fwz - swz) <= 1e-12 * awz);
    CHECK(dfcsr_kernel_launches() > 0);
    printf("%s %d\n", fails ? "failed" : "ok", fails);
    return fails ? 1 : 0;
}
"""


@cuda
@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_c_host_runs_moments_and_deposit(tmp_path):
    lib = build.build()
    src = tmp_path / "host.c"
    src.write_text(HOST_C)
    exe = tmp_path / "host"
    libdir = os.path.dirname(lib)
    cudalib = os.path.join(CUDA_HOME, "lib64")
    cmd = ["gcc", "-std=c11", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(CUDA_HOME, "include"), str(src), "-o", str(exe),
           "-L", libdir, "-l:" + os.path.basename(lib), "-Wl,-rpath," + libdir,
           "-L", cudalib, "-lcudart", "-Wl,-rpath," + cudalib, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok 0"), r.stdout
