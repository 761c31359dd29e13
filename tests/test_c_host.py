"""A C host program built against include/dfcsr_gb300.h and the in-tree
library, the way a C or C++ caller of the wake path links it: the header
compiles as strict C11, the struct layouts a C compiler gives agree with
the library's (dfcsr_abi_sizeof), and calls that need no GPU (sizes, status
names, argument errors, the empty wake) behave as documented.  No kernel
launches: this runs without a device."""
import os
import shutil
import subprocess

import pytest

from pydfcsr_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HOST_C = r"""
#include <stdio.h>
#include <string.h>
#include "dfcsr_gb300.h"

static int fails = 0;
#define CHECK(c) do { if (!(c)) { printf("FAIL line %d: %s\n", __LINE__, #c); ++fails; } } while (0)

int main(void) {
    CHECK(dfcsr_version() >= 100);
    CHECK(dfcsr_abi_sizeof(0) == sizeof(dfcsr_df_params));
    CHECK(dfcsr_abi_sizeof(1) == sizeof(dfcsr_wake_job));
    CHECK(strcmp(dfcsr_status_name(DFCSR_OK), "OK") == 0);
    CHECK(strcmp(dfcsr_status_name(DFCSR_BAD_ARG), "BAD_ARG") == 0);
    CHECK(strcmp(dfcsr_status_name(99), "UNKNOWN") == 0);
    CHECK(dfcsr_wake_workspace_bytes(100, 100, 4096) > 0);
    CHECK(dfcsr_deposit_workspace_bytes(1 << 20, 256, 256) <= dfcsr_deposit_noalloc_max_bytes());
    long long launches = dfcsr_kernel_launches();
    /* an empty wake is a no-op; a null job with points is an argument error */
    CHECK(dfcsr_wake_mixed_job(NULL, NULL, NULL, 0, 100, 100, 0, NULL, NULL, NULL, 0, NULL) == DFCSR_OK);
    dfcsr_wake_job job;
    memset(&job, 0, sizeof job);
    int st = dfcsr_wake_mixed_job(NULL, (const double *)16, (const double *)16, 5, 100, 100, 0,
                                  (double *)16, (double *)16, NULL, 0, NULL);
    CHECK(st == DFCSR_BAD_ARG);
    CHECK(strstr(dfcsr_last_error(), "null job") != NULL);
    st = dfcsr_wake_mixed_job(&job, (const double *)16, (const double *)16, 5, 2000, 100, 0,
                              (double *)16, (double *)16, NULL, 0, NULL);
    CHECK(st == DFCSR_BAD_ARG);
    CHECK(strstr(dfcsr_last_error(), "xbins") != NULL);
    st = dfcsr_df_axis_tables(0.0, 1.0, 1, 0.0, 1.0, 8, 0, 0, (double *)16, (double *)16,
                              (double *)16, (double *)16, NULL);
    CHECK(st == DFCSR_BAD_ARG);
    CHECK(dfcsr_kernel_launches() == launches);
    printf("%s %d\n", fails ? "failed" : "ok", fails);
    return fails ? 1 : 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_c_host_links_and_calls(tmp_path):
    lib = build.build()
    src = tmp_path / "host.c"
    src.write_text(HOST_C)
    exe = tmp_path / "host"
    libdir = os.path.dirname(lib)
    cmd = ["gcc", "-std=c11", "-Wall", "-Wextra", "-pedantic", "-Werror",
           "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
           "-L", libdir, "-l:" + os.path.basename(lib), "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok 0"), r.stdout
