"""Build the sm_103a shared library ``libdfcsr_gb300.so`` in-tree with nvcc.

    python -m pydfcsr_gb300.build          # incremental
    python -m pydfcsr_gb300.build --force

Each CUDA translation unit is compiled in parallel for
``-gencode arch=compute_103a,code=sm_103a`` and linked into one shared
library with a plain C ABI (``include/dfcsr_gb300.h``).  ``wake_fp64.cu`` is
compiled with ``-fmad=false`` so that the FP64 drop-in kernel rounds every
product and sum separately, like numpy.

``build(checked=True)`` (``--checked``) builds the same sources with
``-DDFCSR_BOUNDS_CHECK=1`` into ``libdfcsr_gb300_checked.so``: every kernel
tests its computed global-memory indices, records the first failure in a
status word read by ``dfcsr_bounds_status`` and skips the access.  Setting
``DFCSR_GB300_CHECKED=1`` makes the Python package load that library.
"""
import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libdfcsr_gb300.so")
LIB_CHECKED = os.path.join(BUILD, "libdfcsr_gb300_checked.so")
CHECKED_FLAGS = ["-DDFCSR_BOUNDS_CHECK=1"]
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I", INCLUDE]
UNITS = {
    "beam_ops.cu": [],
    "capi.cu": [],
    "deposit.cu": [],
    "deposit_noalloc.cu": [],
    "dfstage.cu": [],
    "history.cu": [],
    "interp.cu": [],
    "probe.cu": [],
    "wake_fp64.cu": ["-fmad=false"],
    "wake_mixed.cu": [],
}


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build dfcsr_gb300")
    return path


def _sources_mtime():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "dfcsr_gb300.h"))
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def lib_path(checked=False):
    return LIB_CHECKED if checked else LIB


def up_to_date(checked=False):
    lib = lib_path(checked)
    return os.path.exists(lib) and os.path.getmtime(lib) >= _sources_mtime()


def _compile(unit, extra, objdir):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(objdir, unit.replace(".cu", ".o"))
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force=False, verbose=False, checked=False):
    """Compile (if needed) and return the path of the shared library (the
    bounds-checked variant with ``checked``)."""
    lib = lib_path(checked)
    if not force and up_to_date(checked):
        return lib
    objdir = os.path.join(BUILD, "checked") if checked else BUILD
    os.makedirs(objdir, exist_ok=True)
    flags = CHECKED_FLAGS if checked else []
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1] + flags, objdir), UNITS.items()))
    tmp = lib + f".{os.getpid()}.tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    if verbose:
        print(f"built {lib}")
    return lib


def build_all(force=False, verbose=False):
    """Both libraries, the release one and the bounds-checked one, compiled
    side by side."""
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        futs = [ex.submit(build, force, verbose, c) for c in (False, True)]
        return [f.result() for f in futs]


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--checked", action="store_true", help="the bounds-checked library")
    a = ap.parse_args()
    print(build(force=a.force, verbose=True, checked=a.checked))
    sys.exit(0)
