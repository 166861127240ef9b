"""Build libacumen_gpu.so in-tree with nvcc for sm_103a (no GPU needed).

Each translation unit is compiled in parallel, then linked into
acumen_gb300/libacumen_gpu.so with the static CUDA runtime.  Host code is
compiled without floating-point contraction so that the geometry tables are
evaluated in the reference's single-precision operation order.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libacumen_gpu.so")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["api.cu", "prep_api.cu", "kernels_radon.cu", "kernels_lines.cu", "kernels_fft.cu", "kernels_tv.cu", "kernels_prep.cu",
           "kernels_grad.cu", "batch.cu", "noalloc.cu", "tables.cpp"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str, obj: str, verbose_ptxas: bool) -> str:
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose_ptxas and src.endswith(".cu"):
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "acumen_gpu.h"), __file__]
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= max(os.path.getmtime(d) for d in deps):
        return OUT
    os.makedirs(BUILD, exist_ok=True)
    objs = [os.path.join(BUILD, s + ".o") for s in srcs]
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        logs = list(ex.map(lambda a: _compile(*a, verbose_ptxas), zip(srcs, objs)))
    if verbose_ptxas:
        for s, l in zip(srcs, logs):
            sys.stderr.write(f"== {s}\n{l}")
    tmp = OUT + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


DRIVERS = ["fits_to_hpc", "raw_to_hpc", "projections_to_sinogram_hpc", "fbp_hpc", "tv_hpc", "tv_hpc_slice", "to_tiff"]
BIN = os.path.join(HERE, "bin")


def build_drivers(force: bool = False) -> list:
    """The C++ drop-ins for the reference's driver programs, linked against
    libacumen_gpu.so (found next to the package through the rpath)."""
    lib = build(force)
    os.makedirs(BIN, exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    out = []
    def one(name):
        src = os.path.join(HERE, "drivers", name + ".cpp")
        exe = os.path.join(BIN, name)
        deps = [src, os.path.join(HERE, "drivers", "hpc_io.h"), os.path.join(HERE, "drivers", "fits.h"), lib]
        if force or not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(d) for d in deps):
            cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-pthread", src, "-o", exe, "-L" + HERE, "-lacumen_gpu",
                   "-Wl,-rpath,$ORIGIN/.."]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"driver build failed for {name}:\n{r.stderr}")
        return exe
    with cf.ThreadPoolExecutor(max_workers=len(DRIVERS)) as ex:
        out = list(ex.map(one, DRIVERS))
    return out


PROBE = os.path.join(BIN, "l1_peak")


def build_probe(force: bool = False) -> str:
    """The L1 load-bandwidth probe (csrc/l1_peak.cu), a standalone program that
    bench.py runs for the measured ceiling of the gather kernels."""
    src = os.path.join(CSRC, "l1_peak.cu")
    os.makedirs(BIN, exist_ok=True)
    if force or not os.path.exists(PROBE) or os.path.getmtime(PROBE) < os.path.getmtime(src):
        r = subprocess.run([nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", src, "-o", PROBE],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"probe build failed:\n{r.stderr}")
    return PROBE


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    build_drivers(force="--force" in sys.argv)
    build_probe(force="--force" in sys.argv)
    print(OUT)
