"""Build libgrx.so (the CUDA engine) in-tree for sm_103a.

Each .cu translation unit is compiled by nvcc in parallel, then linked into
graspa_gb300/_build/libgrx.so. No CMake; the only requirement is nvcc on PATH or
under /usr/local/cuda/bin. Usage: python -m graspa_gb300.build [--force]
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgrx.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["grx_box.cu", "grx_pair.cu", "grx_ewald.cu", "grx_widom.cu", "grx_noalloc.cu", "grx_gcmc.cu", "grx_gcmc_cluster.cu", "grx_gcmc_swap.cu", "grx_arena.cu", "grx_server.cu", "grx_probe.cu", "grx_voxel.cu"]
HEADERS = ["grx_internal.cuh", "grx_host.h", "grx_warp.cuh", "grx_df.cuh", "grx_cbmc.cuh", "grx_gcmc_kernel.cuh"]
HOST = os.path.join(HERE, "host")
HOST_SOURCES = ["graspa_host.cpp", "graspa_input.cpp"]
HOST_PROGRAMS = {"gcmc_driver": "gcmc_driver.cpp", "graspa_run": "graspa_run.cpp"}
DRIVER = os.path.join(OUT, "gcmc_driver")
RUNNER = os.path.join(OUT, "graspa_run")


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v",
                   "-Xcudafe", "--diag_suppress=1444", "-Xcompiler", "-Wno-deprecated-declarations",
                   "-I", os.path.join(HERE, "..", "include")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src):
    obj = os.path.join(OUT, os.path.basename(src).replace(".cu", ".o"))
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in HEADERS] + \
        [os.path.join(HERE, "..", "include", "grx.h")]
    if not _stale(obj, deps):
        return obj, ""
    cmd = [nvcc()] + _flags() + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    if force:
        for f in os.listdir(OUT):
            if f.endswith(".o") or f.endswith(".so"):
                os.remove(os.path.join(OUT, f))
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(_compile, SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                print(log)
    if _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    build_host()
    return LIB


def build_host():
    """The C++ host layer (graspa_gb300/host) and its programs, linked against
    libgrx.so with g++ (no CUDA headers needed on this side)."""
    inc = os.path.join(HERE, "..", "include")
    common = [os.path.join(HOST, s) for s in HOST_SOURCES]
    headers = [os.path.join(HOST, h) for h in ("graspa_host.hpp", "graspa_input.hpp")] + \
        [os.path.join(inc, "grx.h"), os.path.join(inc, "grx_philox.h")]
    for exe, src in HOST_PROGRAMS.items():
        target = os.path.join(OUT, exe)
        srcs = common + [os.path.join(HOST, src)]
        if not _stale(target, srcs + headers + [LIB]):
            continue
        cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-I", inc, "-I", HOST] + srcs + \
            ["-L", OUT, "-lgrx", "-Wl,-rpath,$ORIGIN", "-o", target]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"host layer build failed for {exe}:\n{r.stdout}\n{r.stderr}")
    return DRIVER


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
