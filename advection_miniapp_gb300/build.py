"""Build recipe of libadvection_gb300.so (in-tree, no cmake).

Compiles the host C++ and the sm_103a CUDA sources in parallel with nvcc and
links one shared library next to this file.  Objects go to _build/ (ignored by
git).  Rebuilds only what is older than its sources.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD_DIR = os.path.join(os.path.dirname(HERE), "_build", "advection_gb300")
LIB_PATH = os.path.join(HERE, "libadvection_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["tables.cpp", "geometry.cpp", "fdm.cpp", "api.cu", "implicit_api.cu", "stage_fp64.cu", "stage_fp32.cu",
           "diag_kernels.cu", "implicit_kernels.cu", "batch_kernels.cu", "server.cu", "stage_gauss64.cu", "stage_gauss32.cu", "output.cu"]
HEADERS = ["tables.h", "geometry.h", "fdm.h", "handle.h", "implicit_kernels.h", "batch_kernels.h", "kernels.h", "device_common.cuh", "stage_kernel.cuh", "stage_gauss.cuh"]


def nvcc():
    exe = shutil.which("nvcc")
    if exe is None:
        cand = "/usr/local/cuda/bin/nvcc"
        if os.path.exists(cand):
            return cand
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libadvection_gb300.so")
    return exe


def _flags(src):
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp", "-I", os.path.join(os.path.dirname(HERE), "include")]
    if src.endswith(".cu"):
        return common + ARCH + ["-lineinfo", "--expt-relaxed-constexpr"]
    return common


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths if os.path.exists(p))


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD_DIR, src + ".o")
    deps = [path] + [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(os.path.dirname(HERE), "include", "advection_gb300.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= _newest(deps):
        return obj, ""
    cmd = [nvcc(), "-c", path, "-o", obj] + _flags(src)
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "c++", "-c", path, "-o", obj] + _flags(src)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compilation of {src} failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj, res.stderr


def build(verbose=False, force=False):
    """Compile every source (in parallel) and link libadvection_gb300.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force:
        for f in os.listdir(BUILD_DIR):
            os.remove(os.path.join(BUILD_DIR, f))
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(_compile, SOURCES))
    objs = [r[0] for r in results]
    if verbose:
        for src, (_, log) in zip(SOURCES, results):
            if log.strip():
                print(f"[{src}]\n{log}", file=sys.stderr)
    if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < _newest(objs):
        cmd = [nvcc(), "-shared", "-o", LIB_PATH] + objs + ARCH + ["-Xcompiler", "-fopenmp", "-lgomp"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return LIB_PATH


DRIVER_SRC = os.path.join(HERE, "cpp", "advection_solver.cpp")
DRIVER_BIN = os.path.join(BUILD_DIR, "advection_solver")


def build_driver():
    """Compile the C++ driver program (cpp/advection_solver.cpp) against the library."""
    lib = build()
    deps = [DRIVER_SRC, lib, os.path.join(os.path.dirname(HERE), "include", "advection_gb300.hpp")]
    if os.path.exists(DRIVER_BIN) and os.path.getmtime(DRIVER_BIN) >= _newest(deps):
        return DRIVER_BIN
    cmd = [nvcc(), "-O2", "-std=c++17", "-I", os.path.join(os.path.dirname(HERE), "include"), DRIVER_SRC,
           "-o", DRIVER_BIN, "-L", HERE, "-ladvection_gb300", "-Xlinker", "-rpath," + HERE]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return DRIVER_BIN


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
