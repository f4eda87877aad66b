"""Builds libhyperball_gb300.so in-tree for sm_103a.

Translation units compile in parallel: the CUDA kernels with nvcc
(-gencode arch=compute_103a,code=sm_103a), the host engine and graph layer with
g++ (-ffp-contract=off so host f64 arithmetic is never fused). The link uses
nvcc with the static CUDA runtime, so the library loads on machines without a
GPU (every device call then returns HB_ERR_NO_DEVICE).
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "libhyperball_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HEADERS = [
    os.path.join(CSRC, "hb_internal.h"),
    os.path.join(CSRC, "hll_device.cuh"),
    os.path.join(CSRC, "graph_gen.h"),
    os.path.join(REPO, "include", "hyperball_gb300.h"),
]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.isdir(c):
            return c
    nvcc = shutil.which("nvcc")
    return os.path.dirname(os.path.dirname(nvcc)) if nvcc else "/usr/local/cuda"


def _units():
    cuda = _cuda_home()
    inc = ["-I" + os.path.join(REPO, "include"), "-I" + CSRC]
    units = []
    for name in ("hb_kernels.cu", "visits.cu", "sum_sweep.cu"):
        src = os.path.join(CSRC, name)
        obj = os.path.join(OBJ, name + ".o")
        cmd = [os.path.join(cuda, "bin", "nvcc"), *ARCH, "-O3", "-lineinfo", "-std=c++17",
               "-Xcompiler", "-fPIC", *inc, "-c", src, "-o", obj]
        units.append((src, obj, cmd))
    for name in ("hb_engine.cpp", "graph_host.cpp", "graph_gen.cpp", "hb_server.cpp"):
        src = os.path.join(CSRC, name)
        obj = os.path.join(OBJ, name + ".o")
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off", "-Wall",
               "-Wno-unused-function", *inc, "-I" + os.path.join(cuda, "include"),
               "-c", src, "-o", obj]
        units.append((src, obj, cmd))
    return units


def _stale(src, obj):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or any(os.path.getmtime(h) > t for h in HEADERS)


def build(force=False, verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    units = _units()
    procs = []
    for src, obj, cmd in units:
        if force or _stale(src, obj):
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            procs.append((src, subprocess.Popen(cmd)))
    failed = [src for src, p in procs if p.wait() != 0]
    if failed:
        raise RuntimeError("compilation failed: " + ", ".join(failed))
    objs = [obj for _, obj, _ in units]
    if force or procs or not os.path.exists(LIB) or any(
            os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cuda = _cuda_home()
        cmd = [os.path.join(cuda, "bin", "nvcc"), *ARCH, "-shared", "-o", LIB, *objs,
               "-cudart", "static", "-Xcompiler", "-pthread", "-ldl", "-lrt"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        if subprocess.call(cmd) != 0:
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
