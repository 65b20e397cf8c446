"""Builds liblla_gb300.so in-tree with nvcc for sm_103a (GB300).

Each translation unit is compiled in parallel, then linked into one shared
library with the CUDA runtime linked statically, so the library loads without
libcudart on the library path (the CUDA driver is opened at run time).
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblla_gb300.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
         "--expt-relaxed-constexpr"]
SOURCES = ["lla_potrf.cu", "lla_trsm.cu", "lla_layout.cu", "lla_api.cpp"]


def _sources():
    extra = sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")) and f not in SOURCES)
    return SOURCES + extra


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(HERE, "..", "include", "lla_gb300.h"))
    return hs


def _compile(src):
    obj = os.path.join(BUILD, src + ".o")
    path = os.path.join(CSRC, src)
    if not _stale(obj, [path] + _headers()):
        return obj, None
    cmd = [NVCC] + ARCH + FLAGS + ["-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [NVCC] + FLAGS + ["-x", "cu"] + ARCH + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(_compile, srcs))
    objs = [o for o, _ in results]
    if verbose:
        for (o, log) in results:
            if log:
                print(log, file=sys.stderr)
    if _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
