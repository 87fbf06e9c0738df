"""Builds the CUDA library (csrc/) for sm_103a with nvcc, in-tree.

Each translation unit is compiled in parallel, then linked into
``csrc/_build/libollin_gpu.so``.  Host code is compiled without FMA
contraction so that host arithmetic (initial data, time bookkeeping) is the
same on x86 and Arm hosts.
"""
import concurrent.futures
import os
import subprocess

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(CSRC, "_build")
LIB = os.environ.get("OLLIN_GPU_LIB") or os.path.join(BUILD, "libollin_gpu.so")
SOURCES = ["rhs.cu", "rhs_stale.cu", "rhs_sync.cu", "rhs_stale_sync.cu", "rhs_o2.cu", "rhs_o2_stale.cu",
           "rhs_o2_sync.cu", "rhs_o2_stale_sync.cu", "aux.cu", "transfer.cu", "elliptic.cu", "multigrid.cu", "noalloc.cu", "host.cpp", "serve.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2"]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _compile(src):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + ARCH + COMMON + ["-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc()] + COMMON + ["-x", "cu"] + ARCH + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".cpp", ".h"))]
    deps.append(os.path.join(os.path.dirname(PKG), "include", "ollin_gpu.h"))
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


def build(force=False):
    """Compile and link; return the path of the shared library."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    os.replace(tmp, LIB)
    return LIB
