"""Build libfmmbem.so (CUDA for sm_103a + C++ host code) in-tree with nvcc.

Translation units compile in parallel; the shared library lands in
``fmbem_gpu_c_gb300/_lib/libfmmbem.so``.  Host code is compiled with
``-ffp-contract=off`` so the octree's double arithmetic rounds like the reference's.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libfmmbem.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                  "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + SRC]

SOURCES = ["plan.cu", "tables.cu", "passes.cu", "octree_gpu.cu", "octree_host.cpp", "legacy.cu", "noalloc.cu", "batched.cu", "vjp.cu", "mesh.cpp", "tc_dense.cu", "scene.cu", "tc_rcr3.cu"]


def _sources():
    return [s for s in SOURCES if os.path.exists(os.path.join(SRC, s))]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    cmd = ["nvcc"] + NVFLAGS + ["-c", os.path.join(SRC, src), "-o", obj]
    if src.endswith(".cpp"):
        cmd = ["nvcc", "-x", "cu"] + NVFLAGS + ["-c", os.path.join(SRC, src), "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, res.stdout, res.stderr))
    return obj


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    if not force and not _stale():
        return LIB
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(_compile, srcs))
    cmd = ["nvcc"] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (res.stdout, res.stderr))
    if verbose:
        print("built", LIB, file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
