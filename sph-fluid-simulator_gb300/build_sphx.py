"""Builds libsphx.so (the sm_103a SPH step and its C-ABI) in-tree.

CUDA translation units go through nvcc with one ``-gencode`` for sm_103a;
host C++ goes through g++ with ``-ffp-contract=off`` (host code that must be
bit-identical to the reference — settings constants, lattices — may not fuse
multiply-adds on either x86-64 or aarch64).  Objects are compiled in parallel
and relinked only when a source or header changed.
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib", "libsphx.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-ffp-contract=off", "--expt-relaxed-constexpr"] + ARCH
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra=()):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not _stale(obj, [src] + _headers()):
        return obj, False
    inc = ["-I", INCLUDE, "-I", CSRC]
    if src.endswith(".cu"):
        cmd = [NVCC, *NVCC_FLAGS, *extra, *inc, "-c", src, "-o", obj]
    else:
        cmd = ["g++", *CXX_FLAGS, *inc, "-I", os.path.join(CUDA_HOME, "include"), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    if extra and r.stderr:
        sys.stderr.write(r.stderr)
    return obj, True


def build(verbose=False, ptxas_info=False):
    """Compiles every translation unit under csrc/ and links lib/libsphx.so
    (``ptxas_info``: print each kernel's registers, spills and shared memory)."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    if ptxas_info:  # recompile the CUDA units so that ptxas reports
        for s in srcs:
            obj = os.path.join(BUILD, os.path.basename(s) + ".o")
            if s.endswith(".cu") and os.path.exists(obj):
                os.remove(obj)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), srcs))
    objs = [o for o, _ in results]
    if any(changed for _, changed in results) or _stale(LIB, objs):
        cmd = [NVCC, "-shared", *ARCH, "-o", LIB, *objs, "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas-info" in sys.argv)
