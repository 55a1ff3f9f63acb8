"""Build recipe of the CUDA library (libaurora_gb300.so) for sm_103a.

Each .cu file under csrc/ is compiled in parallel with nvcc, then linked into
one shared library with the CUDA runtime linked statically, so the library
loads on hosts without a GPU. Device code uses -fmad=false with IEEE division
and square root; host code uses -ffp-contract=off.
"""
import concurrent.futures
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libaurora_gb300.so")
INCLUDE = os.path.join(HERE, "..", "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
                     "-Xcompiler", "-fPIC,-ffp-contract=off,-O3", "-I" + INCLUDE]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _deps():
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) +
            glob.glob(os.path.join(INCLUDE, "*.h")) + [__file__])


def _compile(src, extra, verbose):
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    newest = max(os.path.getmtime(p) for p in _deps() + [src])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    cmd = [nvcc(), *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)
    return obj


def build(verbose=False, ptxas_info=False):
    """Compiles csrc/*.cu and links libaurora_gb300.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, verbose or ptxas_info), srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", LIB]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    return LIB


HOST = os.path.join(HERE, "host")
DRIVER = os.path.join(BUILD, "aurora_render")


def build_host(verbose=False):
    """Builds the C++ host layer and the standalone driver aurora_render
    against libaurora_gb300.so (g++, no CUDA headers needed)."""
    lib = build(verbose)
    srcs = [os.path.join(HOST, "aurora.cpp"), os.path.join(HOST, "aurora_render.cpp")]
    deps = srcs + [os.path.join(HOST, "aurora.h"), os.path.join(INCLUDE, "aurora_gb300.h"), lib, __file__]
    if os.path.exists(DRIVER) and os.path.getmtime(DRIVER) >= max(os.path.getmtime(p) for p in deps):
        return DRIVER
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + INCLUDE, "-I" + HOST, *srcs, "-L" + BUILD,
           "-laurora_gb300", "-Wl,-rpath,$ORIGIN", "-o", DRIVER]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("host build failed:\n%s%s" % (r.stdout, r.stderr))
    return DRIVER


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
    print(build_host())
