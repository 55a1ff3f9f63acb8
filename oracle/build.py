"""Build recipe for the oracle (test infrastructure only).

build_oracle() compiles aur_oracle.cpp, the CPU restatement of the reference
algorithms, into oracle/_build/liboracle.so. build_ref() compiles the
reference's own traversal headers, read in place from the reference source
tree, through the shim in ref_shim/ into oracle/_ref/libaurora_ref.so; it is
skipped when that tree is absent. The tree is found at $AURORA_REFERENCE,
else at DEFAULT_REFERENCE, the directory where the build container mounts
the reference checkout (read only); on a machine without it (the GPU host)
build_ref() does nothing and the tests that need it skip. Both use -ffp-contract=off so that no
multiply-add is fused, like the -fmad=false CUDA build they are compared with.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libaurora_ref.so")
DEFAULT_REFERENCE = "/root/reference"
FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-pthread"]


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force=False):
    src = os.path.join(HERE, "aur_oracle.cpp")
    hdr = os.path.join(HERE, "..", "include", "aurora_gb300.h")
    if force or _stale(ORACLE_SO, [src, hdr, __file__]):
        os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
        subprocess.check_call(["g++", *FLAGS, src, "-o", ORACLE_SO])
    return ORACLE_SO


def build_ref(reference=None, force=False):
    ref = reference or os.environ.get("AURORA_REFERENCE", DEFAULT_REFERENCE)
    if not os.path.isdir(os.path.join(ref, "src")):
        return None
    srcs = [os.path.join(HERE, "ref_shim", "ref_traverse.cpp"), os.path.join(HERE, "ref_shim", "ref_shade.cpp")]
    if force or _stale(REF_SO, srcs + [__file__]):
        os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
        # -fpermissive: util/bsdf.h declares a member with an extra class qualification, which MSVC accepts
        subprocess.check_call(["g++", *FLAGS, "-w", "-fpermissive", "-I" + os.path.join(HERE, "ref_shim"),
                               "-I" + os.path.join(ref, "src"), "-I" + os.path.join(HERE, "..", "include"),
                               *srcs, "-o", REF_SO])
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
