"""Builds libmm.so, the CUDA library behind include/mm.h, for sm_103a.

nvcc compiles each translation unit in parallel; the result is project-marshmallow_gb300/build/
libmm.so.  A content hash of the sources and flags decides whether a rebuild is needed, so a copy
of the tree with fresh timestamps does not rebuild needlessly and a changed source always does.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD = os.path.join(PKG_DIR, "build")
LIB = os.path.join(BUILD, "libmm.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                      "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", os.path.join(REPO, "include")]
# Units whose results must equal the CPU oracle bit for bit: no FMA contraction.
EXACT_UNITS = {"march_exact.cu", "march_exact_sw.cu", "noise.cu", "reproject.cu", "shadow_exact.cu", "post_exact.cu"}
# Production-arithmetic units (gated against the FP64 oracle, not bit-exact): FP32 denormals are
# flushed to zero, which drops the denormal handling around the SFU operations (rsqrt, rcp, ex2,
# lg2) from the march's dependent chains.
FAST_UNITS = {"march_fast.cu", "surrogate.cu", "batch.cu", "reproject_fast.cu", "shadow.cu", "post.cu"}
CUDA_UNITS = ["api.cu", "march_fast.cu", "march_exact.cu", "march_exact_sw.cu", "noise.cu", "peaks.cu", "noalloc.cu", "mlp.cu", "surrogate.cu", "batch.cu", "reproject.cu", "reproject_fast.cu", "shadow.cu", "shadow_exact.cu", "post.cu", "post_exact.cu"]
CXX_UNITS = ["scene.cpp", "assets.cpp"]
HEADERS = ["mm_internal.h", "mm_math.h", "march_kernel.cuh", "tc.cuh", "shadow_kernel.cuh", "post_kernel.cuh"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _extra_flags():
    """Extra nvcc flags from the environment (MM_NVCC_FLAGS), e.g. -DMM_MARCH_MIN_BLOCKS=3."""
    return os.environ.get("MM_NVCC_FLAGS", "").split()


def _cmd_for(unit, obj):
    src = os.path.join(CSRC, unit)
    if unit.endswith(".cu"):
        flags = list(NVCC_COMMON) + _extra_flags()
        if unit in EXACT_UNITS:
            flags += ["-fmad=false"]
        if unit in FAST_UNITS:
            flags += ["-ftz=true"]
        return [nvcc()] + flags + ["-c", src, "-o", obj]
    return ["g++", "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall",
            "-I", os.path.join(REPO, "include"), "-c", src, "-o", obj]


def _digest():
    h = hashlib.sha256()
    for name in sorted(CUDA_UNITS + CXX_UNITS + HEADERS):
        with open(os.path.join(CSRC, name), "rb") as f:
            h.update(name.encode() + b"\0" + f.read())
    with open(os.path.join(REPO, "include", "mm.h"), "rb") as f:
        h.update(f.read())
    h.update(" ".join(NVCC_COMMON + sorted(EXACT_UNITS) + sorted(FAST_UNITS) + _extra_flags()).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force=False, verbose=False):
    """Compiles libmm.so if the sources changed; returns its path."""
    os.makedirs(os.path.join(BUILD, "obj"), exist_ok=True)
    stamp = os.path.join(BUILD, "libmm.sha256")
    digest = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return LIB
    units = CUDA_UNITS + CXX_UNITS
    objs = [os.path.join(BUILD, "obj", u.rsplit(".", 1)[0] + ".o") for u in units]

    def run(args):
        r = subprocess.run(args, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: %s\n%s%s" % (" ".join(args), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        list(ex.map(run, [_cmd_for(u, o) for u, o in zip(units, objs)]))
    tmp = LIB + ".tmp"
    run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lpthread", "-ldl", "-lrt"])
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
