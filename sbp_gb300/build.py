"""Builds libsbpgpu.so (the CUDA C-ABI library) in-tree for sm_103a.

Each translation unit is compiled by nvcc in parallel into sbp_gb300/_build/ and linked
into sbp_gb300/libsbpgpu.so.  Rebuilds only when a source or header is newer than the
library.  No CMake; one -gencode (compute_103a -> sm_103a).
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libsbpgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no floating-point contraction, so host-side entropy tables round the same on
# x86_64 and aarch64 hosts
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + [os.path.join(ROOT, "include", "sbpgpu.h"), __file__]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force=False, verbose=False, extra_flags=()):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    exe = nvcc()

    def compile_one(src):
        obj = os.path.join(OUT, os.path.basename(src).replace(".cu", ".o"))
        cmd = [exe] + ARCH + NVCC_FLAGS + list(extra_flags) + ["-I", os.path.join(ROOT, "include"), "-c", src,
                                                               "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = LIB + ".tmp"
    cmd = [exe] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
