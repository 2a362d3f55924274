"""Build ``libslakonet_gb300.so`` from ``csrc/*.cu`` with nvcc for sm_103a.

Translation units compile in parallel into ``_build/`` and link into the
package directory (in-tree, git-ignored).  Rebuilds only when a source or
header is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import fcntl
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libslakonet_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
# Extra launch shapes of the eigensolver, exported with a suffix and chosen per problem-size
# bucket by slakonet_gb300.autotune: (suffix, threads per CTA, CTAs per SM, unroll, shared-memory staging n,
# blocked Cholesky and reduction).
EIG_SHAPES = [("_t32", 32, 16, 2, 16, 0), ("_t64", 64, 8, 2, 16, 0), ("_t256", 256, 3, 2, 32, 0),
              ("_blk", 128, 3, 2, 24, 1)]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build slakonet_gb300")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    return any(os.path.getmtime(p) > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every translation unit for sm_103a and link the in-tree shared library (skipped when it
    is newer than every source).  Processes that build at the same time take turns on a lock file, and
    one that waited finds the library built."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with open(os.path.join(BUILD, ".build.lock"), "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        if not force and not _stale():
            return LIB
        return _build_locked(verbose)


def _build_locked(verbose: bool) -> str:
    cc = nvcc()
    inc = ["-I", os.path.join(ROOT, "include")]

    def compile_one(job):
        src, extra, tag = job
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + tag + ".o")
        cmd = [cc, *ARCH, *FLAGS, *inc, *extra, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    jobs = [(src, [], "") for src in sources()]
    eig = os.path.join(CSRC, "eigh.cu")
    for suffix, nt, minb, unr, smem_n, blocked in EIG_SHAPES:
        jobs.append((eig, [f"-DSKN_EIG_SUFFIX={suffix}", f"-DSKN_EIG_NT={nt}", f"-DSKN_EIG_MINB={minb}",
                           f"-DSKN_EIG_UNR={unr}", f"-DSKN_EIG_SMEM_N={smem_n}", f"-DSKN_EIG_BLOCKED={blocked}"],
                     suffix))
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, jobs))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
