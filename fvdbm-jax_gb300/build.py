"""Build libfvdbm.so in-tree with nvcc for sm_103a (GB300).

The step kernels must not contract multiply-adds (``--fmad=false``) and the
host code must not either (``-ffp-contract=off``): the float32 results are
specified operation by operation and are compared bit for bit with the CPU
oracle.  Translation units compile in parallel; the library is rebuilt only
when a source or a flag changes.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
BUILD = os.path.join(ROOT, "_build", "fvdbm")
LIB = os.path.join(LIBDIR, "libfvdbm.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-I" + os.path.join(ROOT, "include")]
SOURCES = ["kernels.cu", "tile.cu", "monitor.cu", "capi.cu", "plan.cpp", "batch.cpp", "mpnn.cu", "d2q13.cu",
           "pcg.cu", "features.cu"]
HEADERS = [os.path.join(CSRC, "fvdbm_internal.h"), os.path.join(CSRC, "fvdbm_math.cuh"),
           os.path.join(ROOT, "include", "fvdbm.h"), os.path.join(ROOT, "include", "fvdbm_mpnn.h")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfvdbm")


def _stamp(extra: list[str]) -> str:
    h = hashlib.sha256()
    for f in [os.path.join(CSRC, s) for s in SOURCES] + HEADERS:
        with open(f, "rb") as fh:
            h.update(fh.read())
    h.update(" ".join(ARCH + NVFLAGS + extra).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile (if needed) and return the path of libfvdbm.so."""
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    stamp = _stamp(extra)
    stamp_file = os.path.join(BUILD, "stamp")
    if not force and os.path.exists(LIB) and os.path.exists(stamp_file):
        with open(stamp_file) as fh:
            if fh.read() == stamp:
                return LIB
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, src + ".o")
        cmd = [cc, *ARCH, *NVFLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    if verbose or ptxas_info:
        for _, log in results:
            if log.strip():
                print(log)
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp] + [o for o, _ in results] + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp_file, "w") as fh:
        fh.write(stamp)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
