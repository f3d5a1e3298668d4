"""Builds libhgb.so (the sm_103a kernels + C ABI) in-tree with nvcc.

Output: hala_gb300/_lib/libhgb.so.  Translation units compile in parallel; one -gencode
(sm_103a), -lineinfo for profiling.  Nothing here needs a GPU: nvcc cross-compiles.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libhgb.so")
SOURCES = ["hgb_core.cu", "hgb_spmv.cu", "hgb_ilu.cu", "hgb_solvers.cu", "hgb_batch.cu", "hgb_bsolve.cu", "hgb_static.cu", "hgb_mrhs.cu", "hgb_pattern.cu", "hgb_complex.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libhgb")


def _compile(src, obj, extra):
    # host code without contracted multiply-adds: the host-side scalar work gives the same bits on
    # x86 and Arm hosts
    cmd = [nvcc_path(), "-std=c++17", "-O3", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-I" + os.path.join(ROOT, "include"), "-c", os.path.join(CSRC, src), "-o", obj, *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "hgb.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra=()):
    """Compile every CUDA source for sm_103a and link libhgb.so.  Returns the library path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    objs = [os.path.join(OUT_DIR, s.replace(".cu", ".o")) for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        logs = list(ex.map(lambda so: _compile(so[0], so[1], list(extra)), zip(SOURCES, objs)))
    if verbose:
        for log in logs:
            sys.stderr.write(log)
    tmp = LIB + ".tmp"
    cmd = [nvcc_path(), "-shared", *ARCH, "-o", tmp, *objs, "-cudart", "shared",
           "-Xlinker", "-rpath", "-Xlinker", "/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
