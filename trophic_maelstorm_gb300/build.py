"""Build libtm.so (the sm_103a kernels + C ABI) in-tree.

    python -m trophic_maelstorm_gb300.build

Translation units compile in parallel, each with one -gencode for sm_103a.
-fmad=false keeps every multiply and add separately rounded unless the source
asks for an fma(), which is what makes the kernels' arithmetic reproducible
bit for bit (the tests compare them with a CPU restatement).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "lib")
OBJ_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "libtm.so")
SWEEP = os.path.join(OUT_DIR, "tm_sweep")
SOURCES = ["tm_step.cu", "tm_rk4.cu", "tm_measure.cu", "tm_capi.cu", "tm_noalloc.cu", "tm_spectrum.cu", "tm_fke.cu",
           "tm_mlp.cu"]
HEADERS = ["tm_device.cuh", "tm_kernels.cuh", "tm_zig_table.cuh", os.path.join("..", "..", "include", "tm.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
           "-diag-suppress", "1444"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose):
    obj = os.path.join(OBJ_DIR, os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in HEADERS]
    if not _stale(obj, deps):
        return obj, ""
    cmd = [nvcc()] + ARCH + NVFLAGS + (["-Xptxas", "-v"] if verbose else []) + \
        ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    if force:
        for f in os.listdir(OBJ_DIR):
            os.remove(os.path.join(OBJ_DIR, f))
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    if force or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lcufft"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    # the command-line sweep driver (host C++ over the C ABI)
    src = os.path.join(CSRC, "tm_sweep.cpp")
    if force or _stale(SWEEP, [src, LIB]):
        cmd = [nvcc(), "-std=c++17", "-O2", "-o", SWEEP, src, "-L" + OUT_DIR, "-ltm",
               "-Xlinker", "-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"tm_sweep build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
