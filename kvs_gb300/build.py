"""Build recipe for libkvsmc.so: every CUDA source compiled for sm_103a.

    python -m kvs_gb300.build          # or kvs_gb300.build.build()

The translation units compile in parallel with nvcc and link into
kvs_gb300/lib/libkvsmc.so (git-ignored).  --fmad=false keeps every float and
double operation uncontracted: the kernels reproduce the reference's IEEE
operation sequence bit for bit.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB_DIR = os.path.join(PKG, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libkvsmc.so")
OBJ_DIR = os.path.join(PKG, "_build")

SOURCES = ["api.cu", "autotune.cu", "batch.cu", "cells.cu", "checksum.cu", "export.cu", "ingest.cu", "kvsml_export.cu", "slice.cu", "mc_gather.cu", "mc_snode.cu", "mc_stream.cu", "noalloc.cu", "plan.cu", "ply.cu", "profile.cu", "selftest.cu", "server.cu", "stl_ascii.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers_mtime():
    return max(os.path.getmtime(os.path.join(CSRC, f)) for f in os.listdir(CSRC)
               if f.endswith((".h", ".cuh"))) if os.path.isdir(CSRC) else 0


def _compile(src, extra):
    obj = os.path.join(OBJ_DIR, os.path.splitext(src)[0] + ".o")
    srcp = os.path.join(CSRC, src)
    newest = max(os.path.getmtime(srcp), _headers_mtime(),
                 os.path.getmtime(os.path.join(ROOT, "include", "kvsmc.h")),
                 os.path.getmtime(os.path.abspath(__file__)))
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj, ""
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", srcp, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr[-6000:]}")
    return obj, r.stderr


def build(verbose=False, extra=()):
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(SOURCES))) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra)), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err:
                print(err, file=sys.stderr)
    if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr[-4000:])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else []))
