"""Build the GB300 hot-path library ``_build/libeulerian_liquid_gb300.so`` in-tree.

Every CUDA translation unit under ``csrc/`` is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked into one shared
library whose exported symbols are exactly the C ABI of
``include/eulerian_liquid_gb300.h``.  The C++ host shim (``host/``) is compiled into the same
library.  Usage: ``python eulerian-liquid_gb300/build.py [--force]``.
"""

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libeulerian_liquid_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden", "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def nvcc():
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def sources():
    cu = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = []
    if os.path.isdir(HOST):
        cpp = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".cpp"))
    return cu, cpp


def headers():
    hs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    if os.path.isdir(HOST):
        for dp, _, fs in os.walk(HOST):
            hs += [os.path.join(dp, f) for f in fs if f.endswith((".h", ".hpp"))]
    return hs


def _compile(src):
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
    else:
        cmd = [nvcc(), "-x", "c++", "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
               "-fvisibility=hidden", "-I", os.path.join(ROOT, "include"), "-I", HOST, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    cu, cpp = sources()
    return all(os.path.getmtime(f) <= t for f in cu + cpp + headers() + [__file__])


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cu, cpp = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, cu + cpp))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
