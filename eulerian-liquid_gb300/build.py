"""Build the GB300 hot-path library ``_build/libeulerian_liquid_gb300.so`` in-tree.

Every CUDA translation unit under ``csrc/`` is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked into one shared
library whose exported symbols are exactly the C ABI of ``include/eulerian_liquid_gb300.h``.

The C++ host interface in ``host/`` (the reference's fluid:: functions and Simulator methods
over that ABI) is compiled on the caller's side: ``build_cpp_program`` compiles it together with
a C++ program and links the library, as a C++ user of the reference would.
Usage: ``python eulerian-liquid_gb300/build.py [--force]``.
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
# the debug build: every kernel index check on (-DEL_CHECKED); objects in _build/checked/
LIB_CHECKED = os.path.join(OUT_DIR, "libeulerian_liquid_gb300_checked.so")

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
    return cu, []


def headers():
    hs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs


def _compile(src, checked=False):
    obj_dir = os.path.join(OUT_DIR, "checked") if checked else OUT_DIR
    obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *(["-DEL_CHECKED"] if checked else []), "-c", src, "-o", obj]
    else:
        cmd = [nvcc(), "-x", "c++", "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
               "-fvisibility=hidden", "-I", os.path.join(ROOT, "include"), "-I", HOST, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def up_to_date(checked=False):
    lib = LIB_CHECKED if checked else LIB
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    cu, cpp = sources()
    return all(os.path.getmtime(f) <= t for f in cu + cpp + headers() + [__file__])


def build(force=False, verbose=False, checked=False):
    """The product library, or with checked=True the debug build with the kernels' index checks."""
    lib = LIB_CHECKED if checked else LIB
    if not force and up_to_date(checked):
        return lib
    os.makedirs(os.path.join(OUT_DIR, "checked") if checked else OUT_DIR, exist_ok=True)
    cu, cpp = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda f: _compile(f, checked), cu + cpp))
    tmp = lib + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    if verbose:
        print(lib)
    return lib


def build_cpp_program(main_src, out_name, force=False):
    """Compile a C++ program with the host interface (host/shim.cpp) against the library."""
    lib = build()
    out = os.path.join(OUT_DIR, out_name)
    srcs = [main_src, os.path.join(HOST, "shim.cpp"), os.path.join(HOST, "nama_gb300.h")]
    if not force and os.path.exists(out) and all(os.path.getmtime(f) <= os.path.getmtime(out) for f in srcs + [lib]):
        return out
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
    libdirs = [d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib")) if os.path.isdir(d)]
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I", HOST, "-I",
           os.path.join(cuda, "include"), main_src, os.path.join(HOST, "shim.cpp"), "-o", out + ".tmp", "-L", OUT_DIR,
           "-leulerian_liquid_gb300", "-Wl,-rpath," + OUT_DIR]
    for d in libdirs:
        cmd += ["-L", d, "-Wl,-rpath," + d]
    cmd += ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, checked="--checked" in sys.argv)
