"""Build recipe for the oracle (test infrastructure only).

* ``build_oracle()`` compiles the CPU restatement ``oracle/oracle.cpp`` into
  ``oracle/_build/liboracle.so`` (g++, OpenMP, ``-ffp-contract=off`` so x86_64 and
  aarch64 round identically).
* ``build_ref(ref_root)`` compiles ``oracle/ref_adapter.cpp`` against the reference's own
  header templates (``include/nama/math/interpolation.h``, ``include/nama/math/ode.h``)
  found under ``ref_root`` into ``oracle/_ref/libnama_ref.so``.  The rest of the reference
  needs Eigen, OpenGL/GLFW and GoogleTest, none of which exist here, so only these two
  Eigen-free headers are compiled.  Run with the reference tree present; on machines
  without it the step is skipped.

Usage: ``python oracle/build.py [--ref /path/to/reference]``
"""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
            "-fvisibility=hidden"]


def _needs_build(out, srcs):
    if not os.path.exists(out):
        return True
    mtime = os.path.getmtime(out)
    return any(os.path.getmtime(s) > mtime for s in srcs)


def build_oracle(force=False):
    src = os.path.join(HERE, "oracle.cpp")
    out_dir = os.path.join(HERE, "_build")
    out = os.path.join(out_dir, "liboracle.so")
    if force or _needs_build(out, [src]):
        os.makedirs(out_dir, exist_ok=True)
        subprocess.check_call(["g++", *CXXFLAGS, src, "-o", out + ".tmp"])
        os.replace(out + ".tmp", out)
    return out


def build_ref(ref_root, force=False):
    inc = os.path.join(ref_root, "include")
    hdrs = [os.path.join(inc, "nama", "math", "interpolation.h"),
            os.path.join(inc, "nama", "math", "ode.h")]
    if not all(os.path.exists(h) for h in hdrs):
        return None
    src = os.path.join(HERE, "ref_adapter.cpp")
    out_dir = os.path.join(HERE, "_ref")
    out = os.path.join(out_dir, "libnama_ref.so")
    if force or _needs_build(out, [src, *hdrs]):
        os.makedirs(out_dir, exist_ok=True)
        subprocess.check_call(["g++", *CXXFLAGS, "-I", inc, src, "-o", out + ".tmp"])
        os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    ref = None
    if "--ref" in sys.argv:
        ref = sys.argv[sys.argv.index("--ref") + 1]
    print(build_oracle(force=True))
    if ref:
        print(build_ref(ref, force=True))
