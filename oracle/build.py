"""Build recipe for the oracle (test infrastructure only).

* ``build_oracle()`` compiles the CPU restatement ``oracle/oracle.cpp`` into
  ``oracle/_build/liboracle.so`` (g++, OpenMP, ``-ffp-contract=off`` so x86_64 and
  aarch64 round identically).
* ``build_ref(ref_root)`` compiles the reference's own code from its tree, unchanged, into
  ``oracle/_ref/libnama_ref.so``:

  - the Eigen-free header templates ``include/nama/math/interpolation.h`` and
    ``include/nama/math/ode.h``, through ``oracle/ref_adapter.cpp``;
  - the simulator sources ``src/project/3d/fluid/{projection,boundary,extrapolation,
    time_stepping,advection,levelset_emitter,reinitialization}.cpp``,
    ``src/project/3d/eulerian_liquid/{simulator,scene}.cpp`` and
    ``src/common/{meshing,mesh}.cpp`` with the vendored ``external/dualmc`` and
    ``external/tinyobjloader``, through ``oracle/ref_sim_adapter.cpp``.

  Eigen is not installed here, so these sources see the independently written Eigen-interface
  subset in ``oracle/eigen_min/`` (vectors, a compressed-row sparse matrix, and a textbook
  CG + IC(0) standing in for Eigen's ConjugateGradient/IncompleteCholesky).  The flags follow
  the reference's Release build (``-O3 -DNDEBUG``, CMakeLists.txt:23) with
  ``-ffp-contract=off`` (an x86-64 build without -march has no FMA to contract into).
  The GL visualisers, the app and the logger's file output are not compiled.  Run where the
  reference tree is present; elsewhere the step is skipped.

The reference tree defaults to ``/root/reference``; ``EL_REFERENCE_TREE`` overrides it.

Usage: ``python oracle/build.py [--ref /path/to/reference]``
"""

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_TREE = os.environ.get("EL_REFERENCE_TREE", "/root/reference")
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fvisibility=hidden"]
REF_CXXFLAGS = ["-O3", "-DNDEBUG", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off",
                "-fvisibility=hidden", "-w"]

# the reference's translation units compiled unchanged (paths inside its tree)
REF_SOURCES = [
    "src/project/3d/fluid/projection.cpp",
    "src/project/3d/fluid/boundary.cpp",
    "src/project/3d/fluid/extrapolation.cpp",
    "src/project/3d/fluid/time_stepping.cpp",
    "src/project/3d/fluid/advection.cpp",
    "src/project/3d/fluid/levelset_emitter.cpp",
    "src/project/3d/fluid/reinitialization.cpp",
    "src/project/3d/eulerian_liquid/simulator.cpp",
    "src/project/3d/eulerian_liquid/scene.cpp",
    "src/common/meshing.cpp",
    "src/common/mesh.cpp",
    "external/tinyobjloader/src/tiny_obj_loader.cc",
]


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
        subprocess.check_call(["g++", *CXXFLAGS, "-shared", src, "-o", out + ".tmp"])
        os.replace(out + ".tmp", out)
    return out


def reference_present(ref_root=None):
    ref_root = ref_root or REFERENCE_TREE
    return all(os.path.exists(os.path.join(ref_root, p)) for p in REF_SOURCES)


def build_ref(ref_root=None, force=False):
    """Compile the reference's code into oracle/_ref/libnama_ref.so; None without the tree."""
    ref_root = ref_root or REFERENCE_TREE
    if not reference_present(ref_root):
        return None
    inc = os.path.join(ref_root, "include")
    incs = ["-I", os.path.join(HERE, "eigen_min"), "-I", inc, "-I", os.path.join(ref_root, "external"),
            "-I", os.path.join(ref_root, "external", "tinyobjloader", "include")]
    out_dir = os.path.join(HERE, "_ref")
    obj_dir = os.path.join(out_dir, "obj")
    out = os.path.join(out_dir, "libnama_ref.so")
    eigen = [os.path.join(HERE, "eigen_min", "Eigen", h)
             for h in ("Core", "Geometry", "SparseCore", "IterativeLinearSolvers")]
    headers = []
    for d, _, files in os.walk(inc):
        headers += [os.path.join(d, f) for f in files if f.endswith(".h")]
    units = [(os.path.join(ref_root, s), REF_CXXFLAGS) for s in REF_SOURCES]
    units += [(os.path.join(HERE, "ref_adapter.cpp"), CXXFLAGS),
              (os.path.join(HERE, "ref_sim_adapter.cpp"), REF_CXXFLAGS)]
    objs = []
    jobs = []
    for src, flags in units:
        obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _needs_build(obj, [src, *eigen, *headers]):
            jobs.append(["g++", *flags, *incs, "-c", src, "-o", obj])
    if jobs or force or _needs_build(out, objs):
        os.makedirs(obj_dir, exist_ok=True)
        with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
            for f in [ex.submit(subprocess.check_call, j) for j in jobs]:
                f.result()
        subprocess.check_call(["g++", "-shared", "-fopenmp", *objs, "-o", out + ".tmp"])
        os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    ref = None
    if "--ref" in sys.argv:
        ref = sys.argv[sys.argv.index("--ref") + 1]
    print(build_oracle(force=True))
    print(build_ref(ref, force=True))
