"""The C-ABI library builds, loads and exports every entry point include/*.h declares (CPU only:
no compute calls)."""

import ctypes as C
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z_0-9]*\s*\**\s+\**(el_[a-z_0-9]+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    for n in ("el_ctx_create", "el_advect_level_set", "el_advect_velocity", "el_solve_pressure", "el_step",
              "el_advect_collocated_grid", "el_advect_staggered_grid", "el_compute_staggered_grid_weight"):
        assert n in names


def test_library_loads_and_exports_every_declared_symbol(el):
    lib = el.load()
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings(el):
    lib = el.load()
    assert el.status_string(el.EL_ERR_NO_FLUID) == "No fluid"
    assert el.status_string(el.EL_OK) == "ok"


def test_invalid_arguments_rejected_without_gpu_work(el):
    lib = el.load()
    h = C.c_void_p()
    assert lib.el_ctx_create(0, 4, 4, 0.25, el.EL_F32, 0, C.byref(h)) == el.EL_ERR_INVALID_ARGUMENT
    assert lib.el_ctx_create(4, 4, 4, -1.0, el.EL_F32, 0, C.byref(h)) == el.EL_ERR_INVALID_ARGUMENT
    assert lib.el_ctx_create(4, 4, 4, 0.25, 7, 0, C.byref(h)) == el.EL_ERR_INVALID_ARGUMENT
    assert lib.el_ctx_destroy(None) == el.EL_ERR_INVALID_ARGUMENT
    g = el.Grid(0, 1, 1, 1.0)
    assert lib.el_advect_collocated_grid(C.byref(g), el.EL_F32, 1, 2, 3, 4, 5, 0.1, 0, 0, None) == \
        el.EL_ERR_INVALID_ARGUMENT
