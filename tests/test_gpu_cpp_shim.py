"""The C++ host interface (eulerian-liquid_gb300/host/) compiled into a C++ program that drives
the Simulator like the reference's app does, and one step it takes compared with the oracle."""

import os
import subprocess

import numpy as np
import pytest

from conftest import rel_err
from helpers import RTOL_F32, oracle_step, residual_rel

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
N = 32                 # the program's grid (tests/cpp/test_shim.cpp)
DT = 1.0 / 240.0       # its fixed last step
GRAVITY = 9.80665      # Simulator::gravity of the host interface


def _run(tmp_path):
    import importlib
    build = importlib.import_module("eulerian_liquid_gb300.build")
    exe = build.build_cpp_program(os.path.join(HERE, "cpp", "test_shim.cpp"), "test_shim")
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok")


def test_cpp_host_interface(el, orc, tmp_path):
    _run(tmp_path)

    def rd(name, dtype, shape):
        return np.fromfile(os.path.join(tmp_path, name), dtype=dtype).reshape(shape)

    cell = (N, N, N)
    faces = [tuple(orc.face_shape(N, N, N, c)) for c in range(3)]
    state = {"phi": rd("in_phi", np.float32, cell), "valid_phi": rd("in_valid_phi", np.uint8, cell),
             "dx": orc.float_dx(N, np.float32),
             "weights": tuple(rd("weight_" + f, np.float32, s) for f, s in zip("uvw", faces))}
    for f, s in zip("uvw", faces):
        state[f] = rd("in_" + f, np.float32, s)
        state["valid_" + f] = rd("in_valid_" + f, np.uint8, s)
    # the program's step: trilinear / RK2 for both fields, the mixed solver to 1e-6
    ref, mats = oracle_step(orc, state, DT, 0, 0, 0, 0, GRAVITY)
    assert rel_err(rd("out_phi", np.float32, cell), ref["phi"]) <= RTOL_F32
    p = rd("out_pressure", np.float32, cell)
    # the pressure solves the oracle's system to the solve tolerance (FP32 grid rounding)
    assert residual_rel(orc, mats, p) <= 5e-5
    # the velocity is the oracle's pre-projection velocity updated with that pressure
    want = orc.update_velocity(*ref["pre_projection"], p, ref["phi"], state["dx"], DT)
    for f, s, a in zip("uvw", faces, want):
        assert rel_err(rd("out_" + f, np.float32, s), a) <= RTOL_F32, f
