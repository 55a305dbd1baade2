"""The C++ host interface (eulerian-liquid_gb300/host/) compiled into a C++ program that drives
the Simulator like the reference's app does."""

import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_cpp_host_interface(el):
    import importlib
    build = importlib.import_module("eulerian_liquid_gb300.build")
    exe = build.build_cpp_program(os.path.join(HERE, "cpp", "test_shim.cpp"), "test_shim")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok")
