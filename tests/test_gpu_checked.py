"""The debug build (compiled with -DEL_CHECKED): the main kernels check their store indices
(and indirect loads) against the arrays before each access and record a failed check instead
of making the access.  Steps of the FP32 tile and segment solvers, the FP64 multigrid and the
batch graph on it leave the check word clear."""

import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_checked_build_runs_clean(el):
    import importlib
    build = importlib.import_module("eulerian_liquid_gb300.build")
    build.build(checked=True)
    env = dict(os.environ, EL_CHECKED="1")
    r = subprocess.run([sys.executable, os.path.join(HERE, "checked_run.py")], capture_output=True, text=True,
                       timeout=900, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    line = r.stdout.strip().splitlines()[-1]
    assert line.endswith("check_word 0"), line
    assert "batch_bad 0" in line, line
    assert "statuses [0, 0, 0, 0, 0]" in line, line
