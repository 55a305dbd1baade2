"""The GPU FP32 path against the reference's own outputs: tests/golden/step_ref_f32.npz holds
one sub-step of update_second_order (without reinitialize()) run piece by piece on the
reference's Simulator, compiled from its own sources (tests/golden/make_golden.py).  Each GPU
piece starts from the fixture's input to that piece, so every comparison is independent."""

import os

import numpy as np
import pytest

from conftest import rel_err
from helpers import RTOL_F32

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "step_ref_f32.npz")


@pytest.fixture(scope="module")
def g():
    return np.load(GOLDEN)


@pytest.fixture
def sim(el, g):
    ni, nj, nk = (int(x) for x in g["shape"])
    s = el.Simulator(ni, nj, nk, dtype=el.EL_F32)
    assert s.dx == float(g["dx"])
    s.upload("solid_nodal", g["in_solid_nodal"])
    s.upload("phi", g["in_phi"])
    for f in "uvw":
        s.upload(f, g[f"in_{f}"])
    yield s
    s.close()


def test_boundary_pieces_bitexact(sim, g):
    sim.calc_cell_centered_solid_phi()
    sim.compute_weights()
    sim.find_valid_level_set()
    np.testing.assert_array_equal(sim.download("solid_cell"), g["in_solid_cell"])
    np.testing.assert_array_equal(sim.download("valid_phi"), g["in_phi_valid"])
    for f in ("weight_u", "weight_v", "weight_w"):
        np.testing.assert_array_equal(sim.download(f), g[f"in_{f}"])
    assert sim.calc_time_step(1.0) == float(g["dt"])


def test_extrapolation_bitexact(sim, g):
    sim.compute_weights()
    for f in "uvw":
        sim.upload("valid_" + f, np.ones(sim.shape("valid_" + f), np.uint8))
    sim.upload("valid_phi", g["in_phi_valid"])
    sim.extrapolate_velocity(10)
    sim.extrapolate_level_set(10)
    for f in "uvw":
        np.testing.assert_array_equal(sim.download(f), g[f"extrap_{f}"])
        np.testing.assert_array_equal(sim.download("valid_" + f), g[f"extrap_valid_{f}"])
    np.testing.assert_array_equal(sim.download("phi"), g["extrap_phi"])


def test_advection_trilinear_rk2(sim, g):
    dt = float(g["dt"])
    sim.upload("phi", g["extrap_phi"])
    for f in "uvw":
        sim.upload(f, g[f"extrap_{f}"])
    sim.advect_level_set(dt)
    sim.advect_velocity(dt)
    assert rel_err(sim.download("phi"), g["advect_phi"]) <= RTOL_F32
    for f in "uvw":
        assert rel_err(sim.download(f), g[f"advect_{f}"]) <= RTOL_F32, f


def test_gravity_masks_and_zero_bitexact(sim, g):
    dt = float(g["dt"])
    sim.compute_weights()
    sim.upload("phi", g["advect_phi"])
    for f in "uvw":
        sim.upload(f, g[f"advect_{f}"])
    sim.add_gravity(dt, 9.80665)
    np.testing.assert_array_equal(sim.download("v"), g["gravity_v"])
    sim.find_valid_velocity()
    sim.set_invalid_velocity_zero()
    for f in "uvw":
        np.testing.assert_array_equal(sim.download("valid_" + f), g[f"masks_valid_{f}"])
        np.testing.assert_array_equal(sim.download(f), g[f"masks_{f}"])


def test_matrix_and_velocity_update_bitexact(sim, g):
    dt = float(g["dt"])
    sim.compute_weights()
    sim.upload("phi", g["advect_phi"])
    for f in "uvw":
        sim.upload(f, g[f"masks_{f}"])
    n, idx = sim.assign_indices()
    assert n == int(g["mat_size"])
    np.testing.assert_array_equal(idx, g["indices"])
    for a, key in zip(sim.build_matrix(dt), ("diag", "offx", "offy", "offz", "rhs")):
        np.testing.assert_array_equal(a, g[key])
    sim.upload("pressure", g["update_pressure"])
    sim.update_velocity_using_pressure(dt)
    for f in "uvw":
        np.testing.assert_array_equal(sim.download(f), g[f"update_{f}"])
