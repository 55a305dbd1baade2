"""The step pieces (extrapolation, gravity, valid masks, time step) bit-exact against the oracle,
and whole steps of the benchmark workloads against the oracle's composition of
update_second_order (apps/eulerian_liquid_3d.cpp:106-120) without reinitialisation."""

import numpy as np
import pytest

import conftest
from conftest import rel_err
from helpers import RTOL_F64, make_sim, oracle_step, scene_fields, smooth_fields

pytestmark = pytest.mark.gpu

DTYPES = [np.float32, np.float64]


@pytest.mark.parametrize("dtype", DTYPES)
def test_extrapolation_bitexact(el, orc, dtype):
    n = 20
    spec = conftest.load_package().scenes.spheres_pool(n, 4)
    phi, solid, wts = scene_fields(orc, spec, dtype)
    rng = np.random.default_rng(8)
    vel = [rng.uniform(-1, 1, a.shape).astype(dtype) for a in wts]
    sim = make_sim(el, n, dtype, spec)
    for f, a in zip(("u", "v", "w"), vel):
        sim.upload(f, a)
    sim.find_valid_velocity()
    masks = orc.find_valid_velocity(phi, *wts)
    for f, m in zip(("valid_u", "valid_v", "valid_w"), masks):
        np.testing.assert_array_equal(sim.download(f), m)
    sim.extrapolate_velocity(10)
    for f, a, m in zip(("u", "v", "w"), vel, masks):
        g, mm = orc.extrapolate(a, m, 10)
        np.testing.assert_array_equal(sim.download(f), g)
        np.testing.assert_array_equal(sim.download("valid_" + f), mm)
    # level set: extrapolate_const leaves the mask alone
    vphi = sim.download("valid_phi")
    sim.extrapolate_level_set(3)
    g, _ = orc.extrapolate(phi, vphi, 3)
    np.testing.assert_array_equal(sim.download("phi"), g)
    np.testing.assert_array_equal(sim.download("valid_phi"), vphi)
    sim.close()


@pytest.mark.parametrize("dtype", DTYPES)
def test_gravity_masks_zero_and_time_step(el, orc, dtype):
    n = 18
    spec = conftest.load_package().scenes.dam_break(n)
    phi, solid, wts = scene_fields(orc, spec, dtype)
    rng = np.random.default_rng(3)
    vel = [rng.uniform(-2, 2, a.shape).astype(dtype) for a in wts]
    sim = make_sim(el, n, dtype, spec)
    for f, a in zip(("u", "v", "w"), vel):
        sim.upload(f, a)
    cfl = 1.0
    assert sim.calc_time_step(cfl) == orc.calc_time_step(*vel, sim.dx, cfl)
    dt = 0.0123
    sim.add_gravity(dt, 9.80665)
    t = dtype
    want_v = (vel[1] - t(t(9.80665) * t(dt))).astype(dtype)
    np.testing.assert_array_equal(sim.download("v"), want_v)
    sim.find_valid_velocity()
    sim.set_invalid_velocity_zero()
    masks = orc.find_valid_velocity(phi, *wts)
    for f, a, m in zip(("u", "v", "w"), (vel[0], want_v, vel[2]), masks):
        np.testing.assert_array_equal(sim.download(f), np.where(m == 0, 0, a).astype(dtype))
    sim.close()


def _state_from_sim(sim, orc, spec, dtype):
    phi, solid, wts = scene_fields(orc, spec, dtype)
    st = {"phi": phi, "weights": wts, "dx": sim.dx, "valid_phi": sim.download("valid_phi")}
    for f in ("u", "v", "w"):
        st[f] = sim.download(f)
        st["valid_" + f] = sim.download("valid_" + f)
    return st


@pytest.mark.parametrize("scheme", [(0, 0, 0, 0), (0, 1, 1, 0), (1, 1, 1, 1)])
def test_full_step_fp64_matches_oracle(el, orc, scheme):
    n = 32
    spec = conftest.load_package().scenes.dam_break(n)
    sim = make_sim(el, n, np.float64, spec)
    rng = np.random.default_rng(21)
    # seeded velocity noise on every face sample (the config-2 initial condition)
    for f, shp in zip(("u", "v", "w"), (sim.shape("u"), sim.shape("v"), sim.shape("w"))):
        sim.upload(f, rng.uniform(-1e-3, 1e-3, shp))
    state = _state_from_sim(sim, orc, spec, np.float64)
    for step in range(2):
        dt = min(sim.calc_time_step(1.0), 1.0 / 60.0)
        stats = sim.step(dt, trace_phi=scheme[0], sample_phi=scheme[1], trace_vel=scheme[2],
                         sample_vel=scheme[3], solver=el.SOLVER_MG_FP64, tol=1e-12, max_iter=5000)
        assert stats["status"] == 0
        state, mats = oracle_step(orc, state, dt, *scheme, el.REFERENCE_GRAVITY)
        # the advected level set is not touched by the projection: 1e-12
        assert rel_err(sim.download("phi"), state["phi"]) <= RTOL_F64
        for f in ("u", "v", "w"):
            assert rel_err(sim.download(f), state[f]) <= 1e-9, f
        assert rel_err(sim.download("pressure"), state["pressure"]) <= 1e-9
        # carry the GPU state forward so both sides start the next step from the same fields
        for f in ("phi", "u", "v", "w"):
            state[f] = sim.download(f)
    sim.close()


def test_mixed_step_fp32_matches_oracle_to_solve_tolerance(el, orc):
    n = 40
    spec = conftest.load_package().scenes.spheres_pool(n, 7)
    sim = make_sim(el, n, np.float32, spec)
    state = _state_from_sim(sim, orc, spec, np.float32)
    dt = 1.0 / 60.0
    stats = sim.step(dt, sample_phi=1, trace_vel=1, solver=el.SOLVER_MIXED, tol=1e-6, gravity=9.8)
    assert stats["status"] == 0 and stats["relres"] < 1e-6
    state, mats = oracle_step(orc, state, dt, 0, 1, 1, 0, 9.8)
    assert rel_err(sim.download("phi"), state["phi"]) <= 2e-5
    from helpers import residual_rel
    # the GPU pressure satisfies the oracle's system to the solve tolerance (FP32 grid rounding)
    assert residual_rel(orc, mats, sim.download("pressure")) <= 5e-5
    sim.close()


@pytest.mark.parametrize("shape,density,layers", [((23, 17, 30), 0.02, 10), ((40, 9, 12), 0.3, 3),
                                                  ((12, 33, 20), 0.0005, 40), ((16, 16, 16), 0.9, 1),
                                                  ((18, 14, 11), 0.05, 0), ((300, 37, 19), 0.002, 7),
                                                  ((33, 70, 17), 0.01, 6), ((9, 6, 5), 0.01, 260)])
def test_extrapolation_random_masks_bitexact(el, orc, shape, density, layers):
    """The bitmask layer loop against the oracle's layer loop on random masks and non-cubic
    grids: few valid cells (long reach), dense masks, rows of more than 256 cells and more than
    32 rows (several dilation tiles along each axis, rows of 301 cells ending inside a word),
    more layers than the grid is wide, no layers at all."""
    ni, nj, nk = shape
    rng = np.random.default_rng(ni * 1000 + layers)
    for dtype in DTYPES:
        sim = make_sim(el, shape, dtype)
        vel = {}
        for f in ("u", "v", "w", "phi"):
            vel[f] = rng.standard_normal(sim.shape(f)).astype(dtype)
            sim.upload(f, vel[f])
            m = (rng.random(sim.shape(f)) < density).astype(np.uint8)
            vel["valid_" + f] = m
            sim.upload("valid_" + f, m)
        sim.extrapolate_velocity(layers)
        sim.extrapolate_level_set(layers)
        for f in ("u", "v", "w", "phi"):
            g, mm = orc.extrapolate(vel[f], vel["valid_" + f], layers)
            np.testing.assert_array_equal(sim.download(f), g, err_msg=f)
            # extrapolate_const leaves the level set's mask alone
            want_mask = vel["valid_" + f] if f == "phi" else mm
            np.testing.assert_array_equal(sim.download("valid_" + f), want_mask, err_msg=f)
        sim.close()
