"""GPU parity at the benchmark workloads' own sizes, and on the timed path, against the CPU oracle.

* 64^3 FP64 dam break, trilinear/RK2 (the first workload), three full steps;
* 128^3 FP64 dam break with seeded U(-1e-3, 1e-3) face velocities, WENO6/RK2 level set and
  trilinear/RK3 velocity (the second workload), one full step;
* the batch graph (el_batch_step, the headline's timed path) for a batch of one 48^3
  spheres-and-pool scene, compared with the oracle's step directly;
* a 128^3 FP32 step with the mixed-precision solver: its pressure against a CPU oracle PCG
  solve to 1e-12 of the same system;
* fluid touching an open domain edge (no walls).

Bars: advected fields 1e-12 relative in FP64; the pressure of an FP64 solve to 1e-12 within
1e-9; FP32 fields to FP32 round-off; the mixed solve's pressure within 1e-6 of the oracle's.
"""

import numpy as np
import pytest

import conftest
from conftest import rel_err
from helpers import RTOL_F32, RTOL_F64, make_sim, oracle_step, residual_rel, scene_fields

pytestmark = pytest.mark.gpu


def _state_from_sim(sim, orc, spec, dtype):
    phi, solid, wts = scene_fields(orc, spec, dtype)
    st = {"phi": sim.download("phi"), "weights": wts, "dx": sim.dx, "valid_phi": sim.download("valid_phi")}
    for f in ("u", "v", "w"):
        st[f] = sim.download(f)
        st["valid_" + f] = sim.download("valid_" + f)
    return st


def _next_dt(sim, cfl=1.0, frame=1.0 / 60.0):
    return min(sim.calc_time_step(cfl), frame)


def test_dam_break_64_fp64_three_steps(el, orc):
    n = 64
    spec = conftest.load_package().scenes.dam_break(n)
    sim = make_sim(el, n, np.float64, spec)
    state = _state_from_sim(sim, orc, spec, np.float64)
    scheme = (el.TRACE_RK2, el.SAMPLE_TRILINEAR, el.TRACE_RK2, el.SAMPLE_TRILINEAR)
    for step in range(3):
        dt = _next_dt(sim)
        assert dt == min(orc.calc_time_step(state["u"], state["v"], state["w"], sim.dx, 1.0), 1.0 / 60.0)
        stats = sim.step(dt, trace_phi=scheme[0], sample_phi=scheme[1], trace_vel=scheme[2], sample_vel=scheme[3],
                         gravity=9.8, solver=el.SOLVER_MG_FP64, tol=1e-12, max_iter=5000)
        assert stats["status"] == 0
        state, mats = oracle_step(orc, state, dt, *scheme, 9.8)
        assert state["pcg_status"] == 0
        assert rel_err(sim.download("phi"), state["phi"]) <= RTOL_F64, step
        assert rel_err(sim.download("pressure"), state["pressure"]) <= 1e-9, step
        for f in ("u", "v", "w"):
            assert rel_err(sim.download(f), state[f]) <= 1e-9, (step, f)
        for f in ("phi", "u", "v", "w"):
            state[f] = sim.download(f)
    # the workload's own solver setting: plain FP64 PCG to 1e-6, judged on the oracle's matrix
    state = _state_from_sim(sim, orc, spec, np.float64)
    dt = _next_dt(sim)
    stats = sim.step(dt, trace_phi=scheme[0], sample_phi=scheme[1], trace_vel=scheme[2], sample_vel=scheme[3],
                     gravity=9.8, solver=el.SOLVER_JACOBI_FP64, tol=1e-6, max_iter=20000)
    assert stats["status"] == 0 and stats["relres"] < 1e-6
    state, mats = oracle_step(orc, state, dt, *scheme, 9.8)
    assert residual_rel(orc, mats, sim.download("pressure")) < 1.0001e-6
    sim.close()


def test_dam_break_128_fp64_weno6_rk3(el, orc):
    n = 128
    spec = conftest.load_package().scenes.dam_break(n)
    sim = make_sim(el, n, np.float64, spec)
    rng = np.random.default_rng(0)
    for f in ("u", "v", "w"):
        sim.upload(f, rng.uniform(-1e-3, 1e-3, sim.shape(f)))
    state = _state_from_sim(sim, orc, spec, np.float64)
    scheme = (el.TRACE_RK2, el.SAMPLE_WENO6, el.TRACE_RK3, el.SAMPLE_TRILINEAR)
    dt = _next_dt(sim)
    stats = sim.step(dt, trace_phi=scheme[0], sample_phi=scheme[1], trace_vel=scheme[2], sample_vel=scheme[3],
                     gravity=9.8, solver=el.SOLVER_MG_FP64, tol=1e-12, max_iter=5000)
    assert stats["status"] == 0
    state, mats = oracle_step(orc, state, dt, *scheme, 9.8)
    assert state["pcg_status"] == 0
    assert rel_err(sim.download("phi"), state["phi"]) <= RTOL_F64
    assert rel_err(sim.download("pressure"), state["pressure"]) <= 1e-9
    for f in ("u", "v", "w"):
        assert rel_err(sim.download(f), state[f]) <= 1e-9, f
    sim.close()


def test_batch_graph_of_one_scene_matches_oracle(el, orc):
    """The headline's timed path: one graph launch per sub-step, dt and solver loops on the device."""
    n = 48
    spec = conftest.load_package().scenes.spheres_pool(n, 5)
    sim = make_sim(el, n, np.float32, spec)
    rng = np.random.default_rng(12)
    for f in ("u", "v", "w"):
        sim.upload(f, rng.uniform(-0.3, 0.3, sim.shape(f)).astype(np.float32))
    state = _state_from_sim(sim, orc, spec, np.float32)
    params = el.step_params(trace_phi=el.TRACE_RK2, sample_phi=el.SAMPLE_TRILINEAR, trace_vel=el.TRACE_RK3,
                            sample_vel=el.SAMPLE_TRILINEAR, gravity=9.8, solver=el.SOLVER_MIXED, tol=1e-6,
                            max_iter=400, check_every=4, max_outer=8)
    dt = np.float32(orc.calc_time_step(state["u"], state["v"], state["w"], sim.dx, 1.0))
    dt = float(min(dt, np.float32(1.0 / 60.0)))
    batch = el.Batch([sim], params=params, cfl=1.0, dt_frame=1.0 / 60.0)
    batch.step(1)
    batch.sync()
    st = batch.stats()[0]
    got = {f: sim.download(f) for f in ("phi", "pressure")}
    batch.close()
    assert st["steps"] == 1 and st["unconverged_steps"] == 0 and st["bad_steps"] == 0
    assert st["time"] == pytest.approx(dt, rel=1e-7)
    state, mats = oracle_step(orc, state, dt, el.TRACE_RK2, el.SAMPLE_TRILINEAR, el.TRACE_RK3,
                              el.SAMPLE_TRILINEAR, 9.8)
    assert rel_err(got["phi"], state["phi"]) <= RTOL_F32
    # the graph's pressure solves the oracle's own system to the tolerance (FP32 grid rounding)
    assert residual_rel(orc, mats, got["pressure"]) <= 5e-5
    assert rel_err(got["pressure"], state["pressure"]) <= 1e-4
    sim.close()


def test_mixed_solver_128_pressure_vs_fp64_oracle_solve(el, orc):
    """The mixed FP32-inner / FP64-refined solve to 1e-6 against the oracle's FP64 PCG to 1e-12
    on the same system: pressure error <= 1e-6 relative."""
    n = 128
    spec = conftest.load_package().scenes.spheres_pool(n, 0)
    sim = make_sim(el, n, np.float32, spec)
    rng = np.random.default_rng(3)
    for f in ("u", "v", "w"):
        sim.upload(f, rng.uniform(-0.2, 0.2, sim.shape(f)).astype(np.float32))
    stats = sim.step(1.0 / 60.0, sample_phi=el.SAMPLE_WENO6, trace_vel=el.TRACE_RK3, gravity=9.8,
                     solver=el.SOLVER_MIXED, tol=1e-6)
    assert stats["status"] == 0 and stats["relres"] < 1e-6
    mats = sim.matrix()
    x, st, it, rr = orc.pcg(*mats, precond=orc.PRE_MIC0, tol=1e-12, maxit=20000)
    assert st == 0 and rr < 1e-12
    p_ref = np.where(mats[0] > 0, x, 0.0)
    err = rel_err(sim.download("pressure"), p_ref)
    assert err <= 1e-6, err
    sim.close()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_fluid_on_open_domain_edges(el, orc, dtype):
    """No walls: a pool fills the bottom layer and the x/z edges, every face is open.  A cell's
    neighbour outside the grid is absent (no coupling, no diagonal term), the rule of the oracle;
    the reference would read outside its arrays there (projection.cpp:8-12,70).  The GPU's
    build equals the oracle's bit for bit, and the solve converges."""
    n = 20
    spec = {"name": "open_pool", "shape": (n, n, n), "liquid": [("pool", 0.35), ("sphere", 0.5, 0.7, 0.5, 0.15)],
            "solid": [("box", (2.0, 2.0, 2.0), (3.0, 3.0, 3.0))]}
    phi, solid, wts = scene_fields(orc, spec, dtype)
    assert all(np.all(w == 1) for w in wts)
    sim = make_sim(el, n, dtype, spec)
    rng = np.random.default_rng(2)
    vel = [rng.uniform(-0.5, 0.5, a.shape).astype(dtype) for a in wts]
    for f, a in zip("uvw", vel):
        sim.upload(f, a)
    dt = 0.4 * sim.dx
    n_gpu, idx = sim.assign_indices()
    n_orc, idx_orc = orc.assign_indices(phi, *wts)
    assert n_gpu == n_orc
    np.testing.assert_array_equal(idx, idx_orc)
    live = idx != np.iinfo(np.int32).max
    assert live[0].any() and live[:, :, 0].any() and live[:, :, -1].any()   # fluid on the edges
    got = sim.build_matrix(dt)
    want = orc.build_matrix(phi, *vel, *wts, sim.dx, dt)
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)
    stats = sim.solve_pressure(dt, solver=el.SOLVER_MIXED if dtype == np.float32 else el.SOLVER_MG_FP64, tol=1e-8)
    assert stats["status"] == 0
    assert residual_rel(orc, want, sim.download("pressure")) <= (5e-5 if dtype == np.float32 else 1e-8)
    sim.close()
