"""The mixed solver's finest level on the z-marching tile kernels (TMA-staged planes,
csrc/el_march.cu) against the same solver on the row-segment kernels, and against the oracle's
matrix.  The two paths evaluate the same expressions; only the dot products' summation order
differs, so solves to a tight tolerance agree to that tolerance and take the same number of
iterations within one."""

import numpy as np
import pytest

import conftest
from conftest import rel_err
from helpers import residual_rel

pytestmark = pytest.mark.gpu

SHAPES = [(64, 64, 64), (96, 72, 80), (128, 40, 56)]


def _scene(el, shape, seed):
    spec = dict(conftest.load_package().scenes.spheres_pool(shape[0], seed), shape=shape)
    sim = el.Simulator(*shape, dtype=el.EL_F32)
    sim.init_scene(spec)
    rng = np.random.default_rng(seed)
    for f in ("u", "v", "w"):
        sim.upload(f, rng.uniform(-0.4, 0.4, sim.shape(f)).astype(np.float32))
    return sim


def _update_class(el, sim, dt, tiles):
    """A profiled mixed solve: the update class's launches and algorithmic bytes (36 bytes per
    active cell on the tile path, where the update is fused with the pre-smoother; 24 on the
    segment path)."""
    sim.set_tuning(solver_tiles=tiles)
    sim.profile_begin(1 << el.EL_KC_UPDATE)
    st = sim.solve_pressure(dt, solver=el.SOLVER_MIXED, tol=1e-6)
    return st, sim.profile_end()["update"]


@pytest.mark.parametrize("shape", SHAPES)
def test_tiles_match_segments(el, orc, shape):
    sims = [_scene(el, shape, 4), _scene(el, shape, 4)]
    sims[0].set_tuning(solver_tiles=1)
    sims[1].set_tuning(solver_tiles=0)
    dt = 0.01
    stats = [s.solve_pressure(dt, solver=el.SOLVER_MIXED, tol=1e-10, max_iter=400) for s in sims]
    for st in stats:
        assert st["status"] == 0 and st["relres"] < 1e-10, st
    assert abs(stats[0]["iterations"] - stats[1]["iterations"]) <= stats[0]["outer_iterations"], stats
    p = [s.download("pressure") for s in sims]
    assert rel_err(p[0], p[1]) <= 2e-7   # both FP64 solutions to 1e-10, stored in FP32
    for f in ("u", "v", "w"):
        assert rel_err(sims[0].download(f), sims[1].download(f)) <= 1e-6, f
    mats = sims[0].matrix()
    assert residual_rel(orc, mats, p[0]) <= 5e-5   # FP32 pressure grid rounding
    # and the product tolerance: same iteration count within one per refinement sweep
    for s in sims:
        s.close()


def test_tile_path_is_taken_where_supported(el):
    sim = _scene(el, (64, 64, 64), 2)
    per_launch = {}
    for tiles in (1, 0):
        st, entry = _update_class(el, sim, 0.01, tiles)
        assert st["status"] == 0 and entry["launches"] > 0
        per_launch[tiles] = entry["bytes"] / entry["launches"]
    assert per_launch[1] / per_launch[0] == pytest.approx(36.0 / 24.0, rel=1e-9)
    sim.close()
    # a grid the tile kernels do not take (ni not a multiple of 8) runs the segments either way
    sim = _scene(el, (60, 64, 64), 2)
    st, entry = _update_class(el, sim, 0.01, 1)
    st0, entry0 = _update_class(el, sim, 0.01, 0)
    assert entry["bytes"] / entry["launches"] == pytest.approx(entry0["bytes"] / entry0["launches"], rel=1e-12)
    sim.close()


def test_batch_graph_on_tiles_matches_host_driven(el):
    """A batch of one 64^3 scene (the tile kernels inside the captured step's conditional loops)
    against host-driven steps of the same scene."""
    shape = (64, 64, 64)
    params = el.step_params(sample_phi=el.SAMPLE_WENO6, trace_vel=el.TRACE_RK3, gravity=9.8,
                            solver=el.SOLVER_MIXED, tol=1e-6, max_iter=400, check_every=4, max_outer=8)
    a, b = _scene(el, shape, 9), _scene(el, shape, 9)
    batch = el.Batch([a], params=params, cfl=1.0, dt_frame=1.0 / 60.0)
    batch.step(3)
    batch.sync()
    st = batch.stats()[0]
    fields = {f: a.download(f) for f in ("phi", "u", "v", "w", "pressure")}
    batch.close()
    iters = 0
    f32 = np.float32
    frame_t = f32(0)
    for _ in range(3):
        # Simulator::update's sub-step rule (simulator.cpp:28-36), in float
        dt = f32(b.calc_time_step(1.0))
        if frame_t + dt > f32(1.0 / 60.0):
            dt = f32(1.0 / 60.0) - frame_t
        h = b.step(float(dt), params)
        assert h["status"] == 0
        iters += h["iterations"]
        frame_t = f32(frame_t + dt)
        if not frame_t < f32(1.0 / 60.0):
            frame_t = f32(0)
    assert st["steps"] == 3 and st["unconverged_steps"] == 0 and st["bad_steps"] == 0
    assert abs(st["iterations"] - iters) <= 3
    for f, v in fields.items():
        assert np.all(np.isfinite(v)), f
        assert rel_err(v, b.download(f)) <= 1e-5, f
    a.close()
    b.close()
