"""Runs the hot path on the debug build of the library (EL_CHECKED=1: every guarded kernel index
is checked before its access) and prints the check word; launched by tests/test_gpu_checked.py
in a process of its own, since a process loads one build of the library."""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import conftest  # noqa: E402


def main():
    assert os.environ.get("EL_CHECKED") == "1"
    el = conftest.load_package()
    el.load()
    checked, word = el.debug_check_take()
    assert checked, "the debug build was not loaded"
    rng = np.random.default_rng(3)

    def scene(shape, dtype, seed):
        spec = dict(el.scenes.spheres_pool(shape[0], seed), shape=shape)
        sim = el.Simulator(*shape, dtype=dtype)
        sim.init_scene(spec)
        for f in ("u", "v", "w"):
            sim.upload(f, rng.uniform(-0.3, 0.3, sim.shape(f)).astype(np.float32 if dtype == el.EL_F32 else np.float64))
        return sim

    runs = []
    # FP32: the tile solver (64 x 40 x 32), then the row-segment solver, WENO6 / RK3
    for tiles in (1, 0):
        sim = scene((64, 40, 32), el.EL_F32, 5)
        sim.set_tuning(solver_tiles=tiles)
        for _ in range(2):
            st = sim.step(min(sim.calc_time_step(1.0), 1.0 / 60.0), sample_phi=el.SAMPLE_WENO6,
                          trace_vel=el.TRACE_RK3, solver=el.SOLVER_MIXED, tol=1e-6, gravity=9.8)
            runs.append(st["status"])
        sim.close()
    # FP64 with the FP64 multigrid, trilinear / RK2, an uneven grid
    sim = scene((27, 19, 23), el.EL_F64, 6)
    st = sim.step(0.005, solver=el.SOLVER_MG_FP64, tol=1e-8, gravity=9.8)
    runs.append(st["status"])
    sim.close()
    # the batch graph: two scenes of different sizes
    params = el.step_params(sample_phi=el.SAMPLE_WENO6, trace_vel=el.TRACE_RK3, gravity=9.8,
                            solver=el.SOLVER_MIXED, tol=1e-6, max_iter=400, check_every=4, max_outer=8)
    scenes = [scene((64, 48, 40), el.EL_F32, 7), scene((40, 36, 24), el.EL_F32, 8)]
    batch = el.Batch(scenes, params=params, cfl=1.0, dt_frame=1.0 / 60.0)
    batch.step(2)
    batch.sync()
    bad = sum(s["bad_steps"] for s in batch.stats())
    batch.close()
    for s in scenes:
        s.close()
    checked, word = el.debug_check_take()
    print(f"statuses {runs} batch_bad {bad} check_word {word}")


if __name__ == "__main__":
    main()
