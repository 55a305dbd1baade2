"""The mixed solver's coarse multigrid levels in one cooperative launch per V-cycle
(mg_coarse_cycle_kernel, csrc/el_solve.cu) against the per-level launches: the same device
functions in the same order, so the pressure, the iteration counts and the velocity are
bit-identical, on the tile path and on the segment path of the finest level, host-driven and
inside the batch's captured graph; and the fused path launches fewer kernels."""

import numpy as np
import pytest

import conftest
from helpers import residual_rel

pytestmark = pytest.mark.gpu


def _scene(el, shape, seed):
    spec = dict(conftest.load_package().scenes.spheres_pool(shape[0], seed), shape=shape)
    sim = el.Simulator(*shape, dtype=el.EL_F32)
    sim.init_scene(spec)
    rng = np.random.default_rng(seed)
    for f in ("u", "v", "w"):
        sim.upload(f, rng.uniform(-0.4, 0.4, sim.shape(f)).astype(np.float32))
    return sim


@pytest.mark.parametrize("shape,tiles,level", [((96, 72, 80), 1, 1), ((96, 72, 80), 0, 1), ((70, 50, 60), 1, 1),
                                              ((96, 72, 80), 1, 2), ((160, 120, 136), 1, 2)])
def test_fused_coarse_cycle_is_bit_identical(el, orc, shape, tiles, level):
    """level: the first level of the fused cycle (coarse_fused = 1 or 2)."""
    sims = [_scene(el, shape, 3), _scene(el, shape, 3)]
    out = []
    for sim, fused in zip(sims, (level, 0)):
        sim.set_tuning(solver_tiles=tiles, coarse_fused=fused)
        sim.profile_begin(1 << el.EL_KC_MG_COARSE)
        st = sim.solve_pressure(0.01, solver=el.SOLVER_MIXED, tol=1e-8, max_iter=400)
        prof = sim.profile_end()["mg_coarse"]
        assert st["status"] == 0 and st["relres"] < 1e-8, st
        out.append((st, prof, {f: sim.download(f) for f in ("pressure", "u", "v", "w")}))
    (st1, prof1, f1), (st0, prof0, f0) = out
    assert st1["iterations"] == st0["iterations"] and st1["outer_iterations"] == st0["outer_iterations"]
    for f in f1:
        np.testing.assert_array_equal(f1[f], f0[f], err_msg=f)
    # one launch per V-cycle instead of four per level pass pair plus the bottom
    assert prof1["launches"] < prof0["launches"] / (3 if level == 1 else 1.3), (prof1, prof0)
    assert residual_rel(orc, sims[0].matrix(), f1["pressure"]) <= 5e-5
    for s in sims:
        s.close()


def test_fused_coarse_cycle_in_batch_graph(el):
    """Three batch sub-steps of two scenes of different sizes with the fused coarse cycle inside
    the captured conditional loops, against the same batch with per-level launches."""
    params = el.step_params(sample_phi=el.SAMPLE_WENO6, trace_vel=el.TRACE_RK3, gravity=9.8,
                            solver=el.SOLVER_MIXED, tol=1e-6, max_iter=400, check_every=4, max_outer=8)
    results = []
    for fused in (1, 0):
        scenes = [_scene(el, (64, 64, 64), 5), _scene(el, (48, 56, 40), 6)]
        for s in scenes:
            s.set_tuning(coarse_fused=fused)
        batch = el.Batch(scenes, params=params, cfl=1.0, dt_frame=1.0 / 60.0)
        batch.step(3)
        batch.sync()
        stats = batch.stats()
        results.append(([{f: s.download(f) for f in ("phi", "u", "v", "w", "pressure")} for s in scenes],
                        [(st["iterations"], st["bad_steps"], st["unconverged_steps"]) for st in stats]))
        batch.close()
        for s in scenes:
            s.close()
    (f1, s1), (f0, s0) = results
    assert s1 == s0 and all(b == 0 and u == 0 for _, b, u in s1), (s1, s0)
    for a, b in zip(f1, f0):
        for f in a:
            np.testing.assert_array_equal(a[f], b[f], err_msg=f)


@pytest.mark.parametrize("tiles", [1, 0])
def test_dependent_launch_is_bit_identical(el, tiles):
    """The solver's chained kernels as programmatic dependent launches (each scheduled while the
    one before it drains) give the same bits as ordinary launches, host-driven and in a batch."""
    shape = (96, 72, 80)
    out = []
    for pdl in (1, 0):
        sim = _scene(el, shape, 11)
        sim.set_tuning(solver_tiles=tiles, dependent_launch=pdl)
        st = sim.solve_pressure(0.01, solver=el.SOLVER_MIXED, tol=1e-8, max_iter=400)
        assert st["status"] == 0, st
        params = el.step_params(sample_phi=el.SAMPLE_WENO6, trace_vel=el.TRACE_RK3, gravity=9.8,
                                solver=el.SOLVER_MIXED, tol=1e-6, max_iter=400, check_every=4, max_outer=8)
        batch = el.Batch([sim], params=params, cfl=1.0, dt_frame=1.0 / 60.0)
        batch.step(2)
        batch.sync()
        bst = batch.stats()[0]
        batch.close()
        out.append((st["iterations"], bst["iterations"], {f: sim.download(f) for f in ("pressure", "u", "phi")}))
        sim.close()
    assert out[0][0] == out[1][0] and out[0][1] == out[1][1]
    for f in out[0][2]:
        np.testing.assert_array_equal(out[0][2][f], out[1][2][f], err_msg=f)
