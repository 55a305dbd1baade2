"""Batched scenes (el_batch_*): every scene's CFL sub-step in one CUDA graph launch, with dt and
the solver loops decided on the device.

The batch must reproduce, scene by scene, the host-driven path that Simulator::update
(simulator.cpp:23-42) describes: dt_sub = calc_time_step(cfl), cut at the frame end in float,
then one el_step with the mixed solver.  Both paths enqueue the same kernels -- the batch with
its dt and solver loops decided on the device -- and must take the same number of iterations;
the fields agree to FP32 round-off (measured: a few ulps after a step, ~1e-6 relative after
four), far inside the solve tolerance, so the test allows 1e-5 relative."""

import numpy as np
import pytest

import conftest
from conftest import rel_err

pytestmark = pytest.mark.gpu

FIELDS = ("phi", "u", "v", "w", "pressure")
MATCH = 1e-5


def _scene_set(el, specs):
    sims = []
    for spec in specs:
        ni, nj, nk = spec["shape"]
        sim = el.Simulator(ni, nj, nk, dtype=el.EL_F32)
        sim.init_scene(spec)
        sims.append(sim)
    return sims


def _specs(count, seed, lo, hi):
    return conftest.load_package().scenes.batch_scenes(count, seed, lo=lo, hi=hi)


def _params(el, sample_phi=None):
    return el.step_params(sample_phi=el.SAMPLE_WENO6 if sample_phi is None else sample_phi,
                          trace_vel=el.TRACE_RK3, gravity=9.8, solver=el.SOLVER_MIXED, tol=1e-6,
                          max_iter=400, check_every=4, max_outer=8)


def _host_substeps(el, sim, params, cfl, dt_frame, steps, frame_t=0.0):
    """Simulator::update's sub-stepping driven from the host through el_calc_time_step/el_step."""
    f32 = np.float32
    out = []
    for _ in range(steps):
        dt = f32(sim.calc_time_step(cfl))
        t = f32(frame_t)
        if dt_frame > 0 and t + dt > f32(dt_frame):
            dt = f32(dt_frame) - t
        st = sim.step(float(dt), params)
        out.append(st)
        t = f32(frame_t) + dt
        frame_t = 0.0 if (dt_frame > 0 and not t < f32(dt_frame)) else float(t)
    return out, frame_t


@pytest.mark.parametrize("cfl,dt_frame", [(1.0, 1.0 / 60.0), (3.0, 0.004)])
def test_batch_matches_host_driven_steps(el, cfl, dt_frame):
    specs = _specs(3, 7, 20, 44)
    params = _params(el)
    batch_sims = _scene_set(el, specs)
    host_sims = _scene_set(el, specs)
    batch = el.Batch(batch_sims, params=params, cfl=cfl, dt_frame=dt_frame)
    # an odd number of launches, then one more: both graphs and both buffer assignments
    batch.step(3)
    batch.step(1)
    stats = batch.stats()
    for q, (bs, hs) in enumerate(zip(batch_sims, host_sims)):
        host, frame_t = _host_substeps(el, hs, params, cfl, dt_frame, 4)
        for f in FIELDS:
            a, b = bs.download(f), hs.download(f)
            assert np.all(np.isfinite(a)), (q, f)
            assert rel_err(a, b) <= MATCH, (q, f, rel_err(a, b))
        st = stats[q]
        assert st["steps"] == 4 and st["bad_steps"] == 0 and st["no_fluid_steps"] == 0
        assert st["unconverged_steps"] == 0
        # the captured and the host-driven steps agree to FP32 round-off (MATCH), which can move a
        # solve's convergence across the tolerance by an iteration
        assert abs(st["iterations"] - sum(h["iterations"] for h in host)) <= st["steps"]
        assert st["outer_iterations"] == sum(h["outer_iterations"] for h in host)
        assert st["time"] == pytest.approx(sum(h["dt"] for h in host), rel=1e-12)
        assert st["frame_time"] == pytest.approx(frame_t, rel=1e-6, abs=1e-12)
        assert st["max_relres"] < 1e-6
        assert st["kernels"] > 0
    batch.close()
    for s in batch_sims + host_sims:
        s.close()


def test_batch_frames_and_reset(el):
    specs = _specs(2, 3, 24, 32)
    sims = _scene_set(el, specs)
    dt_frame = 0.003
    batch = el.Batch(sims, params=_params(el, el.SAMPLE_TRILINEAR), cfl=4.0, dt_frame=dt_frame)
    batch.step(6)
    st = batch.stats()
    for s in st:
        # every completed frame is dt_frame long; the clock holds the rest
        assert s["steps"] == 6
        assert s["time"] == pytest.approx(s["frames"] * dt_frame + s["frame_time"], rel=1e-5)
        assert s["last_dt"] <= dt_frame * (1 + 1e-6)
    batch.reset_stats()
    st2 = batch.stats()
    assert all(s["steps"] == 0 and s["iterations"] == 0 for s in st2)
    assert [s["frame_time"] for s in st2] == [s["frame_time"] for s in st]
    batch.step(2)
    assert all(s["steps"] == 2 for s in batch.stats())
    batch.close()
    for s in sims:
        s.close()


def test_batch_refuses_scene_stepped_outside(el):
    specs = _specs(2, 5, 20, 24)
    sims = _scene_set(el, specs)
    params = _params(el, el.SAMPLE_TRILINEAR)
    batch = el.Batch(sims, params=params, cfl=1.0)
    batch.step(1)
    sims[1].step(0.001, params)  # swaps that scene's buffers behind the batch's back
    with pytest.raises(el.ELError) as e:
        batch.step(1)
    assert e.value.status == el.EL_ERR_INVALID_ARGUMENT
    batch.close()
    for s in sims:
        s.close()


def test_batch_rejects_bad_arguments(el):
    sims = _scene_set(el, _specs(1, 1, 20, 20))
    with pytest.raises(el.ELError):
        el.Batch(sims + sims, params=_params(el))  # the same context twice
    with pytest.raises(el.ELError):
        el.Batch(sims, params=el.step_params(solver=el.SOLVER_JACOBI_FP64))
    for s in sims:
        s.close()


def test_autotune_picks_and_caches(el, tmp_path, monkeypatch):
    cache = tmp_path / "tuning.json"
    monkeypatch.setenv("EL_GB300_TUNING_CACHE", str(cache))
    specs = _specs(3, 9, 20, 36)
    sims = _scene_set(el, specs)
    params = _params(el, el.SAMPLE_TRILINEAR)
    before = [s.download("phi") for s in sims]
    cands = [(6, 8, 6, 4, 1), (2, 4, 3, 2, 0)]
    r = el.autotune.tune_batch(el, sims, params, device_name="test", steps=2, candidates=cands)
    assert not r["cached"] and len(r["trials"]) == 2 and cache.exists()
    # the scenes are back where they started and carry the chosen shapes
    for s, b in zip(sims, before):
        assert np.array_equal(s.download("phi"), b)
        assert s.get_tuning() == r["tuning"]
    # a second call hits the cache and applies the same shapes
    for s in sims:
        s.set_tuning(seg_blocks_per_sm=5)
    r2 = el.autotune.tune_batch(el, sims, params, device_name="test", steps=2, candidates=cands)
    assert r2["cached"] and r2["tuning"] == r["tuning"]
    assert all(s.get_tuning() == r["tuning"] for s in sims)
    # any tuning gives the same step to round-off of the reductions' order
    b = el.Batch(sims, params=params)
    b.step(2)
    st = b.stats()
    assert all(x["unconverged_steps"] == 0 and x["bad_steps"] == 0 for x in st)
    b.close()
    for s in sims:
        s.close()


def test_tuning_rejects_out_of_range(el):
    sim = el.Simulator(16, 16, 16)
    with pytest.raises(el.ELError):
        sim.set_tuning(seg_blocks_per_sm=9)
    with pytest.raises(el.ELError):
        sim.set_tuning(advect_rows=3)
    sim.set_tuning(seg_blocks_per_sm=2, advect_rows=8)
    assert sim.get_tuning()["seg_blocks_per_sm"] == 2 and sim.get_tuning()["advect_rows"] == 8
    sim.close()


def test_async_transfers_pipelined(el):
    """el_download_async / el_upload_async on two streams ordered by events (the benchmark's
    end-to-end pattern) move the same bytes as the synchronous copies."""
    torch = pytest.importorskip("torch")
    sim = el.Simulator(40, 24, 32, dtype=el.EL_F32)
    rng = np.random.default_rng(5)
    want = {f: rng.standard_normal(sim.shape(f)).astype(np.float32) for f in ("phi", "u", "v", "w")}
    pinned = {f: torch.empty(sim.shape(f), dtype=torch.float32, pin_memory=True).numpy() for f in want}
    back = {f: torch.empty(sim.shape(f), dtype=torch.float32, pin_memory=True).numpy() for f in want}
    s_up, s_down = torch.cuda.Stream(), torch.cuda.Stream()
    ev = {f: torch.cuda.Event() for f in want}
    for f, a in want.items():
        pinned[f][...] = a
        sim.upload_async(f, pinned[f], s_up.cuda_stream)
        ev[f].record(s_up)
    for f in want:
        s_down.wait_event(ev[f])
        sim.download_async(f, back[f], s_down.cuda_stream)
    torch.cuda.synchronize()
    for f, a in want.items():
        np.testing.assert_array_equal(back[f], a)
        np.testing.assert_array_equal(sim.download(f), a)
    with pytest.raises(ValueError):
        sim.download_async("phi", np.empty((3, 3, 3), np.float32))
    sim.close()
