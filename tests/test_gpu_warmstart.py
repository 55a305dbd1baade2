"""Warm start of the pressure solve: the solver's initial-guess path, the network's inputs and
targets, and what a trained network gains over the zero initial guess.

A warm-started solve runs to the same relative residual as a solve from zero, so its pressure
must agree with the zero-guess solve to the solve tolerance; only the iteration count may
change."""

import numpy as np
import pytest

import conftest
from conftest import rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SOLVERS = ("SOLVER_JACOBI_FP64", "SOLVER_MG_FP64", "SOLVER_MIXED")


def _pool_sim(el, n=32, seed=3, steps=2):
    pkg = conftest.load_package()
    sim = el.Simulator(n, n, n, dtype=el.EL_F32)
    sim.init_scene(pkg.scenes.spheres_pool(n, seed))
    prm = el.step_params(solver=el.SOLVER_MIXED, tol=1e-6, max_iter=500)
    for _ in range(steps):  # some flow, so that the right-hand side is not trivial
        sim.step(min(sim.calc_time_step(1.0), 1 / 60), prm)
    return sim


def _solve(el, sim, dt, solver, tol, guess=None, **kw):
    saved = {f: sim.download(f) for f in ("u", "v", "w")}
    if guess is not None:
        sim.upload("pressure", guess.astype(np.float32))
    st = sim.solve_pressure(dt, solver=solver, tol=tol, max_iter=5000, check_every=4,
                            initial_guess=int(guess is not None), **kw)
    p = sim.download("pressure")
    for f, a in saved.items():
        sim.upload(f, a)
    return st, p


@pytest.mark.parametrize("solver_name", SOLVERS)
def test_initial_guess_paths(el, solver_name):
    solver = getattr(el, solver_name)
    sim = _pool_sim(el)
    dt = 1.0 / 120.0
    tol = 1e-8
    st0, p0 = _solve(el, sim, dt, solver, tol)
    assert st0["status"] == el.EL_OK and st0["iterations"] > 0
    fluid = p0 != 0
    # zero guess: the scaling factor is 0, the solve starts exactly where a solve from zero does
    stz, pz = _solve(el, sim, dt, solver, tol, guess=np.zeros_like(p0))
    assert stz["iterations"] == st0["iterations"]
    assert rel_err(pz, p0) < 1e-12
    # the converged pressure as the guess: nothing left to do (the pressure grid is FP32, so the
    # stored solution meets 1e-5, not the 1e-8 it was solved to)
    ste, pe = _solve(el, sim, dt, solver, 1e-5, guess=p0)
    assert ste["status"] == el.EL_OK and ste["iterations"] == 0
    assert rel_err(pe, p0) < 1e-6
    # a perturbed solution: fewer iterations, same answer to the tolerance
    rng = np.random.default_rng(0)
    noisy = p0 * (1 + 0.01 * rng.standard_normal(p0.shape)).astype(np.float32)
    stn, pn = _solve(el, sim, dt, solver, tol, guess=noisy)
    assert stn["status"] == el.EL_OK and stn["iterations"] < st0["iterations"]
    assert rel_err(pn, p0) < 1e-5
    # garbage (huge and random, also off the fluid): still the same answer
    junk = (1e6 * rng.standard_normal(p0.shape)).astype(np.float32)
    stj, pj = _solve(el, sim, dt, solver, tol, guess=junk)
    assert stj["status"] == el.EL_OK
    assert rel_err(pj, p0) < 1e-5
    assert np.all(pj[~fluid] == 0)
    sim.close()


def test_features_targets_and_guess_round_trip(el):
    W = el.warmstart
    L = W.lib()
    sim = _pool_sim(el)
    n = sim.ni
    feat = torch.empty((n, n, n, 16), dtype=torch.bfloat16, device="cuda")
    target = torch.empty((n, n, n), dtype=torch.float32, device="cuda")
    fluid = torch.empty((n, n, n), dtype=torch.uint8, device="cuda")
    import ctypes as C
    coup = torch.empty((n, n, n, 4), dtype=torch.bfloat16, device="cuda")
    scales = (C.c_double * 3)()
    # after a step: the system that step solved and its pressure
    assert L.el_warmstart_features(sim.h, 0, 0.0, feat.data_ptr(), coup.data_ptr(), target.data_ptr(),
                                   fluid.data_ptr(), scales) == 0
    torch.cuda.synchronize()
    p = sim.download("pressure").astype(np.float64)
    phi = sim.download("phi").astype(np.float64)
    solid = sim.download("solid_cell")
    f = feat.float().cpu().numpy()
    fl = fluid.cpu().numpy().astype(bool)
    assert fl.sum() > 0
    # channel 0: clamp(phi / 3dx), channel 2: solid mask, the rest zero
    assert rel_err(f[..., 0], np.clip(phi / (3 * sim.dx), -1, 1)) < 1e-2
    assert np.array_equal(f[..., 2] > 0.5, solid < 0)
    assert np.all(f[..., 3:] == 0)
    # target = p * a / rms(b) on fluid cells
    rms, a = scales[0], scales[1]
    assert rms > 0 and a > 0
    assert rel_err(target.cpu().numpy(), np.where(fl, p * a / rms, 0)) < 1e-6
    # channel 1 is b / rms(b): unit root-mean-square over the fluid
    b1 = f[..., 1][fl].astype(np.float64)
    assert abs(np.sqrt(np.mean(b1 * b1)) - 1.0) < 1e-2
    # couplings: the scaled matrix in Laplacian form (diagonal excess, face weights +x, +y, +z)
    diag, offx, offy, offz, _ = sim.matrix()
    cp = coup.float().cpu().numpy().astype(np.float64)
    for k, off in ((1, offx), (2, offy), (3, offz)):
        assert rel_err(cp[..., k] * a, np.where(fl, -off, 0)) < 1e-2
    t = target.cpu().numpy().astype(np.float64)
    At = cp[..., 0] * t
    energy = float(np.sum(cp[..., 0] * t * t))
    for k, ax in ((1, 2), (2, 1), (3, 0)):
        w = np.moveaxis(cp[..., k], ax, 0)[:-1]
        tt = np.moveaxis(t, ax, 0)
        d = tt[:-1] - tt[1:]
        flux = w * d
        np.moveaxis(At, ax, 0)[:-1] += flux
        np.moveaxis(At, ax, 0)[1:] -= flux
        energy += float(np.sum(w * d * d))
    # the energy of the scaled solution, t . A^ t = t . b^
    assert abs(energy - scales[2]) < 2e-2 * scales[2]
    # A^ t reproduces b^ (to the bf16 rounding of the couplings and the solve tolerance)
    assert rel_err(np.where(fl, At, 0), np.where(fl, f[..., 1], 0)) < 3e-2
    # set_guess(target) puts the pressure back
    sim.upload("pressure", np.zeros_like(p, dtype=np.float32))
    assert L.el_warmstart_set_guess(sim.h, target.data_ptr()) == 0
    back = sim.download("pressure").astype(np.float64)
    assert rel_err(back, np.where(fl, p, 0)) < 1e-6
    sim.close()


def test_trained_network_beats_zero_guess(el):
    """Record solves from seeded scenes, train briefly, and compare iterations to 1e-6 of the
    plain FP64 PCG from the learned guess and from zero on held-out scenes."""
    W = el.warmstart
    pkg = conftest.load_package()
    n = 32
    torch.manual_seed(0)
    prm = el.step_params(solver=el.SOLVER_MIXED, tol=1e-6, max_iter=500)
    specs = [pkg.scenes.spheres_pool(n, s) for s in range(8)]
    ds = W.record(el, torch, specs, 6, (n, n, n), prm)
    assert len(ds) == 48
    net = W.WarmStartNet(torch, seed=0, lr=2e-3)
    out = W.train(net, ds, epochs=30, batch=2, log=24)
    hist = [h[1] for h in out["history"]]
    assert hist[-1] < 0.5 * hist[0], hist
    zero_it, warm_it = [], []
    for seed in (100, 101, 102):
        sim = el.Simulator(n, n, n, dtype=el.EL_F32)
        sim.init_scene(pkg.scenes.spheres_pool(n, seed))
        for _ in range(3):
            dt = min(sim.calc_time_step(1.0), 1 / 60)
            saved = {f: sim.download(f) for f in ("phi", "u", "v", "w", "valid_u", "valid_v", "valid_w")}
            st0 = sim.step(dt, el.step_params(solver=el.SOLVER_JACOBI_FP64, tol=1e-6, max_iter=5000))
            p0 = sim.download("pressure")
            for f, a in saved.items():
                sim.upload(f, a)
            # the same step with the learned guess: advance to the projection, predict, solve
            sim.extrapolate_velocity(10)
            sim.extrapolate_level_set(10)
            sim.advect_level_set(dt)
            sim.advect_velocity(dt)
            sim.add_gravity(dt, el.REFERENCE_GRAVITY)
            sim.find_valid_velocity()
            sim.set_invalid_velocity_zero()
            W.predict_guess(net, sim, dt)
            st1 = sim.solve_pressure(dt, solver=el.SOLVER_JACOBI_FP64, tol=1e-6, max_iter=5000, initial_guess=1)
            assert st1["status"] == el.EL_OK
            assert rel_err(sim.download("pressure"), p0) < 1e-4
            zero_it.append(st0["iterations"])
            warm_it.append(st1["iterations"])
        sim.close()
    assert np.mean(warm_it) < np.mean(zero_it), (zero_it, warm_it)
