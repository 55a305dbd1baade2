"""Pressure projection on the GPU vs the oracle (a7-a13): weights, cell flags and numbering,
ghost-fluid coefficients (bit-exact), the three solvers (to the solve tolerance, measured with the
oracle's own matrix) and the velocity update (bit-exact), plus the error paths."""

import numpy as np
import pytest

import conftest
from conftest import rel_err
from helpers import make_sim, residual_rel, scene_fields

pytestmark = pytest.mark.gpu

DTYPES = [np.float32, np.float64]


def _spec(n, seed=3):
    return conftest.load_package().scenes.spheres_pool(n, seed)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("n", [16, 23])
def test_scene_weights_and_solid_bitexact(el, orc, dtype, n):
    spec = _spec(n)
    phi, solid, (wu, wv, ww) = scene_fields(orc, spec, dtype)
    sim = make_sim(el, n, dtype, spec)
    np.testing.assert_array_equal(sim.download("phi"), phi)
    np.testing.assert_array_equal(sim.download("solid_nodal"), solid)
    np.testing.assert_array_equal(sim.download("weight_u"), wu)
    np.testing.assert_array_equal(sim.download("weight_v"), wv)
    np.testing.assert_array_equal(sim.download("weight_w"), ww)
    np.testing.assert_array_equal(sim.download("solid_cell"), orc.cell_solid_phi(solid))
    np.testing.assert_array_equal(sim.download("valid_phi"), (orc.cell_solid_phi(solid) >= 0).astype(np.uint8))
    sim.close()


@pytest.mark.parametrize("dtype", DTYPES)
def test_stateless_weights(el, orc, dtype):
    torch = pytest.importorskip("torch")
    n = 19
    _, solid, (wu, wv, ww) = scene_fields(orc, _spec(n, 8), dtype)
    ts = torch.from_numpy(solid).cuda()
    outs = [torch.empty(a.shape, dtype=ts.dtype, device="cuda") for a in (wu, wv, ww)]
    el.compute_staggered_grid_weight(n, n, n, 1.0 / n, el.EL_F64 if dtype == np.float64 else el.EL_F32,
                                     [o.data_ptr() for o in outs], ts.data_ptr())
    torch.cuda.synchronize()
    for o, want in zip(outs, (wu, wv, ww)):
        np.testing.assert_array_equal(o.cpu().numpy(), want)


def _velocity(orc, shape_src, dtype, seed):
    rng = np.random.default_rng(seed)
    return [rng.uniform(-1, 1, a.shape).astype(dtype) for a in shape_src]


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("n", [16, 29])
def test_assign_indices_and_build_matrix_bitexact(el, orc, dtype, n):
    spec = _spec(n)
    phi, solid, wts = scene_fields(orc, spec, dtype)
    u, v, w = _velocity(orc, wts, dtype, 4)
    sim = make_sim(el, n, dtype, spec)
    for f, a in (("u", u), ("v", v), ("w", w)):
        sim.upload(f, a)
    m, idx = sim.assign_indices()
    m_ref, idx_ref = orc.assign_indices(phi, *wts)
    assert m == m_ref
    np.testing.assert_array_equal(idx, idx_ref)
    dt = 0.013
    got = sim.build_matrix(dt)
    want = orc.build_matrix(phi, u, v, w, *wts, sim.dx, dt)
    for g, r, name in zip(got, want, ("diag", "offx", "offy", "offz", "rhs")):
        np.testing.assert_array_equal(g, r, err_msg=name)
    sim.close()


@pytest.mark.parametrize("dtype", DTYPES)
def test_build_matrix_wide_weight_range_bitexact(el, orc, dtype):
    """Face weights spread over forty binades (1, 2^-10, 2^-30, 2^-40 times U(0.1, 1), and zero):
    a row's diagonal terms then lie too far apart in exponent for the build's exact integer sum
    in many rows, which take the FP64 additions instead; every row, and the rhs's double sums
    of products of such weights, still equal the oracle's build."""
    n = 20
    spec = _spec(n)
    phi, _, wts = scene_fields(orc, spec, dtype)
    rng = np.random.default_rng(31)
    wide = []
    for a in wts:
        scale = rng.choice([1.0, 2.0 ** -10, 2.0 ** -30, 2.0 ** -40, 0.0], size=a.shape,
                           p=[0.55, 0.15, 0.1, 0.1, 0.1])
        wide.append((rng.uniform(0.1, 1.0, a.shape) * scale).astype(dtype))
    u, v, w = _velocity(orc, wts, dtype, 5)
    sim = make_sim(el, n, dtype, spec)
    for f, a in zip(("weight_u", "weight_v", "weight_w", "u", "v", "w"), (*wide, u, v, w)):
        sim.upload(f, a)
    dt = 0.013
    got = sim.build_matrix(dt)
    want = orc.build_matrix(phi, u, v, w, *wide, sim.dx, dt)
    for g, r, name in zip(got, want, ("diag", "offx", "offy", "offz", "rhs")):
        np.testing.assert_array_equal(g, r, err_msg=name)
    # the build the mixed solver runs (which also writes its FP32 / FP16 records) gives the same
    # system; the solve itself may stall on so ill-conditioned a matrix, which is not the point
    try:
        sim.solve_pressure(dt, solver=el.SOLVER_MIXED, tol=1e-3, max_iter=50)
    except RuntimeError:
        pass
    got = sim.matrix()
    for g, r, name in zip(got, want, ("diag", "offx", "offy", "offz", "rhs")):
        np.testing.assert_array_equal(g, r, err_msg=name)
    sim.close()


@pytest.mark.parametrize("m", [-100, 93])
def test_mixed_solve_is_scale_equivariant(el, orc, m):
    """FP32 fields with velocities scaled by 2^m (m = -100: |u| below 1e-30, pressures down to
    1e-32; m = 93: near 1e28; both keep every scaled velocity a normal float, so the scaled
    system is exactly the unscaled one times 2^m):
    the mixed solve still reaches the tolerance, and its pressure is the unscaled solve's times
    2^m -- the double-float residual holds b and x shifted by a power of two near |b| = 1, so
    neither a tiny nor a huge system leaves its pairs' exponent range, and every rounding of the
    solve scales with the system."""
    n = 24
    spec = _spec(n)
    _, _, wts = scene_fields(orc, spec, np.float32)
    u, v, w = _velocity(orc, wts, np.float32, 7)
    out = []
    for e in (0, m):
        sim = make_sim(el, n, np.float32, spec)
        for f, a in (("u", u), ("v", v), ("w", w)):
            sim.upload(f, np.ldexp(a, e).astype(np.float32))
        st = sim.solve_pressure(0.01, solver=el.SOLVER_MIXED, tol=1e-6)
        assert st["status"] == 0 and st["relres"] < 1e-6, (e, st)
        out.append((st, sim.download("pressure").astype(np.float64)))
        sim.close()
    (st0, p0), (st1, p1) = out
    assert st1["iterations"] == st0["iterations"], (st0, st1)
    np.testing.assert_allclose(p1, np.ldexp(p0, m), rtol=1e-6, atol=0)


@pytest.mark.parametrize("dtype", DTYPES)
def test_rebuild_after_the_fluid_moves_bitexact(el, orc, dtype):
    """Consecutive builds where the fluid region shrinks, moves and grows again: the build only
    rewrites rows that are or were nonzero, and every row (the zero ones included) still equals
    the oracle's build of the current scene, for the FP64 system and the mixed solver's records."""
    n = 24
    spec = _spec(n)
    _, solid, wts = scene_fields(orc, spec, dtype)
    sim = make_sim(el, n, dtype, spec)
    rng = np.random.default_rng(12)
    zs, ys, xs = np.meshgrid(*(np.arange(n) + 0.5 for _ in range(3)), indexing="ij")
    for step, (cx, cy, r) in enumerate(((12, 12, 9), (8, 14, 5), (16, 9, 7), (12, 12, 11))):
        phi = (np.sqrt((xs - cx) ** 2 + (ys - cy) ** 2 + (zs - 12) ** 2) - r).astype(dtype) * sim.dx
        u, v, w = _velocity(orc, wts, dtype, 20 + step)
        for f, a in (("phi", phi), ("u", u), ("v", v), ("w", w)):
            sim.upload(f, a)
        dt = 0.011
        st = sim.solve_pressure(dt, solver=el.SOLVER_MIXED, tol=1e-6)  # builds with the records
        assert st["status"] == 0, (step, st)
        got = sim.matrix()
        want = orc.build_matrix(phi, u, v, w, *wts, sim.dx, dt)
        for g, r, name in zip(got, want, ("diag", "offx", "offy", "offz", "rhs")):
            np.testing.assert_array_equal(g, r, err_msg=f"step {step} {name}")
    sim.close()


@pytest.mark.parametrize("dtype", DTYPES)
def test_update_velocity_using_pressure_bitexact(el, orc, dtype):
    n = 21
    spec = _spec(n, 6)
    phi, solid, wts = scene_fields(orc, spec, dtype)
    u, v, w = _velocity(orc, wts, dtype, 9)
    p = np.random.default_rng(2).standard_normal(phi.shape).astype(dtype)
    sim = make_sim(el, n, dtype, spec)
    for f, a in (("u", u), ("v", v), ("w", w), ("pressure", p)):
        sim.upload(f, a)
    sim.update_velocity_using_pressure(0.02)
    want = orc.update_velocity(u, v, w, p, phi, sim.dx, 0.02)
    for f, r in zip(("u", "v", "w"), want):
        np.testing.assert_array_equal(sim.download(f), r)
    sim.close()


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("solver", [0, 1, 2])
@pytest.mark.parametrize("n", [24, 40])
def test_solvers_reach_tolerance_on_oracle_matrix(el, orc, dtype, solver, n):
    spec = _spec(n, 12)
    phi, solid, wts = scene_fields(orc, spec, dtype)
    u, v, w = _velocity(orc, wts, dtype, 1)
    sim = make_sim(el, n, dtype, spec)
    for f, a in (("u", u), ("v", v), ("w", w)):
        sim.upload(f, a)
    dt = 0.01
    tol = 1e-6
    stats = sim.solve_pressure(dt, solver=solver, tol=tol, max_iter=5000)
    assert stats["status"] == 0, stats
    mats = orc.build_matrix(phi, u, v, w, *wts, sim.dx, dt)
    p = sim.download("pressure")
    # the GPU pressure, checked against the oracle's own matrix in FP64
    slack = 5.0 if dtype == np.float64 else 50.0  # FP32 pressure grid rounding
    assert residual_rel(orc, mats, p) <= slack * tol
    # against a tight oracle solve, the error is bounded by the conditioning times the residual
    x, st, it, rr = orc.pcg(*mats, precond=orc.PRE_MIC0, tol=1e-13, maxit=20000)
    assert rel_err(np.where(mats[0] > 0, p, 0), x) <= 2e-3
    # the velocity update used that pressure
    want = orc.update_velocity(u, v, w, p, phi, sim.dx, dt)
    for f, r in zip(("u", "v", "w"), want):
        np.testing.assert_array_equal(sim.download(f), r)
    assert stats["fluid_cells"] == int((mats[0] > 0).sum())
    sim.close()


def test_tight_fp64_solve_matches_oracle(el, orc):
    n = 32
    spec = _spec(n, 2)
    phi, solid, wts = scene_fields(orc, spec, np.float64)
    u, v, w = _velocity(orc, wts, np.float64, 3)
    sim = make_sim(el, n, np.float64, spec)
    for f, a in (("u", u), ("v", v), ("w", w)):
        sim.upload(f, a)
    for solver in (0, 1, 2):
        sim.upload("u", u), sim.upload("v", v), sim.upload("w", w)
        stats = sim.solve_pressure(0.01, solver=solver, tol=1e-12, max_iter=20000)
        assert stats["status"] == 0
        mats = orc.build_matrix(phi, u, v, w, *wts, sim.dx, 0.01)
        x, st, it, rr = orc.pcg(*mats, precond=orc.PRE_MIC0, tol=1e-14, maxit=20000)
        assert rel_err(sim.download("pressure"), x) <= 1e-8, solver
    sim.close()


def test_no_fluid_raises(el):
    n = 12
    spec = {"shape": (n, n, n), "liquid": [("pool", -1.0)], "solid": [("room",)]}
    sim = make_sim(el, n, np.float32, spec)
    with pytest.raises(el.NoFluid):
        sim.solve_pressure(0.01)
    with pytest.raises(el.NoFluid):
        sim.assign_indices()
    sim.close()


def test_not_converged_reported(el, orc):
    n = 24
    spec = _spec(n, 1)
    _, _, wts = scene_fields(orc, spec, np.float32)
    sim = make_sim(el, n, np.float32, spec)
    for f, a in zip(("u", "v", "w"), _velocity(orc, wts, np.float32, 5)):
        sim.upload(f, a)
    stats = sim.solve_pressure(0.01, solver=0, tol=1e-10, max_iter=1, check_every=1)
    assert stats["status"] == el.EL_ERR_NOT_CONVERGED and stats["iterations"] == 1
    sim.close()


def test_nan_input_reported(el, orc):
    n = 16
    spec = _spec(n, 1)
    _, _, wts = scene_fields(orc, spec, np.float32)
    phi, _, _ = scene_fields(orc, spec, np.float32)
    u, v, w = _velocity(orc, wts, np.float32, 5)
    D = orc.build_matrix(phi, u, v, w, *wts, 1.0 / n, 0.01)[0]
    k, j, i = np.argwhere(D > 0)[len(np.argwhere(D > 0)) // 2]
    u[k, j, i] = np.nan  # the -x face of a fluid cell enters the right-hand side
    sim = make_sim(el, n, np.float32, spec)
    for f, a in (("u", u), ("v", v), ("w", w)):
        sim.upload(f, a)
    with pytest.raises(el.ELError) as e:
        sim.solve_pressure(0.01, solver=2)
    assert e.value.status == el.EL_ERR_NAN
    sim.close()
