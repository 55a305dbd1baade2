"""The CPU oracle, pinned: golden vectors made by the reference's own templates, the known answers
of the reference's tests, and properties of the restated projection (CPU only)."""

import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

DTYPES = [(np.float32, "f32"), (np.float64, "f64")]


@pytest.mark.parametrize("dtype,suf", DTYPES)
@pytest.mark.parametrize("scheme", ["trilinear", "weno6"])
def test_advection_matches_reference_golden(orc, dtype, suf, scheme):
    g = np.load(os.path.join(GOLDEN, f"advect_{suf}.npz"))
    sample = orc.SAMPLE_WENO6 if scheme == "weno6" else orc.SAMPLE_TRILINEAR
    out = orc.advect_collocated(g["phi"], g["u"], g["v"], g["w"], float(g["dx"]), float(g["dt"]), orc.TRACE_RK2, sample)
    np.testing.assert_array_equal(out, g[f"phi_out_{scheme}"])
    ou, ov, ow = orc.advect_staggered(g["u"], g["v"], g["w"], float(g["dx"]), float(g["dt"]), orc.TRACE_RK2, sample)
    np.testing.assert_array_equal(ou, g[f"u_out_{scheme}"])
    np.testing.assert_array_equal(ov, g[f"v_out_{scheme}"])
    np.testing.assert_array_equal(ow, g[f"w_out_{scheme}"])


@pytest.mark.parametrize("dtype,suf", DTYPES)
def test_interpolation_matches_reference_golden(orc, dtype, suf):
    g = np.load(os.path.join(GOLDEN, f"interp_{suf}.npz"))
    dx = float(g["dx"])
    for n, p in enumerate(g["points"]):
        assert orc.sample_trilinear(g["phi"], (0.0, 0.0, 0.0), dx, p) == g["trilinear"][n]
        assert orc.sample_weno6(g["phi"], (0.0, 0.0, 0.0), dx, p) == g["weno6"][n]
        t = orc.trace(g["u"], g["v"], g["w"], dx, p, -float(g["dt"]), orc.TRACE_RK2)
        np.testing.assert_array_equal(t, g["traces"][n])


def test_reference_known_answers(orc):
    # test/math/interpolation.cpp:13-24: Grid1f(10, 0.1, 0)
    i, f = orc.index_fraction(0.0, 0.0, 0.1, np.float32)
    assert i == -1 and f == pytest.approx(0.5)
    i, f = orc.index_fraction(0.16, 0.0, 0.1, np.float32)
    assert i == 1 and abs(f - 0.1) < 0.1 * 0.01
    # test/math/interpolation.cpp:26-42: lerp / weno6 of an all-zero grid are 0
    for dtype in (np.float32, np.float64):
        z = np.zeros((10, 10, 10), dtype)
        assert orc.sample_trilinear(z, (0, 0, 0), 0.1, (0.5, 0.5, 0.5)) == 0
        assert orc.sample_weno6(z, (0, 0, 0), 0.1, (0.5, 0.5, 0.5)) == 0
    # test/common/grid.cpp:32-39: clamp-to-edge reads outside the grid
    g = np.full((1, 1, 10), 10.0, np.float32)
    g[0, 0, 0] = -10
    assert orc.sample_trilinear(g, (0.05, 0, 0), 0.1, (-0.5, 0.05, 0.05)) == pytest.approx(-10)


def test_oracle_matches_reference_templates_directly(orc):
    """When the reference tree was compiled here (oracle/_ref), compare on fresh seeded inputs."""
    import ctypes as C
    R = orc.ref_lib()
    if R is None:
        pytest.skip("oracle/_ref not built (reference tree absent)")
    rng = np.random.default_rng(7)
    ni, nj, nk = 9, 7, 11
    for dtype, suf in DTYPES:
        dx = orc.float_dx(ni, dtype)
        phi = rng.standard_normal((nk, nj, ni)).astype(dtype)
        u, v, w = (rng.standard_normal(orc.face_shape(ni, nj, nk, c)).astype(dtype) for c in range(3))
        for weno in (0, 1):
            a = orc.advect_collocated(phi, u, v, w, dx, 1.3 * dx, orc.TRACE_RK2, weno)
            b = np.empty_like(phi)
            getattr(R, f"ref_advect_collocated_{suf}")(ni, nj, nk, C.c_double(dx), orc._p(b), orc._p(phi),
                                                       orc._p(u), orc._p(v), orc._p(w), C.c_double(1.3 * dx), weno)
            np.testing.assert_array_equal(a, b)


def test_weno6_1d_matches_reference_golden(orc):
    import ctypes as C
    for dtype, suf in DTYPES:
        g = np.load(os.path.join(GOLDEN, f"interp_{suf}.npz"))
        # the oracle's 1-D WENO is reached through a 6-point-wide grid sampled on its axis
        for vals, f, want in zip(g["weno1d_values"], g["weno1d_fractions"], g["weno1d"]):
            line = np.ascontiguousarray(vals.reshape(1, 1, 6))
            x = (2 + float(f) + 0.5) * 1.0  # node 2 sits at position 2.5 with dx = 1
            got = orc.sample_weno6(np.repeat(np.repeat(line, 6, 0), 6, 1), (0, 0, 0), 1.0, (x, 2.5, 2.5))
            # the y and z passes see six equal values and return them within a rounding
            assert got == pytest.approx(float(want), rel=1e-5 if dtype == np.float32 else 1e-12, abs=1e-6)


def test_trilinear_exact_on_linear_fields(orc):
    ni, nj, nk = 8, 9, 10
    dx = 1.0 / ni
    zs, ys, xs = np.meshgrid((np.arange(nk) + 0.5) * dx, (np.arange(nj) + 0.5) * dx, (np.arange(ni) + 0.5) * dx,
                             indexing="ij")
    f = 0.3 + 1.5 * xs - 0.7 * ys + 2.0 * zs
    for p in [(0.31, 0.42, 0.55), (0.2, 0.6, 0.9)]:
        assert orc.sample_trilinear(f, (0, 0, 0), dx, p) == pytest.approx(0.3 + 1.5 * p[0] - 0.7 * p[1] + 2.0 * p[2],
                                                                          rel=1e-12)


def test_weno6_exact_on_cubics_away_from_walls(orc):
    n = 16
    dx = 1.0 / n
    zs, ys, xs = np.meshgrid(*((np.arange(n) + 0.5) * dx,) * 3, indexing="ij")
    f = 1 + xs ** 3 - 2 * ys ** 2 * xs + zs ** 3 * 0.5
    for p in [(0.47, 0.52, 0.49), (0.41, 0.55, 0.6)]:
        want = 1 + p[0] ** 3 - 2 * p[1] ** 2 * p[0] + p[2] ** 3 * 0.5
        assert orc.sample_weno6(f, (0, 0, 0), dx, p) == pytest.approx(want, rel=1e-9)


def _scene(orc, n, dtype, seed=3):
    import conftest
    el_scenes = conftest.load_package().scenes
    phi, solid = orc.rasterise(el_scenes.spheres_pool(n, seed), dtype)
    wu, wv, ww = orc.compute_weights(solid)
    return phi, solid, wu, wv, ww


def test_weights_in_unit_interval_and_room_walls_closed(orc):
    phi, solid, wu, wv, ww = _scene(orc, 16, np.float32)
    for a in (wu, wv, ww):
        assert a.min() >= 0 and a.max() <= 1
    # room: faces on the outer two node layers are closed (levelset_emitter.cpp:18-32)
    assert np.all(wu[:, :, :2] == 0) and np.all(wu[:, :, -2:] == 0)
    assert np.all(wv[:, :2, :] == 0) and np.all(ww[:2, :, :] == 0)


def test_fraction_inside_cases(orc):
    assert orc.fraction_inside(-1.0, -1.0) == 1
    assert orc.fraction_inside(1.0, 1.0) == 0
    assert orc.fraction_inside(-1.0, 3.0) == pytest.approx(0.25)
    assert orc.fraction_inside4(-1, -1, -1, -1) == 1
    assert orc.fraction_inside4(1, 1, 1, 1) == 0
    assert orc.fraction_inside4(-1, -1, 1, 1) == pytest.approx(0.5)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_matrix_symmetric_spd_and_pcg_matches_direct_solve(orc, dtype):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    phi, solid, wu, wv, ww = _scene(orc, 16, dtype)
    rng = np.random.default_rng(5)
    u, v, w = (rng.uniform(-1, 1, a.shape).astype(dtype) for a in (wu, wv, ww))
    dx = orc.float_dx(16, dtype)
    D, X, Y, Z, B = orc.build_matrix(phi, u, v, w, wu, wv, ww, dx, 0.01)
    n, idx = orc.assign_indices(phi, wu, wv, ww)
    assert n == int((D > 0).sum()) and n > 0
    # assign_indices numbers fluid cells in k-j-i order
    fl = idx.ravel() != np.iinfo(np.int32).max
    assert np.array_equal(idx.ravel()[fl], np.arange(n))
    # compact CSR in the reference's numbering
    rows, cols, vals = [], [], []
    nk, nj, ni = D.shape
    lin = idx.ravel()
    for a, (arr, step) in enumerate(((X, 1), (Y, ni), (Z, ni * nj))):
        c = np.nonzero(arr.ravel())[0]
        rows += [lin[c], lin[c + step]]
        cols += [lin[c + step], lin[c]]
        vals += [arr.ravel()[c], arr.ravel()[c]]
    dd = np.nonzero(D.ravel())[0]
    rows.append(lin[dd]); cols.append(lin[dd]); vals.append(D.ravel()[dd])
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    assert abs(A - A.T).max() == 0
    assert spl.eigsh(A, k=1, which="SA", return_eigenvectors=False)[0] > 0
    b = B.ravel()[dd]
    xd = spl.spsolve(A.tocsc(), b)
    for pre in (orc.PRE_JACOBI, orc.PRE_IC0, orc.PRE_MIC0):
        x, st, it, rr = orc.pcg(D, X, Y, Z, B, precond=pre, tol=1e-12, maxit=2000)
        assert st == 0 and rr < 1e-12
        assert np.max(np.abs(x.ravel()[dd] - xd)) <= 1e-8 * np.max(np.abs(xd))


def test_extrapolation_known_layers(orc):
    g = np.zeros((1, 1, 6), np.float32)
    valid = np.zeros_like(g, np.uint8)
    g[0, 0, 0] = 2.0
    valid[0, 0, 0] = 1
    out, m = orc.extrapolate(g, valid, layers=3)
    assert list(out[0, 0]) == [2, 2, 2, 2, 0, 0] and list(m[0, 0]) == [1, 1, 1, 1, 0, 0]


def test_oracle_reproduces_reference_step_fixture(orc):
    """tests/golden/step_ref_f32.npz holds one sub-step of the reference's own Simulator, piece
    by piece (tests/golden/make_golden.py); the FP32 restatement reproduces every piece exactly."""
    g = np.load(os.path.join(GOLDEN, "step_ref_f32.npz"))
    dx, dt = float(g["dx"]), float(g["dt"])
    solid = g["in_solid_nodal"]
    wts = orc.compute_weights(solid)
    for f, w in zip(("weight_u", "weight_v", "weight_w"), wts):
        np.testing.assert_array_equal(w, g[f"in_{f}"])
    np.testing.assert_array_equal(orc.cell_solid_phi(solid), g["in_solid_cell"])
    np.testing.assert_array_equal((g["in_solid_cell"] >= 0).astype(np.uint8), g["in_phi_valid"])
    assert orc.calc_time_step(g["in_u"], g["in_v"], g["in_w"], dx, 1.0) == dt
    ex = {}
    for f in "uvw":
        ex[f], m = orc.extrapolate(g[f"in_{f}"], np.ones(g[f"in_{f}"].shape, np.uint8), 10)
        np.testing.assert_array_equal(ex[f], g[f"extrap_{f}"])
        np.testing.assert_array_equal(m, g[f"extrap_valid_{f}"])
    phi_x, _ = orc.extrapolate(g["in_phi"], g["in_phi_valid"], 10)
    np.testing.assert_array_equal(phi_x, g["extrap_phi"])
    phi1 = orc.advect_collocated(phi_x, ex["u"], ex["v"], ex["w"], dx, dt)
    np.testing.assert_array_equal(phi1, g["advect_phi"])
    for f, a in zip("uvw", orc.advect_staggered(ex["u"], ex["v"], ex["w"], dx, dt)):
        np.testing.assert_array_equal(a, g[f"advect_{f}"])
    t = np.float32
    np.testing.assert_array_equal((g["advect_v"] - t(t(9.80665) * t(dt))).astype(np.float32), g["gravity_v"])
    masks = orc.find_valid_velocity(phi1, *wts)
    for f, m in zip("uvw", masks):
        np.testing.assert_array_equal(m, g[f"masks_valid_{f}"])
    n, idx = orc.assign_indices(g["advect_phi"], *wts)
    assert n == int(g["mat_size"])
    np.testing.assert_array_equal(idx, g["indices"])
    mats = orc.build_matrix(g["advect_phi"], g["masks_u"], g["masks_v"], g["masks_w"], *wts, dx, dt)
    for a, key in zip(mats, ("diag", "offx", "offy", "offz", "rhs")):
        np.testing.assert_array_equal(a, g[key])
    upd = orc.update_velocity(g["masks_u"], g["masks_v"], g["masks_w"], g["update_pressure"], g["advect_phi"], dx, dt)
    for a, f in zip(upd, "uvw"):
        np.testing.assert_array_equal(a, g[f"update_{f}"])
