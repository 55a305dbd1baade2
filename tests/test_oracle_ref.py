"""The oracle's projection side, pinned bit for bit against the reference's own sources.

oracle/build.py compiles the reference's projection.cpp, boundary.cpp, extrapolation.cpp,
time_stepping.cpp, advection.cpp, levelset_emitter.cpp, scene.cpp, simulator.cpp,
meshing.cpp and mesh.cpp unchanged (against the Eigen-interface subset in oracle/eigen_min)
into oracle/_ref/libnama_ref.so.  Here the CPU restatement's FP32 instantiation
(oracle/oracle.cpp), which the GPU FP32 path is tested against, must give exactly the
reference's bits on seeded scenes.  CPU only; skipped where the reference tree is absent.
"""

import os

import numpy as np
import pytest

import conftest

orc_mod = pytest.importorskip("oracle")


@pytest.fixture(scope="module")
def ref(orc):
    if not orc.ref_sim_available():
        pytest.skip("the reference was not compiled here (no reference tree)")
    return orc


def _scenes():
    el = conftest.load_package()
    return [el.scenes.water_drop(24), el.scenes.spheres_pool(28, 3), el.scenes.dam_break(20),
            dict(el.scenes.spheres_pool(24, 8), shape=(24, 18, 30))]


def _random_velocity(orc, ni, nj, nk, seed, scale=0.7):
    rng = np.random.default_rng(seed)
    return [(scale * rng.standard_normal(orc.face_shape(ni, nj, nk, c))).astype(np.float32) for c in range(3)]


def _ref_scene(orc, spec):
    """The reference's Simulator with the spec's sphere / pool / room emitters; a box emitter
    (new here) is written into the nodal solid field after init_scene."""
    ni, nj, nk = spec["shape"]
    sim = orc.RefSimulator(ni, nj, nk)
    boxes = []
    for e in spec["liquid"]:
        if e[0] == "sphere":
            sim.add_sphere(e[1:4], e[4])
        elif e[0] == "pool":
            sim.add_pool(e[1])
        else:
            boxes.append(e)
    for e in spec["solid"]:
        if e[0] == "room":
            sim.add_room()
        elif e[0] == "sphere":
            sim.add_sphere(e[1:4], e[4], liquid=False)
        else:
            boxes.append(e)
    sim.init_scene()
    return sim, boxes


def test_emitters_and_cell_solid_phi(ref):
    el = conftest.load_package()
    spec = el.scenes.water_drop(24)
    sim, _ = _ref_scene(ref, spec)
    phi, solid = ref.rasterise(spec, np.float32)
    np.testing.assert_array_equal(sim.field("phi"), phi)
    np.testing.assert_array_equal(sim.field("solid_nodal"), solid)
    np.testing.assert_array_equal(sim.field("solid_cell"), ref.cell_solid_phi(solid))
    sim.call("find_valid_level_set")
    np.testing.assert_array_equal(sim.field("phi_valid"), (ref.cell_solid_phi(solid) >= 0).astype(np.uint8))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_face_weights(ref, seed):
    rng = np.random.default_rng(seed)
    ni, nj, nk = 17, 13, 11
    solid = rng.uniform(-1, 1, (nk + 1, nj + 1, ni + 1)).astype(np.float32)
    solid[rng.uniform(size=solid.shape) < 0.1] = 0.0          # the sign test's edge case
    solid[rng.uniform(size=solid.shape) < 0.05] = -0.01       # the room's second layer value
    got = ref.compute_weights(solid)
    want = ref.ref_compute_weights(solid)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, w)


@pytest.mark.parametrize("scene", range(4))
def test_assign_indices_and_build_matrix(ref, scene):
    spec = _scenes()[scene]
    ni, nj, nk = spec["shape"]
    phi, solid = ref.rasterise(spec, np.float32)
    wu, wv, ww = ref.ref_compute_weights(solid)
    u, v, w = _random_velocity(ref, ni, nj, nk, 10 + scene)
    n, idx = ref.assign_indices(phi, wu, wv, ww)
    n_ref, idx_ref = ref.ref_assign_indices(phi, wu, wv, ww)
    assert n == n_ref > 0
    np.testing.assert_array_equal(idx, idx_ref)
    dx = ref.float_dx(ni, np.float32)
    dt = 0.37 * dx
    got = ref.build_matrix(phi, u, v, w, wu, wv, ww, dx, dt)
    D, X, Y, Z, B, odd, nnz = ref.ref_build_matrix(phi, u, v, w, wu, wv, ww, dx, dt)
    assert odd == 0
    for g, r in zip(got, (D, X, Y, Z, B)):
        np.testing.assert_array_equal(g, r)
    # every stored entry is a diagonal or a coupling of two liquid cells (counted both ways)
    assert nnz == int((D > 0).sum()) + 2 * int(sum(int((a != 0).sum()) for a in (X, Y, Z))) \
        + _explicit_zero_couplings(idx, wu, wv, ww)


def _explicit_zero_couplings(idx, wu, wv, ww):
    """Couplings the reference stores with value -0.0 (a zero-weight face between two liquid,
    pressure-valid cells), counted both ways."""
    live = idx != np.iinfo(np.int32).max
    n = 0
    n += int((live[:, :, 1:] & live[:, :, :-1] & (wu[:, :, 1:-1] == 0)).sum())
    n += int((live[:, 1:, :] & live[:, :-1, :] & (wv[:, 1:-1, :] == 0)).sum())
    n += int((live[1:, :, :] & live[:-1, :, :] & (ww[1:-1, :, :] == 0)).sum())
    return 2 * n


def test_no_fluid(ref):
    phi = np.ones((6, 6, 6), np.float32)
    w = [np.ones(ref.face_shape(6, 6, 6, c), np.float32) for c in range(3)]
    assert ref.ref_assign_indices(phi, *w)[0] == -1
    assert ref.assign_indices(phi, *w)[0] == 0


def test_build_grid_from_vector(ref):
    spec = _scenes()[0]
    phi, solid = ref.rasterise(spec, np.float32)
    n, idx = ref.assign_indices(phi, *ref.compute_weights(solid))
    vec = np.random.default_rng(4).standard_normal(n)
    got = ref.ref_build_grid_from_vector(vec, idx, 0.0)
    live = idx != np.iinfo(np.int32).max
    want = np.zeros(idx.shape, np.float32)
    want[live] = vec[idx[live]].astype(np.float32)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("scene", range(4))
def test_update_velocity(ref, scene):
    spec = _scenes()[scene]
    ni, nj, nk = spec["shape"]
    phi, _ = ref.rasterise(spec, np.float32)
    u, v, w = _random_velocity(ref, ni, nj, nk, 20 + scene)
    p = np.random.default_rng(30 + scene).standard_normal(phi.shape).astype(np.float32)
    dx = ref.float_dx(ni, np.float32)
    dt = 0.41 * dx
    got = ref.update_velocity(u, v, w, p, phi, dx, dt)
    want = ref.ref_update_velocity(u, v, w, p, phi, dx, dt)
    for g, r in zip(got, want):
        np.testing.assert_array_equal(g, r)


@pytest.mark.parametrize("density", [0.0, 0.02, 0.3, 0.9, 1.0])
@pytest.mark.parametrize("keep_valid", [False, True])
def test_extrapolate(ref, density, keep_valid):
    rng = np.random.default_rng(int(density * 100) + keep_valid)
    shape = (9, 14, 19)
    grid = rng.standard_normal(shape).astype(np.float32)
    valid = (rng.uniform(size=shape) < density).astype(np.uint8)
    for layers in (1, 3, 10):
        g, m = ref.extrapolate(grid, valid, layers)
        gr, mr = ref.ref_extrapolate(grid, valid, layers, keep_valid)
        np.testing.assert_array_equal(g, gr)
        if keep_valid:
            np.testing.assert_array_equal(mr, valid)
        else:
            np.testing.assert_array_equal(m, mr)


@pytest.mark.parametrize("scene", range(4))
def test_masks_gravity_and_time_step(ref, scene):
    """find_valid_velocity, set_invalid_velocity_zero, add_gravity (simulator.cpp:90-178) and
    calc_time_step (time_stepping.cpp:5-7) run on the reference's Simulator."""
    spec = _scenes()[scene]
    ni, nj, nk = spec["shape"]
    sim, boxes = _ref_scene(ref, spec)
    phi, solid = ref.rasterise(spec, np.float32)
    sim.field("solid_nodal")[...] = solid       # boxes included
    sim.field("phi")[...] = phi
    sim.call("compute_weights")
    wts = ref.compute_weights(solid)
    for f, wt in zip(("weight_u", "weight_v", "weight_w"), wts):
        np.testing.assert_array_equal(sim.field(f), wt)
    vel = _random_velocity(ref, ni, nj, nk, 40 + scene)
    for f, a in zip("uvw", vel):
        sim.field(f)[...] = a
    dx = sim.dx
    assert ref.ref_calc_time_step(*vel, dx, 1.0) == ref.calc_time_step(*vel, dx, 1.0)
    dt = 0.013
    sim.call("add_gravity", dt)
    t = np.float32
    v_g = (vel[1] - t(t(9.80665) * t(dt))).astype(np.float32)
    np.testing.assert_array_equal(sim.field("v"), v_g)
    sim.call("find_valid_velocity")
    vu, vv, vw = ref.find_valid_velocity(phi, *wts)
    for f, m in zip(("valid_u", "valid_v", "valid_w"), (vu, vv, vw)):
        np.testing.assert_array_equal(sim.field(f), m)
    sim.call("set_invalid_velocity_zero")
    for f, a, m in zip("uvw", (vel[0], v_g, vel[2]), (vu, vv, vw)):
        np.testing.assert_array_equal(sim.field(f), np.where(m == 0, t(0), a))
    sim.close()


def test_advection_drivers(ref):
    """advect_collocated_grid / advect_staggered_grid loop drivers (advection.cpp:9-27)."""
    helpers = pytest.importorskip("helpers")
    dx, phi, u, v, w = helpers.smooth_fields(ref, 20, 16, 12, np.float32, seed=5)
    dt = 0.9 * dx
    np.testing.assert_array_equal(ref.ref_advect_collocated(phi, u, v, w, dx, dt),
                                  ref.advect_collocated(phi, u, v, w, dx, dt))
    for g, r in zip(ref.advect_staggered(u, v, w, dx, dt), ref.ref_advect_staggered(u, v, w, dx, dt)):
        np.testing.assert_array_equal(g, r)


def test_step_pieces_match_reference_simulator(ref):
    """One sub-step of update_second_order without reinitialize() on the reference's Simulator,
    piece by piece against oracle/step.py's pieces: bit-exact up to the solve; the pressure solves
    the same (bit-identical) system to the reference's tolerance."""
    el = conftest.load_package()
    spec = el.scenes.water_drop(24)
    ni, nj, nk = spec["shape"]
    sim, _ = _ref_scene(ref, spec)
    sim.call("compute_weights")
    sim.call("find_valid_level_set")
    vel = _random_velocity(ref, ni, nj, nk, 77, scale=0.3)
    for f, a in zip("uvw", vel):
        sim.field(f)[...] = a
    phi0 = sim.field("phi").copy()
    wts = tuple(sim.field(f).copy() for f in ("weight_u", "weight_v", "weight_w"))
    valid_phi = sim.field("phi_valid").copy()
    dx = sim.dx
    dt = ref.calc_time_step(*vel, dx, 1.0)

    sim.call("extrapolate_velocity")
    sim.call("extrapolate_level_set")
    ex = [ref.extrapolate(a, np.ones(a.shape, np.uint8), 10) for a in vel]   # valid starts at 1
    for f, (a, m) in zip("uvw", ex):
        np.testing.assert_array_equal(sim.field(f), a)
    phi_x, _ = ref.extrapolate(phi0, valid_phi, 10)
    np.testing.assert_array_equal(sim.field("phi"), phi_x)
    sim.call("advect_level_set", dt)
    sim.call("advect_velocity", dt)
    ue, ve, we = (a for a, _ in ex)
    phi1 = ref.advect_collocated(phi_x, ue, ve, we, dx, dt)
    np.testing.assert_array_equal(sim.field("phi"), phi1)
    u1, v1, w1 = ref.advect_staggered(ue, ve, we, dx, dt)
    for f, a in zip("uvw", (u1, v1, w1)):
        np.testing.assert_array_equal(sim.field(f), a)
    sim.call("add_gravity", dt)
    sim.call("find_valid_velocity")
    sim.call("set_invalid_velocity_zero")
    t = np.float32
    v1 = (v1 - t(t(9.80665) * t(dt))).astype(np.float32)
    vu, vv, vw = ref.find_valid_velocity(phi1, *wts)
    u1, v1, w1 = (np.where(m == 0, t(0), a) for a, m in zip((u1, v1, w1), (vu, vv, vw)))
    for f, a in zip("uvw", (u1, v1, w1)):
        np.testing.assert_array_equal(sim.field(f), a)
    mats = ref.build_matrix(phi1, u1, v1, w1, *wts, dx, dt)
    sim.call("solve_pressure", dt)
    p_ref = sim.field("pressure").copy()
    helpers = pytest.importorskip("helpers")
    # the reference's solve stops at relative residual 1e-4 (simulator.cpp:102-107)
    assert helpers.residual_rel(ref, mats, p_ref) < 2e-4
    x, st, _, _ = ref.pcg(*mats, precond=ref.PRE_MIC0, tol=1e-12)
    assert st == 0
    assert conftest.rel_err(p_ref, np.where(mats[0] > 0, x, 0)) < 5e-3
    # the velocity update of the reference's own pressure, restated
    uu, vv2, ww2 = ref.update_velocity(u1, v1, w1, p_ref, phi1, dx, dt)
    for f, a in zip("uvw", (uu, vv2, ww2)):
        np.testing.assert_array_equal(sim.field(f), a)
    sim.close()


def _read_obj(path):
    verts, faces = [], []
    with open(path) as fh:
        for line in fh:
            if line.startswith("v "):
                verts.append([float(t) for t in line.split()[1:4]])
            elif line.startswith("f "):
                faces.append([int(t) - 1 for t in line.split()[1:]])
    return np.array(verts), faces


@pytest.mark.parametrize("method", [0, 1])
def test_marching_cubes_obj_of_a_sphere_scene(ref, tmp_path, method):
    """Headless OBJ output through the reference's own get_mesh + Mesh::save (meshing.cpp:20-127,
    mesh.cpp:53) on a 32^3 sphere level set: a closed surface of genus 0 at the sphere's radius."""
    el = conftest.load_package()
    spec = {"name": "sphere", "shape": (32, 32, 32), "liquid": [("sphere", 0.5, 0.5, 0.5, 0.3)],
            "solid": [("room",)]}
    phi, _ = ref.rasterise(spec, np.float32)
    dx = ref.float_dx(32, np.float32)
    path = str(tmp_path / f"sphere_{method}.obj")
    nv, nf, per = ref.ref_mesh_obj(phi, dx, method=method, path=path)
    verts, faces = _read_obj(path)
    assert per == (3 if method == 0 else 4)
    assert len(verts) == nv > 100 and len(faces) == nf > 100
    assert all(len(f) == per for f in faces)
    # marching cubes shares vertices only within a cell (meshing.cpp:29 keeps a per-cell map), so
    # weld equal positions before counting; dual marching cubes shares them already
    _, weld = np.unique(verts, axis=0, return_inverse=True)
    weld = weld.reshape(-1)
    edges = set()
    for f in faces:
        for a in range(per):
            e = (weld[f[a]], weld[f[(a + 1) % per]])
            edges.add((min(e), max(e)))
    assert int(weld.max()) + 1 - len(edges) + nf == 2          # Euler characteristic of a sphere
    # dual marching cubes places vertices at index coordinates * dx + origin (meshing.cpp:119-121),
    # half a cell from the cell-centre positions marching cubes interpolates between
    centre = 0.5 - (0.5 * dx if method == 1 else 0.0)
    r = np.linalg.norm(verts - centre, axis=1)
    assert np.all(np.abs(r - 0.3) < 0.5 * dx)
    del el
