"""Generate the golden fixtures in tests/golden/ by running the reference's own code.

The reference's Eigen-free header templates (include/nama/math/interpolation.h,
include/nama/math/ode.h) are compiled from the reference tree by oracle/build.py into
oracle/_ref/libnama_ref.so; this script feeds them seeded inputs and stores inputs and outputs.
Run here, where the reference tree exists:

    python oracle/build.py --ref <reference checkout>
    python tests/golden/make_golden.py

Fixtures: advect_<dtype>.npz -- semi-Lagrangian advection (RK2 backtrace, trilinear and WENO6
sampling, cell-centred and staggered) of seeded fields on a 12 x 10 x 8 grid, and
interp_<dtype>.npz -- point samples, RK2 traces and 1-D WENO6 evaluations.

step_ref_f32.npz -- one sub-step of update_second_order without reinitialize() run piece by
piece on the reference's own Simulator (simulator.cpp, projection.cpp, boundary.cpp,
extrapolation.cpp, advection.cpp, levelset_emitter.cpp, compiled by oracle/build.py against
oracle/eigen_min) on a 20 x 16 x 18 scene: spheres and a pool in a room with a solid box
obstacle, seeded velocity.  Every intermediate field is stored, the matrix in grid form, and
the velocity update of a seeded pressure.
"""

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402


def main():
    R = O.ref_lib()
    if R is None:
        raise SystemExit("oracle/_ref/libnama_ref.so is missing: build it with oracle/build.py --ref <reference>")
    ni, nj, nk = 12, 10, 8
    for dtype, suf in ((np.float32, "f32"), (np.float64, "f64")):
        rng = np.random.default_rng(20261203)
        dx = O.float_dx(ni, dtype)
        xs = (np.arange(ni) + 0.5) / ni
        ys = (np.arange(nj) + 0.5) / ni
        zs = (np.arange(nk) + 0.5) / ni
        Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
        phi = (np.sqrt((X - 0.5) ** 2 + (Y - 0.4) ** 2 + (Z - 0.3) ** 2) - 0.25).astype(dtype)
        phi += (1e-3 * rng.standard_normal(phi.shape)).astype(dtype)
        u = (0.6 * rng.uniform(-1, 1, O.face_shape(ni, nj, nk, 0))).astype(dtype)
        v = (0.6 * rng.uniform(-1, 1, O.face_shape(ni, nj, nk, 1))).astype(dtype)
        w = (0.6 * rng.uniform(-1, 1, O.face_shape(ni, nj, nk, 2))).astype(dtype)
        dt = float(dtype(0.8) * dtype(dx))
        out = {"phi": phi, "u": u, "v": v, "w": w, "dx": np.float64(dx), "dt": np.float64(dt)}
        for weno in (0, 1):
            o = np.empty_like(phi)
            getattr(R, f"ref_advect_collocated_{suf}")(ni, nj, nk, C.c_double(dx), O._p(o), O._p(phi), O._p(u),
                                                       O._p(v), O._p(w), C.c_double(dt), weno)
            out[f"phi_out_{'weno6' if weno else 'trilinear'}"] = o
            ou, ov, ow = np.empty_like(u), np.empty_like(v), np.empty_like(w)
            getattr(R, f"ref_advect_staggered_{suf}")(ni, nj, nk, C.c_double(dx), O._p(ou), O._p(ov), O._p(ow),
                                                      O._p(u), O._p(v), O._p(w), C.c_double(dt), weno)
            tag = "weno6" if weno else "trilinear"
            out[f"u_out_{tag}"], out[f"v_out_{tag}"], out[f"w_out_{tag}"] = ou, ov, ow
        np.savez_compressed(os.path.join(HERE, f"advect_{suf}.npz"), **out)

        # point samples of phi at seeded positions (inside and outside the grid: clamping)
        pts = rng.uniform(-0.2, 1.2, (64, 3))
        tri, weno, traces = [], [], []
        for p in pts:
            tri.append(getattr(R, f"ref_sample_{suf}")(O._p(phi), ni, nj, nk, C.c_double(0), C.c_double(0), C.c_double(0), C.c_double(dx),
                                                       *map(C.c_double, p), 0))
            weno.append(getattr(R, f"ref_sample_{suf}")(O._p(phi), ni, nj, nk, C.c_double(0), C.c_double(0), C.c_double(0), C.c_double(dx),
                                                        *map(C.c_double, p), 1))
            t = np.empty(3, dtype)
            getattr(R, f"ref_trace_rk2_{suf}")(ni, nj, nk, C.c_double(dx), O._p(u), O._p(v), O._p(w),
                                               *map(C.c_double, p), C.c_double(-dt), O._p(t))
            traces.append(t)
        vals = rng.standard_normal((64, 6)).astype(dtype)
        fr = rng.uniform(0, 1, 64)
        w1 = []
        for row, f in zip(vals, fr):
            row = np.ascontiguousarray(row)
            w1.append(getattr(R, f"ref_weno6_1d_{suf}")(O._p(row), C.c_double(f)))
        np.savez_compressed(os.path.join(HERE, f"interp_{suf}.npz"), phi=phi, u=u, v=v, w=w, dx=np.float64(dx),
                            dt=np.float64(dt), points=pts, trilinear=np.array(tri, dtype),
                            weno6=np.array(weno, dtype), traces=np.array(traces), weno1d_values=vals,
                            weno1d_fractions=fr, weno1d=np.array(w1, dtype))
    step_fixture()
    print("wrote fixtures to", HERE)


def step_fixture():
    if not O.ref_sim_available():
        raise SystemExit("oracle/_ref/libnama_ref.so lacks the simulator sources: rebuild with oracle/build.py")
    ni, nj, nk = 20, 16, 18
    sim = O.RefSimulator(ni, nj, nk)
    sim.add_sphere((0.3, 0.55, 0.35), 0.16)
    sim.add_sphere((0.7, 0.6, 0.6), 0.12)
    sim.add_pool(0.22)
    sim.add_room()
    sim.init_scene()
    dx = sim.dx
    solid = sim.field("solid_nodal")
    # a solid box obstacle (not one of the reference's emitters), composed with min
    O.emit_box(solid, (-0.5 * dx,) * 3, dx, (0.45, 0.05, 0.3), (0.62, 0.3, 0.55))
    sim.call("calc_cell_centered_solid_phi")
    sim.call("compute_weights")
    sim.call("find_valid_level_set")
    rng = np.random.default_rng(20261204)
    out = {"shape": np.array([ni, nj, nk]), "dx": np.float64(dx)}
    for f in ("u", "v", "w"):
        sim.field(f)[...] = (0.4 * rng.standard_normal(sim.field(f).shape)).astype(np.float32)
    for f in ("phi", "solid_nodal", "solid_cell", "phi_valid", "u", "v", "w", "weight_u", "weight_v", "weight_w"):
        out[f"in_{f}"] = sim.field(f).copy()
    dt = O.ref_calc_time_step(sim.field("u"), sim.field("v"), sim.field("w"), dx, 1.0)
    out["dt"] = np.float64(dt)

    def record(tag, fields):
        for f in fields:
            out[f"{tag}_{f}"] = sim.field(f).copy()

    sim.call("extrapolate_velocity")
    record("extrap", ("u", "v", "w", "valid_u", "valid_v", "valid_w"))
    sim.call("extrapolate_level_set")
    record("extrap", ("phi",))
    sim.call("advect_level_set", dt)
    sim.call("advect_velocity", dt)
    record("advect", ("phi", "u", "v", "w"))
    sim.call("add_gravity", dt)
    record("gravity", ("v",))
    sim.call("find_valid_velocity")
    sim.call("set_invalid_velocity_zero")
    record("masks", ("u", "v", "w", "valid_u", "valid_v", "valid_w"))
    args = [sim.field(f) for f in ("phi", "u", "v", "w", "weight_u", "weight_v", "weight_w")]
    n, idx = O.ref_assign_indices(args[0], *args[4:])
    D, X, Y, Z, B, odd, _ = O.ref_build_matrix(*args, dx, dt)
    assert odd == 0
    out.update(indices=idx, mat_size=np.int64(n), diag=D, offx=X, offy=Y, offz=Z, rhs=B)
    p = np.where(D > 0, rng.standard_normal(D.shape), 0).astype(np.float32)
    uu, vv, ww = O.ref_update_velocity(args[1], args[2], args[3], p, args[0], dx, dt)
    out.update(update_pressure=p, update_u=uu, update_v=vv, update_w=ww)
    sim.close()
    np.savez_compressed(os.path.join(HERE, "step_ref_f32.npz"), **out)


if __name__ == "__main__":
    main()
