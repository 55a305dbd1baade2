"""The oracle's composition of one step (TEST INFRASTRUCTURE / CPU BASELINE ONLY).

update_second_order (apps/eulerian_liquid_3d.cpp:106-120) without reinitialize(), which stays
the reference's own code outside the hot path: extrapolate velocity and level set
(simulator.cpp:115-123), advect the level set then the velocity (simulator.cpp:79-87), add
gravity (:90-93), find the valid faces and zero the others (:125-178), solve the pressure
(:96-112) and update the velocity (projection.cpp:93-134).
"""

import numpy as np

from . import (PRE_MIC0, advect_collocated, advect_staggered, build_matrix, extrapolate, find_valid_velocity,
               pcg, update_velocity)


def initial_state(phi, weights, cell_solid, dx):
    """State after create_grid/init_scene/compute_weights/find_valid_level_set (velocity 0)."""
    dtype = phi.dtype
    wu, wv, ww = weights
    return {"phi": phi, "weights": weights, "dx": dx,
            "u": np.zeros(wu.shape, dtype), "v": np.zeros(wv.shape, dtype), "w": np.zeros(ww.shape, dtype),
            "valid_u": np.ones(wu.shape, np.uint8), "valid_v": np.ones(wv.shape, np.uint8),
            "valid_w": np.ones(ww.shape, np.uint8), "valid_phi": (cell_solid >= 0).astype(np.uint8)}


def step(state, dt, trace_phi, sample_phi, trace_vel, sample_vel, gravity, layers=10, precond=PRE_MIC0,
         tol=1e-13, maxit=20000):
    s = dict(state)
    dtype = s["phi"].dtype
    dx = s["dx"]
    for f in ("u", "v", "w"):
        s[f], s["valid_" + f] = extrapolate(s[f], s["valid_" + f], layers)
    s["phi"], _ = extrapolate(s["phi"], s["valid_phi"], layers)
    phi_new = advect_collocated(s["phi"], s["u"], s["v"], s["w"], dx, dt, trace_phi, sample_phi)
    u, v, w = advect_staggered(s["u"], s["v"], s["w"], dx, dt, trace_vel, sample_vel)
    t = dtype.type
    v = (v - t(t(gravity) * t(dt))).astype(dtype)
    wu, wv, ww = s["weights"]
    vu, vv, vw = find_valid_velocity(phi_new, wu, wv, ww)
    u = np.where(vu == 0, t(0), u).astype(dtype)
    v = np.where(vv == 0, t(0), v).astype(dtype)
    w = np.where(vw == 0, t(0), w).astype(dtype)
    pre_projection = (u, v, w)
    D, X, Y, Z, B = build_matrix(phi_new, u, v, w, wu, wv, ww, dx, dt)
    x, st, it, rr = pcg(D, X, Y, Z, B, precond=precond, tol=tol, maxit=maxit)
    p = np.where(D > 0, x, 0.0).astype(dtype)
    u, v, w = update_velocity(u, v, w, p, phi_new, dx, dt)
    s.update(phi=phi_new, u=u, v=v, w=w, valid_u=vu, valid_v=vv, valid_w=vw, pressure=p, pcg_iterations=it,
             pcg_status=st, pcg_relres=rr, pre_projection=pre_projection)
    return s, (D, X, Y, Z, B)
