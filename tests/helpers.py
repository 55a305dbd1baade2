"""Seeded inputs and the oracle's composition of a step, shared by the GPU parity tests."""

import numpy as np

import conftest

RTOL_F64 = 1e-12   # advected fields vs the FP64 restatement (norm-wise relative)
RTOL_F32 = 2e-5    # FP32 path vs the reference's float instantiation (norm-wise relative)
# WENO6 in FP32: the smoothness indicators are quadratic forms with coefficients up to ~7e3 that
# cancel to ~0 on smooth data, so in float they carry rounding noise far above eps = 1e-6 and
# the nonlinear weights differ between any two float evaluation orders (the reference's float
# instantiation included).  The candidates agree to O(dx^4), which bounds the difference.
RTOL_F32_WENO = 2e-4


def smooth_fields(orc, ni, nj, nk, dtype, seed, speed=0.8):
    """A signed-distance-like level set and a smooth divergent velocity with seeded noise."""
    rng = np.random.default_rng(seed)
    dx = orc.float_dx(ni, dtype)
    zs, ys, xs = np.meshgrid((np.arange(nk) + 0.5) * dx, (np.arange(nj) + 0.5) * dx, (np.arange(ni) + 0.5) * dx,
                             indexing="ij")
    phi = np.sqrt((xs - 0.45) ** 2 + (ys - 0.4 * nj / ni) ** 2 + (zs - 0.5 * nk / ni) ** 2) - 0.2
    phi = (phi + 1e-3 * rng.standard_normal(phi.shape)).astype(dtype)

    def comp(shape, phase):
        k, j, i = np.meshgrid(*(np.arange(s) for s in shape), indexing="ij")
        base = np.sin(0.31 * i + phase) * np.cos(0.23 * j - phase) + 0.5 * np.sin(0.17 * k + 2 * phase)
        return (speed * base + 0.05 * rng.standard_normal(shape)).astype(dtype)

    u = comp(orc.face_shape(ni, nj, nk, 0), 0.1)
    v = comp(orc.face_shape(ni, nj, nk, 1), 0.7)
    w = comp(orc.face_shape(ni, nj, nk, 2), 1.3)
    return dx, phi, u, v, w


def scene_fields(orc, spec, dtype):
    phi, solid = orc.rasterise(spec, dtype)
    wu, wv, ww = orc.compute_weights(solid)
    return phi, solid, (wu, wv, ww)


def oracle_step(orc, state, dt, trace_phi, sample_phi, trace_vel, sample_vel, gravity, layers=10,
                precond=None, tol=1e-13):
    """One step on the oracle (oracle/step.py)."""
    from oracle import step as ostep
    return ostep.step(state, dt, trace_phi, sample_phi, trace_vel, sample_vel, gravity, layers,
                      orc.PRE_MIC0 if precond is None else precond, tol)


def residual_rel(orc, mats, p):
    D, X, Y, Z, B = mats
    r = B - orc.spmv(D, X, Y, Z, np.where(D > 0, p.astype(np.float64), 0.0))
    return float(np.linalg.norm(r) / np.linalg.norm(B))


def make_sim(el, n_or_shape, dtype, spec=None):
    ni, nj, nk = (n_or_shape,) * 3 if isinstance(n_or_shape, int) else n_or_shape
    sim = el.Simulator(ni, nj, nk, dtype=el.EL_F64 if dtype == np.float64 else el.EL_F32)
    if spec is not None:
        sim.init_scene(spec)
    return sim


def package():
    return conftest.load_package()
