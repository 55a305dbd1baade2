"""CPU oracle for the per-step grid hot path (TEST INFRASTRUCTURE ONLY).

ctypes/numpy wrapper around ``oracle/_build/liboracle.so`` (the C++ restatement in
``oracle/oracle.cpp``) and, when built, ``oracle/_ref/libnama_ref.so`` (the reference's own
interpolation/ode templates).  Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU
baseline leg may import this package; the product never does.

Array conventions follow the reference (include/nama/common/array.h:281-286): numpy arrays
of shape (nk, nj, ni) in C order, so that flat index = i + ni*(j + nj*k).
"""

import ctypes as C
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))

TRACE_RK2, TRACE_RK3 = 0, 1
SAMPLE_TRILINEAR, SAMPLE_WENO6 = 0, 1
PRE_NONE, PRE_JACOBI, PRE_IC0, PRE_MIC0 = 0, 1, 2, 3
DEFAULT_GRAVITY = 9.80665  # include/nama/constants.h:6

_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(_build.build_oracle())
        _declare(_lib)
    return _lib


def ref_lib():
    """The reference's own templates compiled from its tree, or None when unavailable."""
    global _ref
    if _ref is None:
        path = os.path.join(HERE, "_ref", "libnama_ref.so")
        if not os.path.exists(path):
            return None
        _ref = C.CDLL(path)
        for suf, ct in (("f32", C.c_float), ("f64", C.c_double)):
            getattr(_ref, f"ref_weno6_1d_{suf}").restype = ct
            getattr(_ref, f"ref_sample_{suf}").restype = ct
    return _ref


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _suffix(dtype):
    dtype = np.dtype(dtype)
    if dtype == np.float32:
        return "f32", C.c_float
    if dtype == np.float64:
        return "f64", C.c_double
    raise TypeError(f"unsupported dtype {dtype}")


def _declare(L):
    vp, i, d, ll = C.c_void_p, C.c_int, C.c_double, C.c_longlong
    for suf, ct in (("f32", C.c_float), ("f64", C.c_double)):
        getattr(L, f"or_advect_collocated_{suf}").argtypes = [i, i, i, d, vp, vp, vp, vp, vp, d, i, i]
        getattr(L, f"or_advect_staggered_{suf}").argtypes = [i, i, i, d, vp, vp, vp, vp, vp, vp, d, i, i]
        f = getattr(L, f"or_sample_trilinear_{suf}")
        f.argtypes = [vp, i, i, i, d, d, d, d, d, d, d]
        f.restype = ct
        f = getattr(L, f"or_sample_weno6_{suf}")
        f.argtypes = [vp, i, i, i, d, d, d, d, d, d, d]
        f.restype = ct
        getattr(L, f"or_index_fraction_{suf}").argtypes = [d, d, d, vp, vp]
        getattr(L, f"or_trace_{suf}").argtypes = [i, i, i, d, vp, vp, vp, d, d, d, d, i, vp]
        f = getattr(L, f"or_fraction_inside_{suf}")
        f.argtypes = [ct, ct]
        f.restype = ct
        f = getattr(L, f"or_fraction_inside4_{suf}")
        f.argtypes = [ct, ct, ct, ct]
        f.restype = ct
        getattr(L, f"or_compute_weights_{suf}").argtypes = [i, i, i, vp, vp, vp, vp]
        f = getattr(L, f"or_assign_indices_{suf}")
        f.argtypes = [i, i, i, vp, vp, vp, vp, vp]
        f.restype = i
        getattr(L, f"or_build_matrix_{suf}").argtypes = [i, i, i, d] + [vp] * 7 + [d] + [vp] * 5
        getattr(L, f"or_update_velocity_{suf}").argtypes = [i, i, i, d, vp, vp, vp, vp, vp, d]
        getattr(L, f"or_extrapolate_{suf}").argtypes = [vp, vp, i, i, i, i]
        getattr(L, f"or_find_valid_velocity_{suf}").argtypes = [i, i, i] + [vp] * 7
        getattr(L, f"or_cell_solid_phi_{suf}").argtypes = [i, i, i, vp, vp]
        f = getattr(L, f"or_max_abs_{suf}")
        f.argtypes = [vp, ll]
        f.restype = ct
        getattr(L, f"or_emit_sphere_{suf}").argtypes = [vp, i, i, i, d, d, d, d, d, d, d, d]
        getattr(L, f"or_emit_pool_{suf}").argtypes = [vp, i, i, i, d, d, d, d, d]
        getattr(L, f"or_emit_box_{suf}").argtypes = [vp, i, i, i, d, d, d, d, vp, vp]
        getattr(L, f"or_emit_room_{suf}").argtypes = [vp, i, i, i]
    L.or_pcg.argtypes = [i, i, i] + [vp] * 6 + [i, d, i, vp, vp]
    L.or_pcg.restype = i
    L.or_spmv.argtypes = [i, i, i] + [vp] * 6


def _c(a, dtype=None):
    a = np.ascontiguousarray(a, dtype=dtype)
    return a


# ----------------------------------------------------------------------------------------
# Grid helpers

def face_shape(ni, nj, nk, comp):
    """numpy shape (nk, nj, ni)-ordered of component comp (0=u, 1=v, 2=w)."""
    return [(nk, nj, ni + 1), (nk, nj + 1, ni), (nk + 1, nj, ni)][comp]


def float_dx(ni, dtype):
    """dx = width / ni with width 1, evaluated in the field type (simulator.cpp:56)."""
    if np.dtype(dtype) == np.float32:
        return float(np.float32(1.0) / np.float32(ni))
    return 1.0 / ni


# ----------------------------------------------------------------------------------------
# Advection

def advect_collocated(phi, u, v, w, dx, dt, trace=TRACE_RK2, sample=SAMPLE_TRILINEAR):
    suf, _ = _suffix(phi.dtype)
    nk, nj, ni = phi.shape
    phi, u, v, w = (_c(a) for a in (phi, u, v, w))
    out = np.empty_like(phi)
    getattr(lib(), f"or_advect_collocated_{suf}")(ni, nj, nk, dx, _p(out), _p(phi), _p(u), _p(v), _p(w),
                                                  dt, trace, sample)
    return out


def advect_staggered(u, v, w, dx, dt, trace=TRACE_RK2, sample=SAMPLE_TRILINEAR):
    suf, _ = _suffix(u.dtype)
    nk, nj, ni1 = u.shape
    ni = ni1 - 1
    u, v, w = (_c(a) for a in (u, v, w))
    ou, ov, ow = np.empty_like(u), np.empty_like(v), np.empty_like(w)
    getattr(lib(), f"or_advect_staggered_{suf}")(ni, nj, nk, dx, _p(ou), _p(ov), _p(ow), _p(u), _p(v), _p(w),
                                                 dt, trace, sample)
    return ou, ov, ow


def sample_trilinear(grid, origin, dx, x):
    suf, _ = _suffix(grid.dtype)
    n2, n1, n0 = grid.shape
    grid = _c(grid)
    return getattr(lib(), f"or_sample_trilinear_{suf}")(_p(grid), n0, n1, n2, *origin, dx, *x)


def sample_weno6(grid, origin, dx, x):
    suf, _ = _suffix(grid.dtype)
    n2, n1, n0 = grid.shape
    grid = _c(grid)
    return getattr(lib(), f"or_sample_weno6_{suf}")(_p(grid), n0, n1, n2, *origin, dx, *x)


def index_fraction(pos, origin, dx, dtype=np.float32):
    suf, ct = _suffix(dtype)
    idx = C.c_int()
    frac = ct()
    getattr(lib(), f"or_index_fraction_{suf}")(pos, origin, dx, C.byref(idx), C.byref(frac))
    return idx.value, frac.value


def trace(u, v, w, dx, x, dt, scheme=TRACE_RK2):
    suf, _ = _suffix(u.dtype)
    nk, nj, ni1 = u.shape
    out = np.empty(3, dtype=u.dtype)
    u, v, w = (_c(a) for a in (u, v, w))
    getattr(lib(), f"or_trace_{suf}")(ni1 - 1, nj, nk, dx, _p(u), _p(v), _p(w), *x, dt, scheme, _p(out))
    return out


def fraction_inside(a, b, dtype=np.float32):
    suf, _ = _suffix(dtype)
    return getattr(lib(), f"or_fraction_inside_{suf}")(a, b)


def fraction_inside4(bl, br, tl, tr, dtype=np.float32):
    suf, _ = _suffix(dtype)
    return getattr(lib(), f"or_fraction_inside4_{suf}")(bl, br, tl, tr)


# ----------------------------------------------------------------------------------------
# Boundary weights, projection

def compute_weights(solid_nodal):
    suf, _ = _suffix(solid_nodal.dtype)
    nk1, nj1, ni1 = solid_nodal.shape
    ni, nj, nk = ni1 - 1, nj1 - 1, nk1 - 1
    s = _c(solid_nodal)
    wu = np.empty(face_shape(ni, nj, nk, 0), s.dtype)
    wv = np.empty(face_shape(ni, nj, nk, 1), s.dtype)
    ww = np.empty(face_shape(ni, nj, nk, 2), s.dtype)
    getattr(lib(), f"or_compute_weights_{suf}")(ni, nj, nk, _p(s), _p(wu), _p(wv), _p(ww))
    return wu, wv, ww


def assign_indices(phi, wu, wv, ww):
    suf, _ = _suffix(phi.dtype)
    nk, nj, ni = phi.shape
    phi, wu, wv, ww = (_c(a) for a in (phi, wu, wv, ww))
    idx = np.empty(phi.shape, np.int32)
    n = getattr(lib(), f"or_assign_indices_{suf}")(ni, nj, nk, _p(phi), _p(wu), _p(wv), _p(ww), _p(idx))
    return n, idx


def build_matrix(phi, u, v, w, wu, wv, ww, dx, dt):
    """Grid-shaped ghost-fluid matrix: (diag, offx, offy, offz, rhs), all float64 (nk,nj,ni)."""
    suf, _ = _suffix(phi.dtype)
    nk, nj, ni = phi.shape
    arrs = [_c(a) for a in (phi, u, v, w, wu, wv, ww)]
    outs = [np.empty(phi.shape, np.float64) for _ in range(5)]
    getattr(lib(), f"or_build_matrix_{suf}")(ni, nj, nk, dx, *[_p(a) for a in arrs], dt, *[_p(o) for o in outs])
    return tuple(outs)


def pcg(diag, offx, offy, offz, rhs, precond=PRE_MIC0, tol=1e-6, maxit=1000):
    """Returns (x, status, iterations, relative residual); status 0 = converged."""
    n2, n1, n0 = diag.shape
    arrs = [_c(a, np.float64) for a in (diag, offx, offy, offz, rhs)]
    x = np.zeros(diag.shape, np.float64)
    it = C.c_int()
    rr = C.c_double()
    st = lib().or_pcg(n0, n1, n2, *[_p(a) for a in arrs], _p(x), precond, tol, maxit, C.byref(it), C.byref(rr))
    return x, st, it.value, rr.value


def spmv(diag, offx, offy, offz, p):
    n2, n1, n0 = diag.shape
    arrs = [_c(a, np.float64) for a in (diag, offx, offy, offz, p)]
    out = np.empty(diag.shape, np.float64)
    lib().or_spmv(n0, n1, n2, *[_p(a) for a in arrs], _p(out))
    return out


def update_velocity(u, v, w, pressure, phi, dx, dt):
    suf, _ = _suffix(phi.dtype)
    nk, nj, ni = phi.shape
    u, v, w = (np.array(a, copy=True, order="C") for a in (u, v, w))
    p, phi = _c(pressure, phi.dtype), _c(phi)
    getattr(lib(), f"or_update_velocity_{suf}")(ni, nj, nk, dx, _p(u), _p(v), _p(w), _p(p), _p(phi), dt)
    return u, v, w


# ----------------------------------------------------------------------------------------
# Extrapolation, masks, time step

def extrapolate(grid, valid, layers=10):
    """Returns (grid, valid) after up to `layers` Jacobi extrapolation layers."""
    suf, _ = _suffix(grid.dtype)
    n2, n1, n0 = grid.shape
    g = np.array(grid, copy=True, order="C")
    m = np.array(valid, dtype=np.uint8, copy=True, order="C")
    getattr(lib(), f"or_extrapolate_{suf}")(_p(g), _p(m), n0, n1, n2, layers)
    return g, m


def find_valid_velocity(phi, wu, wv, ww):
    suf, _ = _suffix(phi.dtype)
    nk, nj, ni = phi.shape
    phi, wu, wv, ww = (_c(a) for a in (phi, wu, wv, ww))
    vu = np.empty(wu.shape, np.uint8)
    vv = np.empty(wv.shape, np.uint8)
    vw = np.empty(ww.shape, np.uint8)
    getattr(lib(), f"or_find_valid_velocity_{suf}")(ni, nj, nk, _p(phi), _p(wu), _p(wv), _p(ww),
                                                    _p(vu), _p(vv), _p(vw))
    return vu, vv, vw


def cell_solid_phi(solid_nodal):
    suf, _ = _suffix(solid_nodal.dtype)
    nk1, nj1, ni1 = solid_nodal.shape
    s = _c(solid_nodal)
    out = np.empty((nk1 - 1, nj1 - 1, ni1 - 1), s.dtype)
    getattr(lib(), f"or_cell_solid_phi_{suf}")(ni1 - 1, nj1 - 1, nk1 - 1, _p(s), _p(out))
    return out


def max_abs(a):
    suf, _ = _suffix(a.dtype)
    a = _c(a)
    return getattr(lib(), f"or_max_abs_{suf}")(_p(a), a.size)


def calc_time_step(u, v, w, dx, cfl):
    """cfl * dx / max(max|u|, 1e-4) in the field type (src/project/3d/fluid/time_stepping.cpp:5-7)."""
    t = u.dtype.type
    m = max(max_abs(u), max_abs(v), max_abs(w))
    return float(t(cfl) * t(dx) / max(t(m), t(1e-4)))


# ----------------------------------------------------------------------------------------
# Emitters

def emit_sphere(grid, origin, dx, center, radius):
    suf, _ = _suffix(grid.dtype)
    n2, n1, n0 = grid.shape
    getattr(lib(), f"or_emit_sphere_{suf}")(_p(grid), n0, n1, n2, *origin, dx, *center, radius)


def emit_pool(grid, origin, dx, height):
    suf, _ = _suffix(grid.dtype)
    n2, n1, n0 = grid.shape
    getattr(lib(), f"or_emit_pool_{suf}")(_p(grid), n0, n1, n2, *origin, dx, height)


def emit_box(grid, origin, dx, lo, hi):
    suf, _ = _suffix(grid.dtype)
    n2, n1, n0 = grid.shape
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    getattr(lib(), f"or_emit_box_{suf}")(_p(grid), n0, n1, n2, *origin, dx, _p(lo), _p(hi))


def emit_room(grid):
    suf, _ = _suffix(grid.dtype)
    n2, n1, n0 = grid.shape
    getattr(lib(), f"or_emit_room_{suf}")(_p(grid), n0, n1, n2)


# ----------------------------------------------------------------------------------------
# Scenes: rasterise a scene specification (see eulerian-liquid_gb300/scenes.py) on the CPU.

def rasterise(spec, dtype=np.float64):
    """Returns (phi (nk,nj,ni), solid_nodal (nk+1,nj+1,ni+1)) for a scene specification.

    Liquid and solid lists start from FLT_MAX and take the min of their emitters
    (src/project/3d/fluid/levelset_emitter.cpp:74-79); the nodal solid grid has origin
    -dx/2 per axis (src/project/3d/eulerian_liquid/simulator.cpp:67-68).
    """
    ni, nj, nk = spec["shape"]
    dx = float_dx(ni, dtype)
    big = np.finfo(np.float32).max
    phi = np.full((nk, nj, ni), big, dtype)
    solid = np.full((nk + 1, nj + 1, ni + 1), big, dtype)
    half = float(np.dtype(dtype).type(0.5) * np.dtype(dtype).type(dx))
    for grid, origin, items in ((phi, (0.0, 0.0, 0.0), spec["liquid"]),
                                (solid, (-half, -half, -half), spec["solid"])):
        for e in items:
            if e[0] == "sphere":
                emit_sphere(grid, origin, dx, e[1:4], e[4])
            elif e[0] == "pool":
                emit_pool(grid, origin, dx, e[1])
            elif e[0] == "box":
                emit_box(grid, origin, dx, e[1], e[2])
            elif e[0] == "room":
                emit_room(grid)
            else:
                raise ValueError(e[0])
    return phi, solid


# ----------------------------------------------------------------------------------------
# The reference's own simulator code (oracle/_ref, built from the reference tree by
# oracle/build.py against oracle/eigen_min).  FP32, as the reference.  Every wrapper raises
# RuntimeError when the library is absent; tests skip on ref_sim_available() == False.

_refsim = None


def ref_sim_available():
    return _ref_sim_lib() is not None


def _ref_sim_lib():
    global _refsim
    if _refsim is None:
        L = ref_lib()
        if L is None or not hasattr(L, "refsim_new"):
            return None
        vp, i, d, ll, cp = C.c_void_p, C.c_int, C.c_double, C.c_longlong, C.c_char_p
        L.refsim_compute_weights.argtypes = [i, i, i, d, vp, vp, vp, vp]
        L.refsim_assign_indices.argtypes = [i, i, i, d, vp, vp, vp, vp, vp]
        L.refsim_assign_indices.restype = i
        L.refsim_build_matrix.argtypes = [i, i, i, d] + [vp] * 7 + [d] + [vp] * 6
        L.refsim_build_matrix.restype = i
        L.refsim_build_grid_from_vector.argtypes = [i, i, i, d, vp, i, vp, d, vp]
        L.refsim_update_velocity.argtypes = [i, i, i, d, vp, vp, vp, vp, vp, d]
        L.refsim_extrapolate.argtypes = [vp, vp, i, i, i, i, i]
        L.refsim_calc_time_step.argtypes = [i, i, i, d, vp, vp, vp, d]
        L.refsim_calc_time_step.restype = C.c_float
        L.refsim_advect_collocated.argtypes = [i, i, i, d, vp, vp, vp, vp, vp, d]
        L.refsim_advect_staggered.argtypes = [i, i, i, d, vp, vp, vp, vp, vp, vp, d]
        L.refsim_new.argtypes = [i, i, i, d]
        L.refsim_new.restype = vp
        L.refsim_free.argtypes = [vp]
        L.refsim_dx.argtypes = [vp]
        L.refsim_dx.restype = d
        L.refsim_add_sphere.argtypes = [vp, i, d, d, d, d]
        L.refsim_add_pool.argtypes = [vp, d]
        L.refsim_add_room.argtypes = [vp]
        L.refsim_init_scene.argtypes = [vp]
        L.refsim_field.argtypes = [vp, cp, C.POINTER(ll), C.POINTER(i)]
        L.refsim_field.restype = vp
        L.refsim_call.argtypes = [vp, cp, d]
        L.refsim_call.restype = i
        L.refsim_mesh_obj.argtypes = [vp, i, i, i, d, d, d, d, d, i, cp, vp]
        L.refsim_mesh_obj.restype = i
        _refsim = L
    return _refsim


def _rs():
    L = _ref_sim_lib()
    if L is None:
        raise RuntimeError("the reference library oracle/_ref/libnama_ref.so is not built")
    return L


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def ref_compute_weights(solid_nodal):
    nk1, nj1, ni1 = solid_nodal.shape
    ni, nj, nk = ni1 - 1, nj1 - 1, nk1 - 1
    s = _f32(solid_nodal)
    outs = [np.empty(face_shape(ni, nj, nk, c), np.float32) for c in range(3)]
    _rs().refsim_compute_weights(ni, nj, nk, float_dx(ni, np.float32), _p(s), *[_p(o) for o in outs])
    return tuple(outs)


def ref_assign_indices(phi, wu, wv, ww):
    nk, nj, ni = phi.shape
    arrs = [_f32(a) for a in (phi, wu, wv, ww)]
    idx = np.empty(phi.shape, np.int32)
    n = _rs().refsim_assign_indices(ni, nj, nk, float_dx(ni, np.float32), *[_p(a) for a in arrs], _p(idx))
    return n, idx


def ref_build_matrix(phi, u, v, w, wu, wv, ww, dx, dt):
    """The reference's build_matrix laid out on the grid: (diag, offx, offy, offz, rhs, odd, nnz)."""
    nk, nj, ni = phi.shape
    arrs = [_f32(a) for a in (phi, u, v, w, wu, wv, ww)]
    outs = [np.empty(phi.shape, np.float64) for _ in range(5)]
    nnz = C.c_longlong()
    odd = _rs().refsim_build_matrix(ni, nj, nk, dx, *[_p(a) for a in arrs], dt, *[_p(o) for o in outs],
                                    C.byref(nnz))
    return (*outs, odd, nnz.value)


def ref_build_grid_from_vector(vec, indices, background=0.0):
    nk, nj, ni = indices.shape
    vec = np.ascontiguousarray(vec, np.float64)
    idx = np.ascontiguousarray(indices, np.int32)
    out = np.empty(indices.shape, np.float32)
    _rs().refsim_build_grid_from_vector(ni, nj, nk, float_dx(ni, np.float32), _p(vec), vec.size, _p(idx),
                                        background, _p(out))
    return out


def ref_update_velocity(u, v, w, pressure, phi, dx, dt):
    nk, nj, ni = phi.shape
    u, v, w = (np.array(a, dtype=np.float32, copy=True, order="C") for a in (u, v, w))
    p, phi = _f32(pressure), _f32(phi)
    _rs().refsim_update_velocity(ni, nj, nk, dx, _p(u), _p(v), _p(w), _p(p), _p(phi), dt)
    return u, v, w


def ref_extrapolate(grid, valid, layers=10, keep_valid=False):
    n2, n1, n0 = grid.shape
    g = np.array(grid, dtype=np.float32, copy=True, order="C")
    m = np.array(valid, dtype=np.uint8, copy=True, order="C")
    _rs().refsim_extrapolate(_p(g), _p(m), n0, n1, n2, layers, int(keep_valid))
    return g, m


def ref_calc_time_step(u, v, w, dx, cfl):
    nk, nj, ni1 = u.shape
    u, v, w = (_f32(a) for a in (u, v, w))
    return float(_rs().refsim_calc_time_step(ni1 - 1, nj, nk, dx, _p(u), _p(v), _p(w), cfl))


def ref_advect_collocated(phi, u, v, w, dx, dt):
    nk, nj, ni = phi.shape
    arrs = [_f32(a) for a in (phi, u, v, w)]
    out = np.empty(phi.shape, np.float32)
    _rs().refsim_advect_collocated(ni, nj, nk, dx, _p(out), *[_p(a) for a in arrs], dt)
    return out


def ref_advect_staggered(u, v, w, dx, dt):
    nk, nj, ni1 = u.shape
    u, v, w = (_f32(a) for a in (u, v, w))
    outs = [np.empty(a.shape, np.float32) for a in (u, v, w)]
    _rs().refsim_advect_staggered(ni1 - 1, nj, nk, dx, *[_p(o) for o in outs], _p(u), _p(v), _p(w), dt)
    return tuple(outs)


def ref_mesh_obj(phi, dx, origin=(0.0, 0.0, 0.0), isolevel=0.0, method=0, path=""):
    """The reference's get_mesh + Mesh::save: returns (vertices, faces, vertices per face)."""
    nk, nj, ni = phi.shape
    counts = np.zeros(3, np.int64)
    phi = _f32(phi)
    rc = _rs().refsim_mesh_obj(_p(phi), ni, nj, nk, dx, *origin, isolevel, method, path.encode(), _p(counts))
    if rc != 0:
        raise OSError(f"cannot write {path}")
    return tuple(int(c) for c in counts)


class RefSimulator:
    """The reference's Simulator (simulator.cpp) on an (ni, nj, nk) grid of width 1."""

    _SHAPES = {"phi": 0, "phi_valid": 0, "pressure": 0, "indices": 0, "solid_cell": 0,
               "u": 1, "weight_u": 1, "valid_u": 1, "v": 2, "weight_v": 2, "valid_v": 2,
               "w": 3, "weight_w": 3, "valid_w": 3, "solid_nodal": 4}

    def __init__(self, ni, nj, nk, cfl=1.0):
        self.shape3 = (ni, nj, nk)
        self.h = _rs().refsim_new(ni, nj, nk, cfl)
        self.dx = _rs().refsim_dx(self.h)

    def close(self):
        if self.h:
            _rs().refsim_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_sphere(self, center, radius, liquid=True):
        _rs().refsim_add_sphere(self.h, int(liquid), *center, radius)

    def add_pool(self, height):
        _rs().refsim_add_pool(self.h, height)

    def add_room(self):
        _rs().refsim_add_room(self.h)

    def init_scene(self):
        _rs().refsim_init_scene(self.h)

    def field(self, name):
        """A numpy view (nk, nj, ni)-shaped onto the reference's own storage of a field."""
        ni, nj, nk = self.shape3
        comp = self._SHAPES[name]
        shape = (nk + 1, nj + 1, ni + 1) if comp == 4 else ((nk, nj, ni) if comp == 0 else
                                                             face_shape(ni, nj, nk, comp - 1))
        count, elem = C.c_longlong(), C.c_int()
        ptr = _rs().refsim_field(self.h, name.encode(), C.byref(count), C.byref(elem))
        dt = {4: np.float32, 1: np.uint8}[elem.value]
        if name == "indices":
            dt = np.int32
        buf = (C.c_char * (count.value * elem.value)).from_address(ptr)
        return np.frombuffer(buf, dtype=dt).reshape(shape)

    def call(self, method, dt=0.0):
        rc = _rs().refsim_call(self.h, method.encode(), dt)
        if rc == -1:
            raise RuntimeError("No fluid")
        if rc == -2:
            raise ValueError(method)
