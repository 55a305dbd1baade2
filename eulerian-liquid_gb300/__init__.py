"""Python binding of the GB300 hot-path library (ctypes over the C ABI).

The product is the C ABI in ``include/eulerian_liquid_gb300.h`` implemented by
``_build/libeulerian_liquid_gb300.so`` (CUDA, sm_103a).  This module loads that library and
offers ``Simulator``, a thin wrapper whose methods carry the names of the reference's
``nama::_3d::eulerian_liquid::Simulator`` (include/nama/project/3d/eulerian_liquid/simulator.h:18-53),
over device-resident fields.  There is no CPU fallback: without the library or a GPU every
call raises.

Arrays use the reference layout: numpy shape (nk, nj, ni) in C order, flat index
i + ni*(j + nj*k) (include/nama/common/array.h:281-286).
"""

import ctypes as C
import os

import numpy as np

from . import build as _build_mod
from . import autotune  # noqa: F401  (re-exported)
from . import state  # noqa: F401  (re-exported)
from . import scenes  # noqa: F401  (re-exported)

HERE = os.path.dirname(os.path.abspath(__file__))

EL_OK = 0
EL_ERR_INVALID_ARGUMENT = 1
EL_ERR_NO_FLUID = 2
EL_ERR_NOT_CONVERGED = 3
EL_ERR_NAN = 4
EL_ERR_CUDA = 5
EL_ERR_OUT_OF_MEMORY = 6
EL_ERR_TIMEOUT = 7
EL_ERR_TOO_LARGE = 8

EL_F32, EL_F64 = 0, 1
TRACE_RK2, TRACE_RK3 = 0, 1
SAMPLE_TRILINEAR, SAMPLE_WENO6 = 0, 1
SOLVER_JACOBI_FP64, SOLVER_MG_FP64, SOLVER_MIXED = 0, 1, 2
# kernel classes of el_ctx_profile_* (enum el_kernel_class)
KERNEL_CLASSES = ("advect_phi", "advect_vel", "extrapolate", "masks", "build", "dir_spmv", "update",
                  "mg_smooth_fine", "mg_restrict_fine", "mg_coarse", "residual_fp64", "other")
(EL_KC_ADVECT_PHI, EL_KC_ADVECT_VEL, EL_KC_EXTRAPOLATE, EL_KC_MASKS, EL_KC_BUILD, EL_KC_DIR_SPMV, EL_KC_UPDATE,
 EL_KC_SMOOTH, EL_KC_RESTRICT, EL_KC_MG_COARSE, EL_KC_RESIDUAL, EL_KC_OTHER) = range(12)
EL_KC_COUNT = 12

FIELDS = {
    "phi": 0, "u": 1, "v": 2, "w": 3, "solid_nodal": 4, "weight_u": 5, "weight_v": 6,
    "weight_w": 7, "pressure": 8, "solid_cell": 9, "valid_u": 10, "valid_v": 11, "valid_w": 12,
    "valid_phi": 13, "indices": 14,
}

REFERENCE_GRAVITY = 9.80665  # include/nama/constants.h:6


class ELError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, status, message):
        super().__init__(f"{message} (status {status})")
        self.status = status


class NoFluid(ELError):
    """The reference's std::runtime_error("No fluid") (src/project/3d/fluid/projection.cpp:24-26)."""


class SolveParams(C.Structure):
    _fields_ = [("solver", C.c_int), ("tol", C.c_double), ("max_iter", C.c_int), ("check_every", C.c_int),
                ("max_outer", C.c_int), ("inner_floor", C.c_double), ("initial_guess", C.c_int)]


class SolveStats(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("outer_iterations", C.c_int),
                ("fluid_cells", C.c_int), ("relres", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class StepParams(C.Structure):
    _fields_ = [("trace_phi", C.c_int), ("sample_phi", C.c_int), ("trace_vel", C.c_int),
                ("sample_vel", C.c_int), ("gravity", C.c_double), ("extrapolation_layers", C.c_int),
                ("solve", SolveParams)]


class StepStats(C.Structure):
    _fields_ = [("dt", C.c_double), ("solve", SolveStats)]


class Grid(C.Structure):
    _fields_ = [("ni", C.c_int), ("nj", C.c_int), ("nk", C.c_int), ("dx", C.c_double)]


class Tuning(C.Structure):
    _fields_ = [("seg_blocks_per_sm", C.c_int), ("stencil_blocks_per_sm", C.c_int),
                ("extrapolate_blocks_per_sm", C.c_int), ("advect_rows", C.c_int), ("advect_tiled", C.c_int),
                ("solver_tiles", C.c_int), ("coarse_fused", C.c_int),
                ("dependent_launch", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchStats(C.Structure):
    _fields_ = [("steps", C.c_int64), ("frames", C.c_int64), ("iterations", C.c_int64),
                ("outer_iterations", C.c_int64), ("kernels", C.c_int64), ("unconverged_steps", C.c_int64),
                ("no_fluid_steps", C.c_int64), ("bad_steps", C.c_int64), ("time", C.c_double),
                ("last_dt", C.c_double), ("max_relres", C.c_double), ("frame_time", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ProfileEntry(C.Structure):
    _fields_ = [("launches", C.c_int64), ("ms", C.c_double), ("bytes", C.c_double)]


_lib = None


def debug_check_take():
    """(checked, word): whether the loaded library is the debug build, and the first failed
    device-side index check since the last call as (site << 40) | index, or 0."""
    w = C.c_uint64()
    on = C.c_int()
    st = load().el_debug_check_take(C.byref(w), C.byref(on))
    if st != EL_OK:
        raise ELError(st, "el_debug_check_take")
    return bool(on.value), int(w.value)


def library_path():
    return _build_mod.LIB


def load(build_if_needed=True):
    """Load the CUDA library (building it in-tree when sources are newer).  With the environment
    variable EL_CHECKED=1 the process loads the debug build instead, whose kernels check their
    indices (el_debug_check_take reports a failed check)."""
    global _lib
    if _lib is not None:
        return _lib
    checked = os.environ.get("EL_CHECKED", "0") == "1"
    path = _build_mod.LIB_CHECKED if checked else _build_mod.LIB
    if build_if_needed and not _build_mod.up_to_date(checked):
        path = _build_mod.build(checked=checked)
    if not os.path.exists(path):
        raise ImportError(f"the CUDA hot-path library is not built: {path}")
    lib = C.CDLL(path)
    _declare(lib)
    _lib = lib
    return lib


def _declare(L):
    vp, i, d, sz = C.c_void_p, C.c_int, C.c_double, C.c_size_t
    ctxp = C.c_void_p
    L.el_status_string.restype = C.c_char_p
    L.el_status_string.argtypes = [i]
    L.el_ctx_last_error.restype = C.c_char_p
    L.el_ctx_last_error.argtypes = [ctxp]
    L.el_ctx_create.argtypes = [i, i, i, d, i, i, C.POINTER(C.c_void_p)]
    L.el_ctx_destroy.argtypes = [ctxp]
    L.el_ctx_set_stream.argtypes = [ctxp, vp]
    L.el_ctx_get_stream.argtypes = [ctxp]
    L.el_ctx_get_stream.restype = vp
    L.el_ctx_sync.argtypes = [ctxp]
    L.el_ctx_kernel_launches.argtypes = [ctxp]
    L.el_ctx_kernel_launches.restype = C.c_int64
    L.el_state_save.argtypes = [ctxp, C.c_char_p, d]
    L.el_state_load.argtypes = [ctxp, C.c_char_p, C.POINTER(C.c_double)]
    L.el_ctx_set_tuning.argtypes = [ctxp, C.POINTER(Tuning)]
    L.el_ctx_profile_begin.argtypes = [ctxp, C.c_uint32]
    L.el_ctx_profile_end.argtypes = [ctxp, C.POINTER(ProfileEntry)]
    L.el_ctx_get_tuning.argtypes = [ctxp, C.POINTER(Tuning)]
    L.el_ctx_solver_tiles_active.argtypes = [ctxp, C.POINTER(C.c_int)]
    L.el_upload.argtypes = [ctxp, i, vp, sz]
    L.el_download.argtypes = [ctxp, i, vp, sz]
    L.el_debug_check_take.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_int)]
    L.el_upload_async.argtypes = [ctxp, i, vp, sz, vp]
    L.el_download_async.argtypes = [ctxp, i, vp, sz, vp]
    L.el_field_device_ptr.argtypes = [ctxp, i, C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)]
    L.el_emit_clear.argtypes = [ctxp, i]
    L.el_emit_sphere.argtypes = [ctxp, i, d, d, d, d]
    L.el_emit_pool.argtypes = [ctxp, i, d]
    L.el_emit_box.argtypes = [ctxp, i, vp, vp]
    L.el_emit_room.argtypes = [ctxp, i]
    for name in ("el_compute_weights", "el_calc_cell_centered_solid_phi", "el_find_valid_level_set",
                 "el_find_valid_velocity", "el_set_invalid_velocity_zero"):
        getattr(L, name).argtypes = [ctxp]
    L.el_advect_level_set.argtypes = [ctxp, d, i, i]
    L.el_advect_velocity.argtypes = [ctxp, d, i, i]
    L.el_add_gravity.argtypes = [ctxp, d, d]
    L.el_extrapolate_level_set.argtypes = [ctxp, i]
    L.el_extrapolate_velocity.argtypes = [ctxp, i]
    L.el_solve_pressure.argtypes = [ctxp, d, C.POINTER(SolveParams), C.POINTER(SolveStats)]
    L.el_calc_time_step.argtypes = [ctxp, d, C.POINTER(C.c_double)]
    L.el_step.argtypes = [ctxp, d, C.POINTER(StepParams), C.POINTER(StepStats)]
    L.el_assign_indices.argtypes = [ctxp, C.POINTER(C.c_int)]
    L.el_build_matrix.argtypes = [ctxp, d]
    L.el_download_matrix.argtypes = [ctxp, vp, vp, vp, vp, vp]
    L.el_update_velocity_using_pressure.argtypes = [ctxp, d]
    L.el_advect_collocated_grid.argtypes = [C.POINTER(Grid), i, vp, vp, vp, vp, vp, d, i, i, vp]
    L.el_advect_staggered_grid.argtypes = [C.POINTER(Grid), i, vp, vp, vp, vp, vp, vp, vp, vp, vp, d, i, i, vp]
    L.el_compute_staggered_grid_weight.argtypes = [C.POINTER(Grid), i, vp, vp, vp, vp, vp]
    bp = C.c_void_p
    L.el_batch_create.argtypes = [C.POINTER(C.c_void_p), i, C.POINTER(StepParams), d, d, C.POINTER(C.c_void_p)]
    L.el_batch_destroy.argtypes = [bp]
    L.el_batch_last_error.argtypes = [bp]
    L.el_batch_last_error.restype = C.c_char_p
    L.el_batch_step.argtypes = [bp, i]
    L.el_batch_sync.argtypes = [bp]
    L.el_batch_stats_get.argtypes = [bp, C.POINTER(BatchStats)]
    L.el_batch_stats_reset.argtypes = [bp]
    L.el_batch_get_stream.argtypes = [bp]
    L.el_batch_get_stream.restype = vp
    L.el_batch_graph_kernels.argtypes = [bp]
    L.el_batch_graph_kernels.restype = C.c_int64


def status_string(status):
    return load().el_status_string(status).decode()


def solve_params(solver=SOLVER_MIXED, tol=1e-6, max_iter=2000, check_every=4, max_outer=8, inner_floor=1e-4,
                 initial_guess=0):
    return SolveParams(solver, tol, max_iter, check_every, max_outer, inner_floor, initial_guess)


def step_params(trace_phi=TRACE_RK2, sample_phi=SAMPLE_TRILINEAR, trace_vel=TRACE_RK2,
                sample_vel=SAMPLE_TRILINEAR, gravity=REFERENCE_GRAVITY, extrapolation_layers=10, **solve):
    return StepParams(trace_phi, sample_phi, trace_vel, sample_vel, gravity, extrapolation_layers,
                      solve_params(**solve))


def _np_dtype(dtype):
    return np.float64 if dtype == EL_F64 else np.float32


class Simulator:
    """A device-resident scene (Simulator::create_grid, simulator.cpp:52-70) driven through the C ABI."""

    def __init__(self, ni, nj, nk, dx=None, dtype=EL_F32, device=0):
        self.lib = load()
        self.ni, self.nj, self.nk = ni, nj, nk
        self.dtype = dtype
        self.np_dtype = _np_dtype(dtype)
        if dx is None:  # width 1: dx = 1 / ni in the field type (simulator.cpp:56)
            dx = float(np.float32(1.0) / np.float32(ni)) if dtype == EL_F32 else 1.0 / ni
        self.dx = dx
        h = C.c_void_p()
        st = self.lib.el_ctx_create(ni, nj, nk, dx, dtype, device, C.byref(h))
        if st != EL_OK:
            raise ELError(st, f"el_ctx_create({ni},{nj},{nk}) failed: {status_string(st)}")
        self.h = h

    # -- lifetime -------------------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.el_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st, what):
        if st == EL_OK:
            return
        msg = self.lib.el_ctx_last_error(self.h).decode()
        if st == EL_ERR_NO_FLUID:
            raise NoFluid(st, "No fluid")
        raise ELError(st, f"{what}: {status_string(st)}: {msg}")

    # -- state files (el_state_save / el_state_load) ------------------------------------------
    def save_state(self, path, time=0.0):
        self._check(self.lib.el_state_save(self.h, os.fsencode(path), time), "save_state")

    def load_state(self, path):
        t = C.c_double()
        self._check(self.lib.el_state_load(self.h, os.fsencode(path), C.byref(t)), "load_state")
        return t.value

    # -- launch shapes ----------------------------------------------------------------------
    def get_tuning(self):
        t = Tuning()
        self._check(self.lib.el_ctx_get_tuning(self.h, C.byref(t)), "get_tuning")
        return t.as_dict()

    def set_tuning(self, **kw):
        t = Tuning(**{**self.get_tuning(), **kw})
        self._check(self.lib.el_ctx_set_tuning(self.h, C.byref(t)), "set_tuning")

    def march_on(self):
        """True when the mixed solver's finest level runs on the z-marching tile kernels."""
        on = C.c_int()
        self._check(self.lib.el_ctx_solver_tiles_active(self.h, C.byref(on)), "solver_tiles_active")
        return bool(on.value)

    # -- fields ---------------------------------------------------------------------------
    def shape(self, field):
        ni, nj, nk = self.ni, self.nj, self.nk
        return {
            "u": (nk, nj, ni + 1), "weight_u": (nk, nj, ni + 1), "valid_u": (nk, nj, ni + 1),
            "v": (nk, nj + 1, ni), "weight_v": (nk, nj + 1, ni), "valid_v": (nk, nj + 1, ni),
            "w": (nk + 1, nj, ni), "weight_w": (nk + 1, nj, ni), "valid_w": (nk + 1, nj, ni),
            "solid_nodal": (nk + 1, nj + 1, ni + 1),
        }.get(field, (nk, nj, ni))

    def field_dtype(self, field):
        if field.startswith("valid"):
            return np.uint8
        if field == "indices":
            return np.int32
        return self.np_dtype

    def upload(self, field, array):
        a = np.ascontiguousarray(array, dtype=self.field_dtype(field))
        if a.shape != self.shape(field):
            raise ValueError(f"{field}: shape {a.shape} != {self.shape(field)}")
        self._check(self.lib.el_upload(self.h, FIELDS[field], a.ctypes.data, a.nbytes), f"upload {field}")

    def download(self, field, out=None):
        """Copy a field to the host (into `out`, e.g. a pinned buffer, when given)."""
        a = out if out is not None else np.empty(self.shape(field), dtype=self.field_dtype(field))
        if a.shape != self.shape(field) or a.dtype != self.field_dtype(field) or not a.flags.c_contiguous:
            raise ValueError(f"{field}: output buffer must be a C-contiguous {self.field_dtype(field)} {self.shape(field)}")
        self._check(self.lib.el_download(self.h, FIELDS[field], a.ctypes.data, a.nbytes), f"download {field}")
        return a

    def _host_buffer(self, field, a):
        if a.shape != self.shape(field) or a.dtype != self.field_dtype(field) or not a.flags.c_contiguous:
            raise ValueError(f"{field}: buffer must be a C-contiguous {self.field_dtype(field)} {self.shape(field)}")
        return a

    def upload_async(self, field, array, stream=None):
        """Enqueue the copy of a (pinned, C-contiguous) host array into a field on `stream` (a
        cudaStream_t handle; None = the context's stream) without waiting for it."""
        a = self._host_buffer(field, array)
        self._check(self.lib.el_upload_async(self.h, FIELDS[field], a.ctypes.data, a.nbytes, stream),
                    f"upload_async {field}")

    def download_async(self, field, out, stream=None):
        """Enqueue the copy of a field into a (pinned) host array without waiting for it."""
        a = self._host_buffer(field, out)
        self._check(self.lib.el_download_async(self.h, FIELDS[field], a.ctypes.data, a.nbytes, stream),
                    f"download_async {field}")
        return a

    @property
    def stream_handle(self):
        """The context's cudaStream_t (el_ctx_get_stream)."""
        return self.lib.el_ctx_get_stream(self.h)

    def device_ptr(self, field):
        p = C.c_void_p()
        n = C.c_size_t()
        self._check(self.lib.el_field_device_ptr(self.h, FIELDS[field], C.byref(p), C.byref(n)), "device_ptr")
        return p.value, n.value

    def set_stream(self, stream_handle):
        self._check(self.lib.el_ctx_set_stream(self.h, stream_handle), "set_stream")

    def stream(self):
        return self.lib.el_ctx_get_stream(self.h)

    def sync(self):
        self._check(self.lib.el_ctx_sync(self.h), "sync")

    def kernel_launches(self):
        return int(self.lib.el_ctx_kernel_launches(self.h))

    # -- per-kernel-class timing (el_ctx_profile_begin / _end) ------------------------------
    def profile_begin(self, class_mask=(1 << EL_KC_COUNT) - 1):
        self._check(self.lib.el_ctx_profile_begin(self.h, class_mask), "profile_begin")

    def profile_end(self):
        """{class name: {launches, ms, bytes}} for the classes that launched while profiling."""
        out = (ProfileEntry * EL_KC_COUNT)()
        self._check(self.lib.el_ctx_profile_end(self.h, out), "profile_end")
        return {KERNEL_CLASSES[c]: {"launches": int(out[c].launches), "ms": out[c].ms, "bytes": out[c].bytes}
                for c in range(EL_KC_COUNT) if out[c].launches}

    # -- scene set-up (levelset_emitter.cpp, boundary.cpp, simulator.cpp:72-76, 160-200) ----
    def emit(self, target, item):
        kind = item[0]
        if kind == "clear":
            st = self.lib.el_emit_clear(self.h, target)
        elif kind == "sphere":
            st = self.lib.el_emit_sphere(self.h, target, *map(float, item[1:5]))
        elif kind == "pool":
            st = self.lib.el_emit_pool(self.h, target, float(item[1]))
        elif kind == "box":
            lo = np.asarray(item[1], np.float64)
            hi = np.asarray(item[2], np.float64)
            st = self.lib.el_emit_box(self.h, target, lo.ctypes.data, hi.ctypes.data)
        elif kind == "room":
            st = self.lib.el_emit_room(self.h, target)
        else:
            raise ValueError(kind)
        self._check(st, f"emit {kind}")

    def init_scene(self, spec):
        """init_scene + compute_weights + find_valid_level_set (apps/eulerian_liquid_3d.cpp:137-139)."""
        for target, items in ((0, spec["liquid"]), (1, spec["solid"])):
            self.emit(target, ("clear",))
            for item in items:
                self.emit(target, item)
        self.calc_cell_centered_solid_phi()
        self.compute_weights()
        self.find_valid_level_set()

    def compute_weights(self):
        self._check(self.lib.el_compute_weights(self.h), "compute_weights")

    def calc_cell_centered_solid_phi(self):
        self._check(self.lib.el_calc_cell_centered_solid_phi(self.h), "calc_cell_centered_solid_phi")

    def find_valid_level_set(self):
        self._check(self.lib.el_find_valid_level_set(self.h), "find_valid_level_set")

    # -- step methods (simulator.h:32-53) -----------------------------------------------
    def advect_level_set(self, dt, trace=TRACE_RK2, sample=SAMPLE_TRILINEAR):
        self._check(self.lib.el_advect_level_set(self.h, dt, trace, sample), "advect_level_set")

    def advect_velocity(self, dt, trace=TRACE_RK2, sample=SAMPLE_TRILINEAR):
        self._check(self.lib.el_advect_velocity(self.h, dt, trace, sample), "advect_velocity")

    def add_gravity(self, dt, gravity=REFERENCE_GRAVITY):
        self._check(self.lib.el_add_gravity(self.h, dt, gravity), "add_gravity")

    def extrapolate_level_set(self, layers=10):
        self._check(self.lib.el_extrapolate_level_set(self.h, layers), "extrapolate_level_set")

    def extrapolate_velocity(self, layers=10):
        self._check(self.lib.el_extrapolate_velocity(self.h, layers), "extrapolate_velocity")

    def find_valid_velocity(self):
        self._check(self.lib.el_find_valid_velocity(self.h), "find_valid_velocity")

    def set_invalid_velocity_zero(self):
        self._check(self.lib.el_set_invalid_velocity_zero(self.h), "set_invalid_velocity_zero")

    def solve_pressure(self, dt, **solve):
        prm = solve_params(**solve)
        stats = SolveStats()
        st = self.lib.el_solve_pressure(self.h, dt, C.byref(prm), C.byref(stats))
        if st == EL_ERR_NOT_CONVERGED:
            return stats.as_dict()
        self._check(st, "solve_pressure")
        return stats.as_dict()

    def calc_time_step(self, cfl):
        dt = C.c_double()
        self._check(self.lib.el_calc_time_step(self.h, cfl, C.byref(dt)), "calc_time_step")
        return dt.value

    def step(self, dt, params=None, **kw):
        prm = params if params is not None else step_params(**kw)
        stats = StepStats()
        st = self.lib.el_step(self.h, dt, C.byref(prm), C.byref(stats))
        if st == EL_ERR_NOT_CONVERGED:
            return {"dt": stats.dt, **stats.solve.as_dict()}
        self._check(st, "step")
        return {"dt": stats.dt, **stats.solve.as_dict()}

    # -- projection pieces (projection.h:10-22) -------------------------------------------
    def assign_indices(self):
        n = C.c_int()
        self._check(self.lib.el_assign_indices(self.h, C.byref(n)), "assign_indices")
        return n.value, self.download("indices")

    def build_matrix(self, dt):
        self._check(self.lib.el_build_matrix(self.h, dt), "build_matrix")
        shape = (self.nk, self.nj, self.ni)
        outs = [np.empty(shape, np.float64) for _ in range(5)]
        self._check(self.lib.el_download_matrix(self.h, *[o.ctypes.data for o in outs]), "download_matrix")
        return tuple(outs)  # diag, offx, offy, offz, rhs

    def matrix(self):
        """The system the last build made (no rebuild): diag, offx, offy, offz, rhs as doubles."""
        shape = (self.nk, self.nj, self.ni)
        outs = [np.empty(shape, np.float64) for _ in range(5)]
        self._check(self.lib.el_download_matrix(self.h, *[o.ctypes.data for o in outs]), "download_matrix")
        return tuple(outs)

    def update_velocity_using_pressure(self, dt):
        self._check(self.lib.el_update_velocity_using_pressure(self.h, dt), "update_velocity_using_pressure")


class Batch:
    """Scenes advanced together, one CUDA graph launch per sub-step (el_batch_*).

    Each sub-step is Simulator::update's CFL sub-step (simulator.cpp:23-42) of every scene with
    its own dt, decided on the device.  `scenes` are Simulator objects; they must outlive the
    batch and must not be stepped on their own between batch steps."""

    def __init__(self, scenes, params=None, cfl=1.0, dt_frame=1.0 / 60.0, **kw):
        self.lib = load()
        self.scenes = list(scenes)
        prm = params if params is not None else step_params(**kw)
        arr = (C.c_void_p * len(self.scenes))(*[s.h.value for s in self.scenes])
        h = C.c_void_p()
        st = self.lib.el_batch_create(arr, len(self.scenes), C.byref(prm), cfl, dt_frame, C.byref(h))
        if st != EL_OK:
            msg = self.lib.el_ctx_last_error(self.scenes[0].h).decode() if self.scenes else ""
            raise ELError(st, f"el_batch_create: {status_string(st)}: {msg}")
        self.h = h

    def _check(self, st, what):
        if st != EL_OK:
            raise ELError(st, f"{what}: {status_string(st)}: {self.lib.el_batch_last_error(self.h).decode()}")

    def step(self, steps=1):
        self._check(self.lib.el_batch_step(self.h, steps), "el_batch_step")

    def sync(self):
        self._check(self.lib.el_batch_sync(self.h), "el_batch_sync")

    def stats(self):
        out = (BatchStats * len(self.scenes))()
        self._check(self.lib.el_batch_stats_get(self.h, out), "el_batch_stats_get")
        return [o.as_dict() for o in out]

    def reset_stats(self):
        self._check(self.lib.el_batch_stats_reset(self.h), "el_batch_stats_reset")

    @property
    def stream(self):
        return self.lib.el_batch_get_stream(self.h)

    def graph_kernels(self):
        return self.lib.el_batch_graph_kernels(self.h)

    def close(self):
        if getattr(self, "h", None):
            self.lib.el_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


# ---- stateless operators on caller-owned device memory ------------------------------------

def advect_collocated_grid(ni, nj, nk, dx, dtype, out_ptr, in_ptr, u_ptr, v_ptr, w_ptr, dt,
                           trace=TRACE_RK2, sample=SAMPLE_TRILINEAR, stream=None):
    g = Grid(ni, nj, nk, dx)
    st = load().el_advect_collocated_grid(C.byref(g), dtype, out_ptr, in_ptr, u_ptr, v_ptr, w_ptr, dt, trace,
                                          sample, stream)
    if st != EL_OK:
        raise ELError(st, "el_advect_collocated_grid")


def advect_staggered_grid(ni, nj, nk, dx, dtype, outs, ins, vel, dt, trace=TRACE_RK2,
                          sample=SAMPLE_TRILINEAR, stream=None):
    g = Grid(ni, nj, nk, dx)
    st = load().el_advect_staggered_grid(C.byref(g), dtype, *outs, *ins, *vel, dt, trace, sample, stream)
    if st != EL_OK:
        raise ELError(st, "el_advect_staggered_grid")


def compute_staggered_grid_weight(ni, nj, nk, dx, dtype, w_ptrs, solid_ptr, stream=None):
    g = Grid(ni, nj, nk, dx)
    st = load().el_compute_staggered_grid_weight(C.byref(g), dtype, *w_ptrs, solid_ptr, stream)
    if st != EL_OK:
        raise ELError(st, "el_compute_staggered_grid_weight")


from . import warmstart  # noqa: E402,F401  (re-exported; needs the names above)
