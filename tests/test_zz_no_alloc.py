"""el_solve_pressure_noalloc: the pressure solve for callers that cannot call cudaMalloc (their
device memory is reserved by another allocator, or they cannot afford an allocation's device
synchronisation).  Its output is checked against the existing el_solve_pressure entry point with
the same solver (plain FP64 Jacobi PCG) through the C ABI, on two calls in a row, since every
call reuses the same fixed scratch array.  Collected last (file name) so that a run stopping at
the first failure has run every other test first; it needs no state from them."""

import ctypes as C

import numpy as np
import pytest

import conftest
from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-8         # solve tolerance of both entry points
MATCH = 1e-6       # norm-wise relative agreement required between the two entry points


def _declare(lib, el):
    f = lib.el_solve_pressure_noalloc
    f.argtypes = [C.POINTER(el.Grid)] + [C.c_void_p] * 8 + [C.c_double, C.c_double, C.c_int,
                                                            C.POINTER(el.SolveStats), C.c_void_p]
    f.restype = C.c_int
    return f


def test_noalloc_matches_solve_pressure_on_two_calls(el, orc):
    torch = pytest.importorskip("torch")
    lib = el.load()
    solve_noalloc = _declare(lib, el)
    n = 40
    spec = conftest.load_package().scenes.spheres_pool(n, 5)
    sim = el.Simulator(n, n, n, dtype=el.EL_F32)
    sim.init_scene(spec)
    phi = sim.download("phi")
    weights = [sim.download(f) for f in ("weight_u", "weight_v", "weight_w")]
    grid = el.Grid(n, n, n, sim.dx)
    dev = {"phi": torch.from_numpy(phi).cuda()}
    for f, a in zip(("weight_u", "weight_v", "weight_w"), weights):
        dev[f] = torch.from_numpy(a).cuda()
    dev["pressure"] = torch.full(phi.shape, np.nan, dtype=torch.float32, device="cuda")
    rng = np.random.default_rng(11)
    for call, dt in enumerate((0.01, 0.004)):
        vel = [rng.uniform(-1, 1, sim.shape(f)).astype(np.float32) for f in ("u", "v", "w")]
        # the existing entry point on a context
        for f, a in zip(("u", "v", "w"), vel):
            sim.upload(f, a)
        ref = sim.solve_pressure(dt, solver=el.SOLVER_JACOBI_FP64, tol=TOL, max_iter=20000, check_every=8)
        assert ref["status"] == el.EL_OK
        want = {f: sim.download(f) for f in ("pressure", "u", "v", "w")}
        # the no-allocation entry point on caller-owned device arrays
        for f, a in zip(("u", "v", "w"), vel):
            dev[f] = torch.from_numpy(a.copy()).cuda()
        stats = el.SolveStats()
        stream = torch.cuda.current_stream().cuda_stream
        rc = solve_noalloc(C.byref(grid), dev["phi"].data_ptr(), dev["u"].data_ptr(), dev["v"].data_ptr(),
                           dev["w"].data_ptr(), dev["weight_u"].data_ptr(), dev["weight_v"].data_ptr(),
                           dev["weight_w"].data_ptr(), dev["pressure"].data_ptr(), dt, TOL, 20000, C.byref(stats),
                           stream)
        torch.cuda.synchronize()
        assert rc == el.EL_OK, (call, rc, el.status_string(rc))
        assert stats.status == el.EL_OK and stats.fluid_cells == ref["fluid_cells"]
        assert stats.relres < TOL
        for f in ("pressure", "u", "v", "w"):
            got = dev[f].cpu().numpy()
            assert np.all(np.isfinite(got)), (call, f)
            assert rel_err(got, want[f]) <= MATCH, (call, f, rel_err(got, want[f]))
        # and the pressure solves the CPU oracle's own system for these inputs: the residual is
        # that of the FP64 solution rounded to the FP32 pressure grid
        mats = orc.build_matrix(phi, *vel, *weights, sim.dx, dt)
        p = dev["pressure"].cpu().numpy().astype(np.float64)
        r = mats[4] - orc.spmv(*mats[:4], np.where(mats[0] > 0, p, 0.0))
        assert np.linalg.norm(r) / np.linalg.norm(mats[4]) <= 5e-5, call
    sim.close()


def test_noalloc_rejects_grids_beyond_the_limit(el):
    lib = el.load()
    solve_noalloc = _declare(lib, el)
    n = 65  # 65^3 > EL_NOALLOC_MAX_CELLS = 64^3
    grid = el.Grid(n, n, n, 1.0 / n)
    stats = el.SolveStats()
    # rejected before any device work, so placeholder pointers are never dereferenced
    rc = solve_noalloc(C.byref(grid), *([16] * 8), 0.01, TOL, 100, C.byref(stats), None)
    assert rc == el.EL_ERR_TOO_LARGE
    assert "limit" in el.status_string(rc)
