"""Advection on the GPU vs the CPU oracle (a1-a6): RK2/RK3 backtrace, trilinear/WENO6 sampling,
FP64 to 1e-12 and FP32 to the float tolerance, through the context and the stateless C ABI."""

import ctypes as C

import numpy as np
import pytest

from conftest import rel_err
from helpers import RTOL_F32, RTOL_F32_WENO, RTOL_F64, make_sim, smooth_fields

pytestmark = pytest.mark.gpu

SCHEMES = [(0, 0), (0, 1), (1, 0), (1, 1)]  # (trace RK2/RK3, sample trilinear/WENO6)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("trace,sample", SCHEMES)
@pytest.mark.parametrize("shape", [(24, 20, 16), (13, 9, 11)])
@pytest.mark.parametrize("cells", [0.9, 2.6])
def test_advect_level_set_and_velocity(el, orc, dtype, trace, sample, shape, cells):
    """cells = dt / dx: at 0.9 every foot point lies in the tiled kernels' staged boxes; at 2.6
    (speeds up to 0.8) part of them leave the boxes and take the global-memory path."""
    ni, nj, nk = shape
    dx, phi, u, v, w = smooth_fields(orc, ni, nj, nk, dtype, seed=11)
    dt = float(dtype(cells) * dtype(dx))
    tol = RTOL_F64 if dtype == np.float64 else (RTOL_F32_WENO if sample == 1 else RTOL_F32)
    sim = make_sim(el, shape, dtype)
    for f, a in (("phi", phi), ("u", u), ("v", v), ("w", w)):
        sim.upload(f, a)
    sim.advect_level_set(dt, trace, sample)
    sim.advect_velocity(dt, trace, sample)
    want_phi = orc.advect_collocated(phi, u, v, w, dx, dt, trace, sample)
    wu, wv, ww = orc.advect_staggered(u, v, w, dx, dt, trace, sample)
    assert rel_err(sim.download("phi"), want_phi) <= tol
    assert rel_err(sim.download("u"), wu) <= tol
    assert rel_err(sim.download("v"), wv) <= tol
    assert rel_err(sim.download("w"), ww) <= tol
    sim.close()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_stateless_advection_operators(el, orc, dtype):
    """el_advect_collocated_grid / el_advect_staggered_grid on caller-owned device memory."""
    torch = pytest.importorskip("torch")
    ni, nj, nk = 20, 18, 14
    dx, phi, u, v, w = smooth_fields(orc, ni, nj, nk, dtype, seed=5)
    dt = float(dtype(0.7) * dtype(dx))
    dev = [torch.from_numpy(a).cuda() for a in (phi, u, v, w)]
    outs = [torch.empty_like(t) for t in dev]
    code = el.EL_F64 if dtype == np.float64 else el.EL_F32
    el.advect_collocated_grid(ni, nj, nk, dx, code, outs[0].data_ptr(), dev[0].data_ptr(), dev[1].data_ptr(),
                              dev[2].data_ptr(), dev[3].data_ptr(), dt, el.TRACE_RK3, el.SAMPLE_WENO6)
    el.advect_staggered_grid(ni, nj, nk, dx, code, [t.data_ptr() for t in outs[1:]],
                             [t.data_ptr() for t in dev[1:]], [t.data_ptr() for t in dev[1:]], dt,
                             el.TRACE_RK2, el.SAMPLE_TRILINEAR)
    torch.cuda.synchronize()
    tol = RTOL_F64 if dtype == np.float64 else RTOL_F32
    tol_weno = RTOL_F64 if dtype == np.float64 else RTOL_F32_WENO
    assert rel_err(outs[0].cpu().numpy(), orc.advect_collocated(phi, u, v, w, dx, dt, 1, 1)) <= tol_weno
    for got, want in zip(outs[1:], orc.advect_staggered(u, v, w, dx, dt, 0, 0)):
        assert rel_err(got.cpu().numpy(), want) <= tol


def test_zero_velocity_is_identity_fp64(el, orc):
    ni = nj = nk = 16
    dx, phi, u, v, w = smooth_fields(orc, ni, nj, nk, np.float64, seed=3)
    sim = make_sim(el, 16, np.float64)
    sim.upload("phi", phi)
    for s in (0, 1):
        sim.advect_level_set(0.01, 0, s)
        assert rel_err(sim.download("phi"), phi) <= 1e-13
    sim.close()


def test_fp32_weno6_close_to_fp64_result(el, orc):
    """The FP32 WENO6 path measured against the FP64 restatement of the same advection."""
    ni, nj, nk = 24, 20, 16
    dx, phi, u, v, w = smooth_fields(orc, ni, nj, nk, np.float64, seed=11)
    dt = 0.9 * dx
    sim = make_sim(el, (ni, nj, nk), np.float32)
    for f, a in (("phi", phi), ("u", u), ("v", v), ("w", w)):
        sim.upload(f, a.astype(np.float32))
    sim.advect_level_set(dt, 0, 1)
    want = orc.advect_collocated(phi, u, v, w, dx, dt, 0, 1)
    assert rel_err(sim.download("phi"), want) <= RTOL_F32_WENO
    sim.close()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("shape", [(72, 40, 36), (67, 33, 26)])
@pytest.mark.parametrize("cells", [0.9, 2.6])
def test_box_copies_match_plain_staging(el, orc, dtype, shape, cells):
    """The tiled kernels with their boxes staged by TMA box copies (advect_tiled = 1; at ni = 72 the
    level set and v, w arrive by copies, at ni = 67 u does, the other arrays by plain loads) against
    the same kernels with plain loads only (advect_tiled = 2): the boxes hold the same clamped
    values, interior and edge tiles alike, so the results are bit-identical, and both match the
    oracle.  Covers WENO6 and trilinear level sets and the velocity."""
    ni, nj, nk = shape
    dx, phi, u, v, w = smooth_fields(orc, ni, nj, nk, dtype, seed=17)
    dt = float(dtype(cells) * dtype(dx))
    results = []
    for tiled in (1, 2):
        sim = make_sim(el, shape, dtype)
        sim.set_tuning(advect_tiled=tiled)
        out = {}
        for trace, sample in ((0, 1), (1, 0)):
            for f, a in (("phi", phi), ("u", u), ("v", v), ("w", w)):
                sim.upload(f, a)
            sim.advect_level_set(dt, trace, sample)
            sim.advect_velocity(dt, 1 - trace, 0)
            for f in ("phi", "u", "v", "w"):
                out[(trace, sample, f)] = sim.download(f)
        results.append(out)
        sim.close()
    for key in results[0]:
        np.testing.assert_array_equal(results[0][key], results[1][key], err_msg=str(key))
    tol = RTOL_F64 if dtype == np.float64 else RTOL_F32
    tol_weno = RTOL_F64 if dtype == np.float64 else RTOL_F32_WENO
    for trace, sample in ((0, 1), (1, 0)):
        want = orc.advect_collocated(phi, u, v, w, dx, dt, trace, sample)
        assert rel_err(results[0][(trace, sample, "phi")], want) <= (tol_weno if sample else tol)
        for f, wf in zip(("u", "v", "w"), orc.advect_staggered(u, v, w, dx, dt, 1 - trace, 0)):
            assert rel_err(results[0][(trace, sample, f)], wf) <= tol
