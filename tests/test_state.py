"""State files (el_state_save / el_state_load): the host-side format on CPU, and on the GPU an
exact restart -- a scene saved after some steps, loaded into a fresh context and stepped on,
must match the original run bit for bit."""

import numpy as np
import pytest

import conftest


def _pkg():
    return conftest.load_package()


def test_state_format_round_trip_on_host(tmp_path):
    S = _pkg().state
    rng = np.random.default_rng(0)
    ni, nj, nk = 5, 4, 3
    fields = {"phi": rng.standard_normal((nk, nj, ni)).astype(np.float32),
              "u": rng.standard_normal((nk, nj, ni + 1)).astype(np.float32),
              "valid_w": (rng.uniform(size=(nk + 1, nj, ni)) < 0.5).astype(np.uint8),
              "solid_nodal": rng.standard_normal((nk + 1, nj + 1, ni + 1)).astype(np.float32)}
    path = tmp_path / "s.elstate"
    S.write_state(path, ni, nj, nk, 0.2, 0, fields, time=1.25)
    d = S.read_state(path)
    assert (d["ni"], d["nj"], d["nk"], d["dx"], d["time"], d["dtype"]) == (ni, nj, nk, 0.2, 1.25, 0)
    assert set(d["fields"]) == set(fields)
    for k, a in fields.items():
        assert np.array_equal(d["fields"][k], a) and d["fields"][k].dtype == a.dtype
    raw = path.read_bytes()
    assert raw[:8] == b"ELGBSTAT" and len(raw) == 64 + sum(16 + a.nbytes for a in fields.values())
    (tmp_path / "bad").write_bytes(b"NOTSTATE" + raw[8:])
    with pytest.raises(ValueError):
        S.read_state(tmp_path / "bad")
    (tmp_path / "short").write_bytes(raw[:100])
    with pytest.raises(ValueError):
        S.read_state(tmp_path / "short")


@pytest.mark.gpu
@pytest.mark.parametrize("dtype_name", ["EL_F32", "EL_F64"])
def test_restart_from_state_is_exact(el, tmp_path, dtype_name):
    dtype = getattr(el, dtype_name)
    n = 24
    spec = el.scenes.spheres_pool(n, 2)
    prm = el.step_params(sample_phi=el.SAMPLE_WENO6, trace_vel=el.TRACE_RK3, solver=el.SOLVER_MIXED, tol=1e-8,
                         max_iter=500)
    a = el.Simulator(n, n, n, dtype=dtype)
    a.init_scene(spec)
    for _ in range(3):
        a.step(min(a.calc_time_step(1.0), 1 / 60), prm)
    path = str(tmp_path / "scene.elstate")
    a.save_state(path, time=0.5)
    # the file is what the host reader sees and what the context holds
    d = el.state.read_state(path)
    assert d["time"] == 0.5 and d["dtype"] == dtype and (d["ni"], d["nj"], d["nk"]) == (n, n, n)
    for name, arr in d["fields"].items():
        assert np.array_equal(arr, a.download(name)), name
    b = el.Simulator(n, n, n, dtype=dtype)
    assert b.load_state(path) == 0.5
    for _ in range(2):
        dt = min(a.calc_time_step(1.0), 1 / 60)
        assert dt == min(b.calc_time_step(1.0), 1 / 60)
        sa, sb = a.step(dt, prm), b.step(dt, prm)
        assert sa["iterations"] == sb["iterations"]
    for name in ("phi", "u", "v", "w", "pressure", "valid_u", "valid_v", "valid_w"):
        assert np.array_equal(a.download(name), b.download(name)), name
    # a file for another grid or field type is refused and changes nothing
    c = el.Simulator(n, n, n + 8, dtype=dtype)
    with pytest.raises(el.ELError):
        c.load_state(path)
    for s in (a, b, c):
        s.close()
