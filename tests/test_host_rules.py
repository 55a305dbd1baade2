"""Host-side rules that need no GPU: the roofline's choice of kernel class in bench.py and the
launch-shape autotuner's defaults and cache key."""

import importlib.util
import os
import sys
import types

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _autotune():
    spec = importlib.util.spec_from_file_location("el_autotune",
                                                  os.path.join(ROOT, "eulerian-liquid_gb300", "autotune.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _rec(launches, ms):
    return {"launches": launches, "ms": ms, "bytes": 1e9}


def test_roofline_class_skips_grouped_and_short_launches():
    breakdown = {
        "extrapolate": _rec(8, 4.6),        # records time groups of kernels: never the roofline's
        "mg_coarse": _rec(426, 5.4),        # 12.7 us per launch: event overhead dominates
        "mg_smooth_fine": _rec(96, 4.2),    # 44 us per launch
        "advect_phi": _rec(2, 3.6),
        "update": _rec(28, 0.9),
    }
    assert bench.dominant_class(breakdown, fine_solver_on=False) == "mg_smooth_fine"
    # with the finest level on the tile kernels, its four classes are one kernel
    assert bench.dominant_class(breakdown) == bench.FINE_SOLVER
    merged = bench.with_fine_solver(breakdown)[bench.FINE_SOLVER]
    assert merged["launches"] == 124 and abs(merged["ms"] - 5.1) < 1e-12
    assert bench.class_mask(bench.FINE_SOLVER) == sum(1 << bench.KC_NAMES.index(k)
                                                      for k in bench.FINE_SOLVER_CLASSES)


def test_roofline_class_falls_back_to_the_largest():
    breakdown = {"extrapolate": _rec(8, 4.6), "mg_coarse": _rec(400, 5.0)}
    assert bench.dominant_class(breakdown) == "mg_coarse"


def test_ncu_traffic_is_per_launch_and_named_for_a_single_kernel_class():
    for cls, traffic in bench.NCU_TRAFFIC_PER_LAUNCH.items():
        assert cls in bench.SINGLE_KERNEL_CLASSES or cls == bench.FINE_SOLVER
        assert 1e6 < traffic < 1e10


def test_autotune_defaults_and_cache_key():
    at = _autotune()
    # an older, shorter cache entry takes the current defaults for the missing parameters
    t = at._as_tuning((4, 2))
    assert t["seg_blocks_per_sm"] == 4 and t["stencil_blocks_per_sm"] == 2
    assert t["extrapolate_blocks_per_sm"] == at.DEFAULT[2] and t["advect_tiled"] == at.DEFAULT[4]
    # the defaults lie inside the searched ranges
    for value, values in zip(at.DEFAULT, at.RANGES):
        assert value in values
    solve = types.SimpleNamespace(solver=2, tol=1e-6, max_outer=8, inner_floor=1e-4)
    params = types.SimpleNamespace(trace_phi=0, sample_phi=1, trace_vel=1, sample_vel=0, extrapolation_layers=10,
                                   solve=solve)
    scenes = [types.SimpleNamespace(ni=48, nj=64, nk=80), types.SimpleNamespace(ni=96, nj=96, nk=96)]
    k1 = at.batch_key("GB300", scenes, params, 1.0, 1 / 60)
    k2 = at.batch_key("GB300", list(reversed(scenes)), params, 1.0, 1 / 60)
    assert k1 == k2  # the scene order does not matter
    scenes[0].ni = 50
    assert at.batch_key("GB300", scenes, params, 1.0, 1 / 60) != k1
    assert at.batch_key("other GPU", list(reversed(scenes)), params, 1.0, 1 / 60) != k1
