"""Launch-shape autotuning for batches of scenes, with a JSON cache.

A batch runs one graph per sub-step in which every scene's kernels are a separate branch, so the
best launch shapes depend on the whole mix of scene sizes, not on one scene: small grids want
fewer resident blocks per kernel so that the branches share the SMs, large ones want the whole
machine.  ``tune_batch`` times a handful of candidate shapes (el_tuning) on the batch itself,
restoring the scenes' fields between candidates so that every candidate advances the same
state, applies the fastest and records it under a key made of the device name, the scene sizes
and the step parameters.  A later call with the same key applies the cached shapes at once.

The search is one pass of coordinate descent from the default shapes: each parameter in turn
swept over its range with the others held at the best found so far (about a dozen trials).

Cache file: $EL_GB300_TUNING_CACHE, else ``tuning/batch_tuning.json`` beside this module.
"""

import hashlib
import json
import os
import time

HERE = os.path.dirname(os.path.abspath(__file__))

# (seg_blocks_per_sm, stencil_blocks_per_sm, extrapolate_blocks_per_sm, advect_rows, advect_tiled,
#  solver_tiles, coarse_fused, dependent_launch)
DEFAULT = (8, 16, 12, 4, 1, 1, 0, 1)
RANGES = ((1, 2, 3, 4, 6, 8), (2, 4, 8, 16), (4, 8, 12, 16), (2, 4, 8), (1, 0), (1, 0), (0, 1, 2), (1, 0))
STATE_FIELDS = ("phi", "u", "v", "w", "valid_u", "valid_v", "valid_w")


def cache_path():
    return os.environ.get("EL_GB300_TUNING_CACHE", os.path.join(HERE, "tuning", "batch_tuning.json"))


def _as_tuning(c):
    c = tuple(c) + DEFAULT[len(c):]  # shorter (older) entries take the defaults for the rest
    return {"seg_blocks_per_sm": c[0], "stencil_blocks_per_sm": c[1], "extrapolate_blocks_per_sm": c[2],
            "advect_rows": c[3], "advect_tiled": c[4], "solver_tiles": c[5], "coarse_fused": c[6],
            "dependent_launch": c[7]}


def batch_key(device_name, sims, params, cfl, dt_frame):
    sizes = sorted((s.ni, s.nj, s.nk) for s in sims)
    p = (params.trace_phi, params.sample_phi, params.trace_vel, params.sample_vel, params.extrapolation_layers,
         params.solve.solver, params.solve.tol, params.solve.max_outer, params.solve.inner_floor, cfl, dt_frame)
    digest = hashlib.sha1(json.dumps([sizes, p]).encode()).hexdigest()[:16]
    return f"{device_name}|{len(sims)} scenes|{digest}"


def _load():
    path = cache_path()
    if os.path.exists(path):
        try:
            return json.load(open(path))
        except (OSError, ValueError):
            return {}
    return {}


def _save(cache):
    path = cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + f".{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def apply(sims, cand):
    for s in sims:
        s.set_tuning(**_as_tuning(cand))


def tune_batch(el, sims, params, cfl=1.0, dt_frame=1.0 / 60.0, device_name="cuda", steps=3, candidates=None,
               use_cache=True):
    """Pick launch shapes for a batch of ``sims`` (Simulator objects, not in a batch yet).

    Returns {"tuning": {...}, "cached": bool, "trials": {label: ms per sub-step}}; the chosen
    shapes are applied to every scene.  Each candidate: restore the scenes, capture a batch,
    one untimed sub-step, then ``steps`` timed sub-steps (host clock around a synchronised
    run; the graph launches are back to back)."""
    key = batch_key(device_name, sims, params, cfl, dt_frame)
    cache = _load() if use_cache else {}
    if key in cache:
        cand = tuple(cache[key]["tuning"])
        apply(sims, cand)
        return {"tuning": _as_tuning(cand), "cached": True, "trials": cache[key].get("trials", {}), "key": key}
    saved = [{f: s.download(f) for f in STATE_FIELDS} for s in sims]

    def restore():
        for s, d in zip(sims, saved):
            for f, a in d.items():
                s.upload(f, a)

    trials = {}

    def trial(cand):
        label = ",".join(map(str, cand))
        if label not in trials:
            apply(sims, cand)
            restore()
            b = el.Batch(sims, params=params, cfl=cfl, dt_frame=dt_frame)
            try:
                b.step(1)
                b.sync()
                t0 = time.perf_counter()
                b.step(steps)
                b.sync()
                trials[label] = (time.perf_counter() - t0) * 1e3 / steps
            finally:
                b.close()
        return trials[label]

    if candidates:
        for cand in candidates:
            trial(tuple(cand))
        best = min(trials, key=trials.get)
        cand = tuple(int(x) for x in best.split(","))
    else:
        cand = DEFAULT
        for axis, values in enumerate(RANGES):
            options = [cand[:axis] + (v,) + cand[axis + 1:] for v in values]
            cand = min(options, key=trial)
    apply(sims, cand)
    restore()
    if use_cache:
        cache = _load()
        cache[key] = {"tuning": list(cand), "trials": trials, "ms_per_step": trials[",".join(map(str, cand))]}
        _save(cache)
    return {"tuning": _as_tuning(cand), "cached": False, "trials": trials, "key": key}
