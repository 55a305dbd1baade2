"""Seeded scene specifications for the benchmark and parity workloads.

A scene is a list of liquid emitters (composed with ``min`` exactly like
``LevelSetEmitterList::apply``, src/project/3d/fluid/levelset_emitter.cpp:74-79) and a list of
solid emitters applied to the nodal solid level set.  Only parameters are produced here; the
fields themselves are rasterised on the GPU by ``el_emit_*`` (and, for checking, by the CPU
oracle).

Emitters:
  ("sphere", cx, cy, cz, r)     signed distance to a sphere (levelset_emitter.cpp:10-12)
  ("pool", h)                   y - h (levelset_emitter.cpp:14-16)
  ("box", lo3, hi3)             exact signed distance to an axis-aligned box; +-inf bounds
                                make a slab or quarter space (new: the reference has no box)
  ("room",)                     nodal wall layers -1 / -0.01 / +1 (levelset_emitter.cpp:18-32)

Workloads (unit cube, dx = 1/ni):
  dam_break(n)       box {x<0.4, y<0.5} and sphere c=(0.7,0.75,0.5) r=0.12, room walls.
  spheres_pool(n, seed)  pool y<0.3 and 3 seeded spheres r in [0.08,0.2], room walls and a
                     seeded solid box holding 5-10 % of the cells.
  water_drop(n)      the reference's own scene: 3 spheres r=0.16 and a pool y<0.25
                     (apps/eulerian_liquid_3d.cpp:49-68).
"""

import math

import numpy as np

INF = math.inf


def dam_break(n):
    return {
        "name": f"dam_break_{n}",
        "shape": (n, n, n),
        "liquid": [("box", (-INF, -INF, -INF), (0.4, 0.5, INF)),
                   ("sphere", 0.7, 0.75, 0.5, 0.12)],
        "solid": [("room",)],
    }


def water_drop(n):
    return {
        "name": f"water_drop_{n}",
        "shape": (n, n, n),
        "liquid": [("sphere", 0.25, 0.6, 0.25, 0.16), ("sphere", 0.5, 0.5, 0.5, 0.16),
                   ("sphere", 0.75, 0.7, 0.75, 0.16), ("pool", 0.25)],
        "solid": [("room",)],
    }


def spheres_pool(n, seed):
    rng = np.random.default_rng(seed)
    liquid = [("pool", 0.3)]
    for _ in range(3):
        r = float(rng.uniform(0.08, 0.2))
        c = [float(rng.uniform(0.1 + r, 0.9 - r)) for _ in range(3)]
        c[1] = float(rng.uniform(0.35 + r, 0.9 - r))
        liquid.append(("sphere", c[0], c[1], c[2], r))
    frac = float(rng.uniform(0.05, 0.10))
    sx = float(rng.uniform(0.3, 0.6))
    sz = float(rng.uniform(0.3, 0.6))
    sy = frac / (sx * sz)
    lo = [float(rng.uniform(0.08, 0.92 - sx)), float(rng.uniform(0.08, 0.92 - sy)),
          float(rng.uniform(0.08, 0.92 - sz))]
    hi = [lo[0] + sx, lo[1] + sy, lo[2] + sz]
    return {
        "name": f"spheres_pool_{n}_s{seed}",
        "shape": (n, n, n),
        "liquid": liquid,
        "solid": [("room",), ("box", tuple(lo), tuple(hi))],
        "solid_fraction": frac,
    }


def batch_scenes(count, seed, lo=48, hi=160):
    """Independent scenes with seeded sizes in {lo..hi} per axis and fill fractions 0.2-0.6."""
    rng = np.random.default_rng(seed)
    scenes = []
    for s in range(count):
        ni, nj, nk = (int(rng.integers(lo, hi + 1)) for _ in range(3))
        fill = float(rng.uniform(0.2, 0.6))
        if rng.uniform() < 0.5:  # dam break with fill-controlled height
            liquid = [("box", (-INF, -INF, -INF), (0.5, min(0.95, 2 * fill), INF))]
        else:  # sphere drop over a pool
            r = 0.12
            liquid = [("pool", max(0.05, fill - 0.05)), ("sphere", 0.5, min(0.85, fill + 0.25), 0.5, r)]
        scenes.append({"name": f"batch_{s}", "shape": (ni, nj, nk), "liquid": liquid,
                       "solid": [("room",)], "fill": fill})
    return scenes
