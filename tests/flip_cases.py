"""Step 8 (FLIP) scenes shared by the oracle pins and the GPU parity tests.

* SCENES: the reference's own main() scene (8-flip/Fluid.cpp:1475-1512: a
  rotated box, rhoAir 0.1, rhoSoot 0.25, diffusion 0.01, dt 0.0025, the
  inflow update() adds itself) at small sizes, plus a moving sphere and a
  body-free case.
* crafted(): a particle state that makes every order-dependent branch of the
  particle step run - cells with more than 12 particles (prune), holes that
  leave grid nodes without weight (CELL_EMPTY cells with and without fluid
  neighbours, on the outer ring and beside the body) and thin cells (seeding).
"""
import math

import numpy as np

BOX = (0, 0.5, 0.6, 0.7, 0.1, math.pi * 0.25, 0.0, 0.0, 0.0)
BALL = (1, 0.35, 0.45, 0.18, 0.18, 0.0, 0.08, 0.02, 0.9)
INFLOW = (0.45, 0.2, 0.2, 0.05, 1.0, 294.0, 0.0, 0.0)  # 8-flip/Fluid.cpp:1368
RHO_AIR, RHO_SOOT, DIFFUSION, DT = 0.1, 0.25, 0.01, 0.0025

# name, w, h, bodies, steps
SCENES = [
    ("main_48", 48, 48, [BOX], 4),
    ("ball_56x40", 56, 40, [BALL], 4),  # h <= w + 2: step 7-8 index v-face densities with the u width
    ("open_32x24", 32, 24, [], 4),
]


def crafted(w, h, x, y, seed=7):
    """(x, y, d, t, u, v) particle arrays built from initial positions x, y."""
    rng = np.random.default_rng(seed)
    cx, cy = np.floor(x).astype(int), np.floor(y).astype(int)
    bx, by = int(0.5 * w), int(0.6 * h)
    holes = (
        ((cx >= w // 4) & (cx < w // 4 + 5) & (cy >= h // 3) & (cy < h // 3 + 5))  # interior 5x5
        | ((cx < 3) & (cy < 3))                                                    # corner
        | ((cx >= w - 4) & (cy >= h // 2) & (cy < h // 2 + 3))                     # right ring
        | ((cx >= bx - 2) & (cx < bx + 3) & (cy >= by + 2) & (cy < by + 6))        # beside the body
    )
    x, y = x[~holes], y[~holes]
    extra_x, extra_y = [], []
    for ccx, ccy, k in ((3 * w // 4, h // 4, 18), (w - 1, h - 1, 15), (w // 2, 2, 14), (1, h // 2, 13)):
        extra_x.append(ccx + rng.random(k))
        extra_y.append(ccy + rng.random(k))
    x = np.concatenate([x] + extra_x)
    y = np.concatenate([y] + extra_y)
    perm = rng.permutation(len(x))
    x, y = x[perm], y[perm]
    n = len(x)
    assert n >= w * h, "seeding tests particle number `cell index`: keep more particles than cells"
    d = rng.random(n)
    t = 294.0 + 60.0 * rng.random(n)
    u = rng.normal(0.0, 0.4, n)
    v = rng.normal(0.0, 0.4, n)
    return x, y, d, t, u, v
