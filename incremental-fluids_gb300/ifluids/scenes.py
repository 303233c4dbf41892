"""Seeded synthetic scenes with the shapes of the benchmark configurations.

No public dataset is involved: every scene is generated from a seed with the
sizes, rectangles and body distributions the configurations state, with the
reference mains' constants where a configuration leaves one open
(3-conjugate-gradients/Fluid.cpp:470-485, 4-solid-boundaries/Fluid.cpp:921-948,
7-variable-density/Fluid.cpp:1086-1112).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Tuple

import numpy as np

# Body tuple: (type, pos_x, pos_y, scale_x, scale_y, theta, vel_x, vel_y, vel_theta);
# type 0 = box (full side lengths), 1 = sphere (diameter in scale_x).
Body = Tuple[int, float, float, float, float, float, float, float, float]
# Inflow: (x, y, w, h, d, t, u, v)
Inflow = Tuple[float, float, float, float, float, float, float, float]


@dataclass
class Scene:
    name: str
    variant: int
    w: int
    h: int
    dt: float
    steps: int
    inflows: List[Inflow]
    bodies: List[Body] = field(default_factory=list)
    density: float = 0.1
    density_soot: float = 1.0
    diffusion: float = 0.01

    @property
    def cells(self) -> int:
        return self.w * self.h


def config0(n: int = 128, steps: int = 100) -> Scene:
    """Plain FP64 step-3 scene: rectangle x in [0.45,0.55], y in [0.20,0.21] (injects nothing at 128^2)."""
    return Scene("c0-plain", 3, n, n, 0.005, steps, [(0.45, 0.20, 0.10, 0.01, 1.0, 0.0, 0.0, 3.0)])


def config0b(n: int = 128, steps: int = 100) -> Scene:
    """Config 0 with the reference main's own rectangle (0.45, 0.2, 0.15, 0.03)."""
    return Scene("c0b-plain", 3, n, n, 0.005, steps, [(0.45, 0.2, 0.15, 0.03, 1.0, 0.0, 0.0, 3.0)])


def _reach(b: Body) -> float:
    """Radius of the circle a body sweeps while it rotates about its centre."""
    return 0.5 * math.hypot(b[3], b[4]) if b[0] == 0 else 0.5 * b[3]


def random_bodies(rng: np.random.Generator, count: int, margin: float = 0.02) -> List[Body]:
    """Boxes and circles: centres U[0.2,0.8]^2, half-sizes U[0.03,0.1], angular velocity U[-2,2].

    Draws are rejected while a body's swept circle comes within `margin` of
    another's.  Two touching bodies that rotate about different centres do not
    move as one rigid body, so the discrete divergence of their solid-face
    velocities no longer sums to zero over the fluid: the pressure system
    becomes inconsistent and the reference's own PCG runs into its iteration
    cap.  Separated bodies keep the scene inside the solver's working range.
    """
    out: List[Body] = []
    while len(out) < count:
        kind = int(rng.integers(0, 2))
        cx, cy = (float(v) for v in rng.uniform(0.2, 0.8, size=2))
        hs = float(rng.uniform(0.03, 0.1))
        hs2 = float(rng.uniform(0.03, 0.1))
        theta = float(rng.uniform(0.0, 2.0 * math.pi))
        omega = float(rng.uniform(-2.0, 2.0))
        if kind == 0:
            b = (0, cx, cy, 2 * hs, 2 * hs2, theta, 0.0, 0.0, omega)
        else:
            b = (1, cx, cy, 2 * hs, 2 * hs, theta, 0.0, 0.0, omega)
        if all(math.hypot(cx - o[1], cy - o[2]) > _reach(b) + _reach(o) + margin for o in out):
            out.append(b)
    return out


def config1(n: int = 1024, steps: int = 200, seed: int = 1, variant: int = 4) -> Scene:
    """Solid-boundary scene: 3 seeded bodies, config-0 rectangle, dt = 0.0025."""
    rng = np.random.default_rng(seed)
    return Scene(f"c1-solid-{n}", variant, n, n, 0.0025, steps,
                 [(0.45, 0.20, 0.10, 0.01, 1.0, 0.0, 0.0, 3.0)], random_bodies(rng, 3))


def config3(n: int = 2048, steps: int = 500) -> Scene:
    """Heat + variable density (step 7): inflow d = 1, T = 700 K, the reference main's box."""
    box = (0, 0.5, 0.6, 0.7, 0.1, math.pi * 0.25, 0.0, 0.0, 0.0)
    return Scene(f"c3-vardens-{n}", 7, n, n, 0.001, steps,
                 [(0.45, 0.2, 0.1, 0.05, 1.0, 700.0, 0.0, 0.0)], [box])


def batch_scenes(count: int = 512, seed: int = 2, lo: int = 64, hi: int = 1024, steps: int = 1) -> List[Scene]:
    """Ragged batch: sides log-uniform in [lo, hi], 1-3 inflow rectangles, 0-4 bodies."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        w = int(math.exp(rng.uniform(math.log(lo), math.log(hi))))
        h = int(math.exp(rng.uniform(math.log(lo), math.log(hi))))
        rects = []
        for _ in range(int(rng.integers(1, 4))):
            x0 = float(rng.uniform(0.1, 0.8))
            rw = float(rng.uniform(0.05, 0.15))
            vv = float(rng.uniform(1.0, 4.0))
            rects.append((x0, 0.2, rw, 0.01, 1.0, 0.0, 0.0, vv))
        bodies = random_bodies(rng, int(rng.integers(0, 5)))
        out.append(Scene(f"batch-{k}", 4, w, h, 0.0025, steps, rects, bodies))
    return out
