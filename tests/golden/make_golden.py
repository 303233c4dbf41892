"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own FluidSolver (each tutorial step's Fluid.cpp compiled
unmodified by oracle/Makefile into oracle/_ref/) on small seeded scenes and
stores the final fields, the pressure and the per-step PCG iteration counts.
The fixtures travel with the repository, so the oracle restatement and the GPU
path can be checked against reference outputs where the reference source is
not available.

    make -C oracle ref && python tests/golden/make_golden.py [scene ...]

Step 8 (FLIP) also stores the particles and their count after every step;
its reference keeps the frand() seed in a static, so at most one step-8 scene
runs per process (here: one).  Its update() adds a fixed inflow, which the
scene's inflow tuple repeats for the other side.
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

BOX = (0, 0.5, 0.6, 0.7, 0.1, math.pi * 0.25, 0.0, 0.0, 0.0)
SPIN = (0, 0.62, 0.6, 0.3, 0.12, 0.3, 0.0, 0.0, 1.5)
PINCH = (0, 0.45, 0.55, 0.3, 0.12, 0.3, 0.0, 0.0, 1.5)
BALL = (1, 0.3, 0.45, 0.2, 0.2, 0.0, 0.05, 0.0, 0.8)

# name, variant, w, h, dt, steps, inflow (x, y, w, h, d, t, u, v), bodies
SCENES = [
    ("gs1_32", 1, 32, 32, 0.005, 6, (0.45, 0.2, 0.1, 0.05, 1.0, 0.0, 0.0, 3.0), []),
    ("gs2_32", 2, 32, 32, 0.005, 6, (0.45, 0.2, 0.15, 0.03, 1.0, 0.0, 0.0, 3.0), []),
    ("plain_32", 3, 32, 32, 0.005, 6, (0.45, 0.2, 0.15, 0.03, 1.0, 0.0, 0.0, 3.0), []),
    ("plain_40x24", 3, 40, 24, 0.005, 6, (0.3, 0.2, 0.3, 0.1, 1.0, 0.0, 0.5, 3.0), []),
    ("solid_32", 4, 32, 32, 0.005, 6, (0.45, 0.2, 0.15, 0.06, 1.0, 0.0, 0.0, 3.0), [SPIN, BALL]),
    # bodies that pinch off fluid cells: the PCG runs into its 2000-iteration cap
    ("solid_cap_32", 4, 32, 32, 0.005, 2, (0.45, 0.2, 0.15, 0.06, 1.0, 0.0, 0.0, 3.0), [PINCH, BALL]),
    ("solid_24x40", 4, 24, 40, 0.005, 6, (0.3, 0.2, 0.4, 0.1, 1.0, 0.0, 0.0, 3.0), [BALL]),
    ("curved_32", 5, 32, 32, 0.005, 6, (0.45, 0.2, 0.15, 0.06, 1.0, 0.0, 0.0, 3.0), [BOX]),
    ("heat_32", 6, 32, 32, 0.005, 6, (0.35, 0.2, 0.2, 0.1, 1.0, 594.0, 0.0, 0.0), [BOX]),
    ("vardens_32", 7, 32, 32, 0.005, 6, (0.45, 0.2, 0.1, 0.1, 1.0, 700.0, 0.0, 0.0), [BOX]),
    ("flip_32", 8, 32, 32, 0.0025, 4, (0.45, 0.2, 0.2, 0.05, 1.0, 294.0, 0.0, 0.0), [BOX]),
]
PARTICLE_KEYS = ("px", "py", "pd", "pt", "pu", "pv")


def run_reference(variant, w, h, dt, steps, inflow, bodies):
    s = O.RefSolver(variant, w, h)
    if bodies:
        s.set_bodies(bodies)
    iters, counts = [], []
    for _ in range(steps):
        s.add_inflow(*inflow)
        s.update(dt)
        s.advance_bodies(dt)
        pr, ht = s.stats()
        iters.append((pr[0], pr[1], ht[0], ht[1]))
        if variant == O.FLIP:
            counts.append(s.particle_count())
    out = {"iters": np.array(iters, dtype=np.int64), "p": s.array(0, O.A_P).copy()}
    if variant == O.FLIP:
        out["np"] = np.array(counts, dtype=np.int64)
        for k, key in enumerate(PARTICLE_KEYS):
            out[key] = s.particles(k).copy()
    for name, q in (("d", O.QD), ("t", O.QT), ("u", O.QU), ("v", O.QV)):
        a = s.array(q, O.A_SRC)
        if a is not None:
            out[name] = a.copy()
    return out


def main():
    only = set(sys.argv[1:])
    for name, variant, w, h, dt, steps, inflow, bodies in SCENES:
        if only and name not in only:
            continue
        if not O.ref_available(variant):
            raise SystemExit(f"reference step {variant} not built: make -C oracle ref")
        out = run_reference(variant, w, h, dt, steps, inflow, bodies)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(name, out["iters"][:, 0].tolist())


if __name__ == "__main__":
    main()
