"""The C oracle against the reference (CPU only).

* Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py
  from the reference's own sources) must be reproduced bit-for-bit.  This runs
  wherever the oracle builds, including hosts without the reference.
* Where the reference compiled in place is available (oracle/_ref), every
  array of every step must match bit-for-bit, including stale solid-cell
  values of the advection buffers and the PCG iteration counts.
"""
import glob
import math
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def _golden_scenes():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return {s[0]: s for s in mod.SCENES}


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_reproduces_golden(path):
    name = os.path.basename(path)[:-4]
    _, variant, w, h, dt, steps, inflow, bodies = _golden_scenes()[name]
    g = np.load(path)
    s = O.OracleSolver(variant, w, h)
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
    assert np.array_equal(np.array(iters), g["iters"])
    for key, q in (("d", O.QD), ("t", O.QT), ("u", O.QU), ("v", O.QV)):
        if key in g:
            assert np.array_equal(s.array(q, O.A_SRC), g[key]), key
    assert np.array_equal(s.array(0, O.A_P), g["p"])
    if variant == O.FLIP:
        assert counts == list(g["np"])
        for k, key in enumerate(("px", "py", "pd", "pt", "pu", "pv")):
            assert np.array_equal(s.particles(k), g[key]), key


BOX = (0, 0.5, 0.6, 0.7, 0.1, math.pi * 0.25, 0.0, 0.0, 0.0)
SPIN = (0, 0.55, 0.55, 0.3, 0.12, 0.7, 0.0, 0.0, 1.0)
BALL = (1, 0.3, 0.45, 0.2, 0.2, 0.0, 0.1, 0.0, 1.0)

STEPWISE = [
    (1, 48, 40, 5, (0.45, 0.2, 0.1, 0.05, 1.0, 0.0, 0.0, 3.0), []),    # Gauss-Seidel, Euler + lerp
    (1, 128, 128, 3, (0.45, 0.2, 0.1, 0.01, 1.0, 0.0, 0.0, 3.0), []),  # 1-matrixless main() scene
    (2, 40, 56, 5, (0.45, 0.2, 0.15, 0.03, 1.0, 0.0, 0.0, 3.0), []),   # Gauss-Seidel, RK3 + cerp
    (3, 48, 48, 6, (0.45, 0.2, 0.15, 0.03, 1.0, 0.0, 0.0, 3.0), []),
    (3, 40, 56, 6, (0.45, 0.2, 0.15, 0.03, 1.0, 0.0, 0.5, 3.0), []),
    (3, 56, 36, 6, (0.2, 0.2, 0.6, 0.1, 1.0, 0.0, -1.0, 2.0), []),  # wide rectangle on a wide grid
    (4, 48, 48, 6, (0.45, 0.2, 0.15, 0.05, 1.0, 0.0, 0.0, 3.0), [SPIN, BALL]),
    (4, 36, 52, 6, (0.3, 0.2, 0.6, 0.05, 1.0, 0.0, 0.0, 3.0), [BALL]),  # x bound uses h > w (wrap)
    (5, 48, 48, 5, (0.45, 0.2, 0.15, 0.05, 1.0, 0.0, 0.0, 3.0), [BOX]),
    (6, 48, 48, 5, (0.35, 0.2, 0.2, 0.1, 1.0, 594.0, 0.0, 0.0), [BOX]),
    (7, 48, 48, 5, (0.45, 0.2, 0.1, 0.1, 1.0, 700.0, 0.0, 0.0), [BOX]),
    (7, 48, 44, 5, (0.45, 0.2, 0.1, 0.1, 1.0, 700.0, 0.0, 0.0), [BOX]),
]


@pytest.mark.skipif(not all(O.ref_available(v) for v in (1, 2, 3, 4, 5, 6, 7)),
                    reason="reference not compiled here (make -C oracle ref)")
@pytest.mark.parametrize("case", STEPWISE, ids=[f"v{c[0]}-{c[1]}x{c[2]}" for c in STEPWISE])
def test_oracle_matches_reference_every_step(case):
    variant, w, h, steps, inflow, bodies = case
    a, b = O.OracleSolver(variant, w, h), O.RefSolver(variant, w, h)
    if bodies:
        a.set_bodies(bodies)
        b.set_bodies(bodies)
    qs = [O.QD, O.QU, O.QV] + ([O.QT] if variant >= O.HEAT else [])
    for step in range(steps):
        for s in (a, b):
            s.add_inflow(*inflow)
            s.update(0.005)
            s.advance_bodies(0.005)
        assert a.stats() == b.stats(), step
        for q in qs:
            for which in (O.A_SRC, O.A_DST):
                assert np.array_equal(a.array(q, which), b.array(q, which)), (step, q, which)
            if variant >= O.SOLID:
                assert np.array_equal(a.bytes(q, O.B_CELL), b.bytes(q, O.B_CELL))
                assert np.array_equal(a.array(q, O.A_NORMALX), b.array(q, O.A_NORMALX))
            if variant >= O.CURVED:
                assert np.array_equal(a.array(q, O.A_VOLUME), b.array(q, O.A_VOLUME))
        solver_arrays = (O.A_R, O.A_P) + ((O.A_PRECON, O.A_ADIAG, O.A_APLUSX, O.A_APLUSY)
                                          if variant >= O.PLAIN else ())
        for which in solver_arrays:
            assert np.array_equal(a.array(0, which), b.array(0, which)), (step, which)
        if variant == O.VARDENS:
            assert np.array_equal(a.array(0, O.A_UDENS), b.array(0, O.A_UDENS))
            assert np.array_equal(a.array(0, O.A_VDENS), b.array(0, O.A_VDENS))
        for heat in ((False, True) if variant >= O.HEAT else (False,)):
            assert np.array_equal(a.to_image(heat), b.to_image(heat)), (step, heat)


def test_config0_as_stated_injects_nothing():
    """The stated config-0 rectangle deposits nothing at 128^2 (its one row's centre is outside)."""
    s = O.OracleSolver(3, 128, 128)
    for _ in range(3):
        s.add_inflow(0.45, 0.20, 0.10, 0.01, 1.0, 0.0, 0.0, 3.0)
        s.update(0.005)
        assert s.stats()[0][1] == O.PCG_INITIAL
    assert not s.array(O.QD, O.A_SRC).any()


def test_pinned_iterations():
    s = O.OracleSolver(3, 32, 32)
    s.set_pinned_iterations(7, -1)
    s.add_inflow(0.45, 0.2, 0.15, 0.03, 1.0, 0.0, 0.0, 3.0)
    s.update(0.005)
    assert s.stats()[0][0] == 7
