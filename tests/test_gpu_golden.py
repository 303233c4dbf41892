"""CUDA path against the golden fixtures made from the reference itself.

Each scene runs several whole update() calls from the zero state with the PCG
pinned to the reference's own per-step iteration counts; the final fields
must then agree to 1e-9 relative (what remains is FP64 rounding of the
parallel dot products, carried through the steps).  Unpinned, the counts
agree within one iteration (test_gpu_parity.py).  Steps 1-2 (Gauss-Seidel,
no reductions) must reproduce the reference's sweep counts and fields
exactly, unpinned."""
import glob
import importlib.util
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def _scenes():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return {s[0]: s for s in mod.SCENES}


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_gpu_fp64_matches_golden(ifl, path):
    name = os.path.basename(path)[:-4]
    _, variant, w, h, dt, steps, inflow, bodies = _scenes()[name]
    g = np.load(path)
    objs = []
    for b in bodies:
        objs.append(ifl.SolidBox(*b[1:]) if b[0] == 0 else ifl.SolidSphere(b[1], b[2], b[3], *b[5:]))
    if variant <= 3:
        s = ifl.FluidSolver(w, h, 0.1, variant=variant)
    elif variant in (4, 5):
        s = ifl.FluidSolver(w, h, 0.1, objs, variant=variant)
    else:
        s = ifl.FluidSolver(w, h, 0.1, 1.0, 0.01, objs, variant=variant)
    ref_iters = g["iters"]
    exact = variant <= 2  # Gauss-Seidel: an exact wavefront, no reduction-order rounding
    capped = not exact and (ref_iters[:, 1] == 2).any()
    iters = []
    for step in range(steps):
        if not capped and not exact:
            # run exactly the reference's iteration counts: no termination flips,
            # so the remaining differences are rounding only
            s.set_pinned_iterations(int(ref_iters[step, 0]), int(ref_iters[step, 2]))
        if variant >= 6:
            s.addInflow(*inflow)
        else:
            s.addInflow(*inflow[:5], *inflow[6:])
        s.update(dt)
        for b in objs:
            b.update(dt)
        (pi, ps, _), (hi, hs, _), flags = s.stats()
        assert flags & 1 == 0
        iters.append((pi, ps))
    if exact:
        assert [tuple(r) for r in ref_iters[:, :2]] == iters
        for key in ("d", "u", "v", "p"):
            assert np.array_equal(s.read_field(key), g[key]), key
        return
    if capped:
        # 2000 iterations of a stagnating solve amplify rounding; only the outcome is compared
        assert all(st == 2 for _, st in iters)
        return
    fluid = np.ones_like(g["p"], dtype=bool)
    if variant >= 4:  # p at solid cells holds stale values nothing reads
        fluid = s.read_field(ifl.field_id(ifl.Q_D, ifl.A_CELL), np.uint8) == 0
    for key in ("d", "t", "u", "v", "p"):
        if key in g:
            a, b = s.read_field(key), g[key]
            if key == "p":
                a, b = a[fluid], b[fluid]
            assert np.abs(a - b).max() <= 1e-9 * max(np.abs(b).max(), 1e-300), key
    if variant == 8:  # FLIP particles: same count, positions to 1e-9 cells, carried values 1e-8
        assert s.particle_count() == int(g["np"][-1])
        for k, key in enumerate(("px", "py", "pd", "pt", "pu", "pv")):
            a, b = s.particles(k), g[key]
            tol = 1e-9 if k < 2 else 1e-8 * max(np.abs(b).max(), 1e-300)
            assert np.abs(a - b).max() <= tol, key
