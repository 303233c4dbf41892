"""Steps 1-2 (Gauss-Seidel pressure solve) on the GPU against the oracle (needs a GB300).

The Gauss-Seidel sweep runs as an exact wavefront, so nothing in these steps
depends on a parallel reduction order: every phase and every whole update is
required to be bit-identical to the oracle (fields, pressure, sweep counts,
the last maximum change, the image).  The oracle is pinned to the reference's
own step-1 and step-2 code in test_oracle_pin.py.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

# variant, w, h, steps, inflow
CASES = [
    (1, 128, 128, 4, (0.45, 0.2, 0.1, 0.01, 1.0, 0.0, 0.0, 3.0)),   # 1-matrixless main() scene
    (1, 70, 40, 5, (0.3, 0.2, 0.4, 0.1, 1.0, 0.0, 0.5, 3.0)),
    (2, 128, 128, 4, (0.45, 0.2, 0.1, 0.01, 1.0, 0.0, 0.0, 3.0)),   # 2-better-advection main() scene
    (2, 40, 97, 5, (0.3, 0.2, 0.6, 0.05, 1.0, 0.0, 0.0, 3.0)),      # inflow x-range wraps (uses h)
    (2, 33, 300, 3, (0.2, 0.1, 0.6, 0.05, 1.0, 0.0, 0.0, 3.0)),     # 10 strips, last one ragged
]
IDS = [f"v{c[0]}-{c[1]}x{c[2]}" for c in CASES]
DT = 0.005


def _fields(ifl, g, o):
    for q in (O.QD, O.QU, O.QV):
        assert np.array_equal(g.read_field(ifl.field_id(q, ifl.A_SRC)), o.array(q, O.A_SRC)), q
    assert np.array_equal(g.read_field("p"), o.array(0, O.A_P))


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_whole_updates_bit_exact(ifl, case):
    variant, w, h, steps, inflow = case
    o = O.OracleSolver(variant, w, h)
    g = ifl.FluidSolver(w, h, 0.1, variant=variant)
    for step in range(steps):
        o.add_inflow(*inflow)
        g.addInflow(*inflow[:5], *inflow[6:])
        o.update(DT)
        g.update(DT)
        (gi, gs, ge), _, flags = g.stats()
        assert (gi, gs, ge) == o.stats()[0], step     # sweeps, outcome, last maximum change
        assert flags == 0
        _fields(ifl, g, o)
    assert np.array_equal(g.to_image(), o.to_image())


@pytest.mark.parametrize("case", CASES[:3], ids=IDS[:3])
def test_phases_bit_exact_from_the_oracle_state(ifl, case):
    """RHS, Gauss-Seidel solve, applyPressure and advection one at a time, from
    an oracle state after a few steps (p carries over between steps)."""
    variant, w, h, steps, inflow = case
    o = O.OracleSolver(variant, w, h)
    for _ in range(steps):
        o.add_inflow(*inflow)
        o.update(DT)
    g = ifl.FluidSolver(w, h, 0.1, variant=variant)
    for q in (O.QD, O.QU, O.QV):
        g.write_field(ifl.field_id(q, ifl.A_SRC), o.array(q, O.A_SRC).copy())
    g.write_field("p", o.array(0, O.A_P).copy())
    for ph in (O.PH_RHS, O.PH_PROJECT, O.PH_APPLY_P, O.PH_ADVECT):
        o.phase(ph, DT)
        g.run_phase(ph, DT)
        if ph == O.PH_RHS:
            assert np.array_equal(g.read_field("r"), o.array(0, O.A_R))
        if ph == O.PH_PROJECT:
            assert g.stats()[0] == o.stats()[0]
        _fields(ifl, g, o)


def test_pinned_sweeps(ifl):
    g = ifl.FluidSolver(48, 48, 0.1, variant=ifl.GS)
    o = O.OracleSolver(2, 48, 48)
    g.set_pinned_iterations(37, -1)
    g.addInflow(0.45, 0.2, 0.15, 0.03, 1.0, 0.0, 3.0)
    g.update(DT)
    assert g.stats()[0][0] == 37
    o.add_inflow(0.45, 0.2, 0.15, 0.03, 1.0, 0.0, 0.0, 3.0)
    o.update(DT)
    assert o.stats()[0][0] > 37


def test_tall_grid_many_strips_bit_exact(ifl):
    """35 strips (one CTA each, more strips than 32): the strip hand-over and
    the grid barrier of the cooperative launch."""
    w, h = 40, 1100
    o = O.OracleSolver(2, w, h)
    g = ifl.FluidSolver(w, h, 0.1, variant=ifl.GS)
    inflow = (0.3, 0.05, 0.4, 0.02, 1.0, 0.0, 0.0, 3.0)
    for step in range(2):
        o.add_inflow(*inflow)
        g.addInflow(*inflow[:5], *inflow[6:])
        o.update(DT)
        g.update(DT)
        assert g.stats()[0] == o.stats()[0], step
        _fields(ifl, g, o)


@pytest.mark.parametrize("variant", [1, 2])
def test_fp32_fields_with_the_fp64_gauss_seidel_solve(ifl, variant):
    """IFL_FP32 on steps 1-2: FP32 fields and advection, the Gauss-Seidel solve
    on FP64 p and r as always.  Three updates of the reference main's scene
    stay within 1e-4 (relative to the field's maximum) of the FP64 oracle."""
    w = h = 64
    inflow = (0.45, 0.2, 0.1, 0.05, 1.0, 0.0, 0.0, 3.0)
    o = O.OracleSolver(variant, w, h)
    g = ifl.FluidSolver(w, h, 0.1, variant=variant, precision=ifl.FP32)
    for _ in range(3):
        o.add_inflow(*inflow)
        g.addInflow(*inflow[:5], *inflow[6:])
        o.update(DT)
        g.update(DT)
    assert g.stats()[2] == 0
    for name, q in (("d", O.QD), ("u", O.QU), ("v", O.QV)):
        a, b = g.read_field(name), o.array(q, O.A_SRC)
        assert np.isfinite(a).all()
        assert np.abs(a - b).max() <= 1e-4 * max(np.abs(b).max(), 1.0), name
