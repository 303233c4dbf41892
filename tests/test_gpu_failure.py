"""Failure detection and the solver's edge semantics, without faulting the GPU.

* Bounded waits: a solve whose device-side waits are given a limit they cannot
  meet (ifl_set_wait_limit) must return, report IFL_ERR_TIMEOUT through
  ifl_get_stats, and leave the GPU usable for the next handle.  The wait runs
  out because nothing releases it within two polls; nothing faults or hangs.
* NaN right-hand side: std::max(0, NaN) is 0 in the reference, so its
  infinityNorm ignores NaN and project() stops "converged" once the residual is
  NaN everywhere (3-conjugate-gradients/Fluid.cpp:341-346, 354-356, 368-369).
  The GPU must stop after the same iteration with the same NaN pattern.
* Iteration cap: max_iter_pressure bounds the solve as the reference's
  `project(limit)` does (3-conjugate-gradients/Fluid.cpp:359-380).
"""
import numpy as np
import pytest

from oracle import oracle as O

DT = 0.005


def _closed_velocities(w, h, seed):
    rng = np.random.default_rng(seed)
    u = rng.normal(size=(h, w + 1))
    v = rng.normal(size=(h + 1, w))
    u[:, 0] = u[:, w] = 0.0
    v[0, :] = v[h, :] = 0.0
    return u, v


def _oracle_system(w, h, seed):
    o = O.OracleSolver(O.PLAIN, w, h)
    u, v = _closed_velocities(w, h, seed)
    o.array(O.QU, O.A_SRC)[...] = u
    o.array(O.QV, O.A_SRC)[...] = v
    o.phase(O.PH_RHS, DT)
    o.phase(O.PH_MATRIX, DT)
    return o


def test_oracle_nan_rhs_stops_converged():
    """The oracle itself: a NaN in r makes project() stop after one iteration, p all NaN."""
    o = _oracle_system(48, 40, 5)
    o.array(0, O.A_R)[17, 23] = np.nan
    o.phase(O.PH_PRECON, DT)
    o.phase(O.PH_PROJECT, DT)
    (it, st, err), _ = o.stats()
    assert (it, st) == (1, O.PCG_CONVERGED)
    assert err == 0.0
    assert np.isnan(o.array(0, O.A_P)).all()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_nan_rhs_matches_oracle(ifl, precision):
    w, h, seed = 48, 40, 5
    o = _oracle_system(w, h, seed)
    g = ifl.FluidSolver(w, h, 0.1, precision=precision)
    u, v = _closed_velocities(w, h, seed)
    g.write_field("u", u)
    g.write_field("v", v)
    g.run_phase(ifl.PH_RHS, DT)
    g.run_phase(ifl.PH_MATRIX, DT)
    r = g.read_field("r")
    r[17, 23] = np.nan
    g.write_field("r", r)
    o.array(0, O.A_R)[17, 23] = np.nan
    for ph_g, ph_o in ((ifl.PH_PRECON, O.PH_PRECON), (ifl.PH_PROJECT, O.PH_PROJECT)):
        g.run_phase(ph_g, DT)
        o.phase(ph_o, DT)
    (it, st, err), _, flags = g.stats()
    (it_o, st_o, err_o), _ = o.stats()
    assert flags & 1 == 0
    assert (it, st, err) == (it_o, st_o, err_o) == (1, ifl.PCG_CONVERGED, 0.0)
    assert np.array_equal(np.isnan(g.read_field("p")), np.isnan(o.array(0, O.A_P)))


@pytest.mark.gpu
def test_iteration_cap_matches_oracle_pinned(ifl):
    """A cap of 7 iterations: status CAP, and p equals the oracle after exactly 7 iterations."""
    w, h, seed, cap = 96, 80, 6, 7
    o = _oracle_system(w, h, seed)
    o.set_pinned_iterations(cap)
    g = ifl.FluidSolver(w, h, 0.1, max_iter_pressure=cap)
    u, v = _closed_velocities(w, h, seed)
    g.write_field("u", u)
    g.write_field("v", v)
    for ph_g, ph_o in ((ifl.PH_RHS, O.PH_RHS), (ifl.PH_MATRIX, O.PH_MATRIX), (ifl.PH_PRECON, O.PH_PRECON),
                       (ifl.PH_PROJECT, O.PH_PROJECT)):
        g.run_phase(ph_g, DT)
        if ph_o not in (O.PH_RHS, O.PH_MATRIX):  # already run by _oracle_system
            o.phase(ph_o, DT)
    (it, st, err), _, flags = g.stats()
    assert flags & 1 == 0
    assert (it, st) == (cap, ifl.PCG_CAP)
    assert o.stats()[0][0] == cap
    p, p_o = g.read_field("p"), o.array(0, O.A_P)
    assert np.abs(p - p_o).max() <= 1e-10 * np.abs(p_o).max()


def _expect_timeout(ifl, fn):
    with pytest.raises(ifl.IflError) as e:
        fn()
    assert e.value.code == ifl.ERR_TIMEOUT


@pytest.mark.gpu
@pytest.mark.parametrize("variant,precision", [(3, 0), (4, 1), (2, 0)], ids=["pcg-fp64", "pcg-fp32", "gauss-seidel"])
def test_wait_limit_times_out_and_gpu_stays_usable(ifl, variant, precision):
    """Two polls per wait cannot cover a 256^2 solve (many strips and blocks): the
    update must come back with IFL_ERR_TIMEOUT; a new handle then solves normally."""
    w = h = 256

    def scene(limit):
        g = ifl.FluidSolver(w, h, 0.1, variant=variant, precision=precision)
        g.set_wait_limit(limit)
        g.addInflow(0.45, 0.2, 0.15, 0.03, 1.0, 0.0, 3.0)
        g.update(DT)
        return g

    g = scene(1)
    _expect_timeout(ifl, g.stats)
    g.close()
    g = scene(0)  # the default limit
    (it, st, err), _, flags = g.stats()
    assert flags & 1 == 0 and it > 0


@pytest.mark.gpu
def test_batch_wait_limit_times_out(ifl):
    """The persistent batched launch: every team stops waiting, the launch returns and
    each member's status word carries the timeout."""
    members = [ifl.FluidSolver(w, h, 0.1, [], precision=1) for w, h in ((200, 300), (256, 96), (64, 520))]
    members[0].set_wait_limit(1)
    b = ifl.Batch(members, threads=64, strips_per_block=1, stages=2)
    for k in range(len(members)):
        b.set_inflows(k, [(0.45, 0.2, 0.15, 0.03, 1.0, 0.0, 3.0)])
    _expect_timeout(ifl, lambda: b.update(0.0025))
    assert any(st[2] & 1 for st in b.stats())
