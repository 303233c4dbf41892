"""The allocation-free pressure solve (ifl_pcg_solve_noalloc) against the solver's own PCG.

For callers that cannot allocate device memory while they run, the library
offers one entry point whose scratch is a fixed device array inside the
library.  This file runs last (it checks that the shared array, which keeps the
previous call's contents, is cleared where it must be).  Calls in a row on
different grids, the largest close to the array's limit first, must each
reproduce the regular solver's pressure and the oracle's project() within the
FP64 tolerance of the other parity tests (1e-10 relative) with the same
iteration count.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
DT = 0.005
TOL = 1e-10


def _velocities(w, h, seed):
    rng = np.random.default_rng(seed)
    u = rng.normal(size=(h, w + 1))
    v = rng.normal(size=(h + 1, w))
    u[:, 0] = u[:, w] = 0.0  # closed walls: the Neumann system is consistent
    v[0, :] = v[h, :] = 0.0
    return u, v


def _reference_solve(ifl, w, h, seed):
    """Matrix, right-hand side and pressure of the regular (allocating) solver."""
    g = ifl.FluidSolver(w, h, 0.1)
    u, v = _velocities(w, h, seed)
    g.write_field("u", u)
    g.write_field("v", v)
    g.run_phase(ifl.PH_RHS, DT)
    g.run_phase(ifl.PH_MATRIX, DT)
    arrays = [g.read_field(n) for n in ("adiag", "aplusx", "aplusy", "r")]
    g.run_phase(ifl.PH_PRECON, DT)
    g.run_phase(ifl.PH_PROJECT, DT)
    (it, st, err), _, flags = g.stats()
    assert flags & 1 == 0
    return arrays, g.read_field("p"), it, st


def _oracle_solve(w, h, seed):
    """The same system through the oracle's buildRhs / buildPressureMatrix / project."""
    from oracle import oracle as O
    o = O.OracleSolver(O.PLAIN, w, h)
    u, v = _velocities(w, h, seed)
    o.array(O.QU, O.A_SRC)[...] = u
    o.array(O.QV, O.A_SRC)[...] = v
    for ph in (O.PH_RHS, O.PH_MATRIX, O.PH_PRECON, O.PH_PROJECT):
        o.phase(ph, DT)
    (it, st, _), _ = o.stats()[:2]
    return o.array(0, O.A_P).copy(), it, st


def _noalloc(ifl, torch, w, h, arrays, max_iter=600):
    dev = torch.device("cuda", 0)
    d = [torch.tensor(a, dtype=torch.float64, device=dev).contiguous() for a in arrays]
    p = torch.full((h, w), float("nan"), dtype=torch.float64, device=dev)
    stats = torch.zeros(2, dtype=torch.float64, device=dev)  # ifl_pcg_stats: int32, int32, double
    torch.cuda.synchronize()
    rc = ifl.pcg_solve_noalloc(w, h, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), d[3].data_ptr(),
                               p.data_ptr(), max_iter, stats.data_ptr())
    torch.cuda.synchronize()
    raw = stats.cpu().numpy().tobytes()
    it, st = (int(x) for x in np.frombuffer(raw[:8], dtype=np.int32))
    return rc, p.cpu().numpy(), it, st


def test_noalloc_matches_regular_solver_and_oracle_in_a_row(ifl):
    torch = pytest.importorskip("torch")
    # 256 x 256 uses 8 x 288 = 2304 strip-diagonals, the whole fixed array
    # (several blocks, halo rows between them); the smaller, differently shaped
    # grids that follow must not see its leftovers.
    for w, h, seed in ((256, 256, 3), (96, 80, 1), (64, 48, 2)):
        arrays, p_ref, it_ref, st_ref = _reference_solve(ifl, w, h, seed)
        rc, got, it, st = _noalloc(ifl, torch, w, h, arrays)
        assert rc == ifl.OK
        assert (it, st) == (it_ref, st_ref), (w, h)
        assert np.abs(got - p_ref).max() <= TOL * np.abs(p_ref).max(), (w, h)
        p_o, it_o, st_o = _oracle_solve(w, h, seed)
        assert (it, st) == (it_o, st_o), (w, h)
        assert np.abs(got - p_o).max() <= TOL * np.abs(p_o).max(), (w, h)


def test_noalloc_rejects_grids_beyond_its_scratch(ifl):
    # 1024 x 1024 needs 32 x 1056 strip-diagonals, far beyond the fixed scratch; the
    # size check comes before any device work, so placeholder pointers are never used
    assert ifl.pcg_solve_noalloc(1024, 1024, 1, 1, 1, 1, 1, 600, 1) == ifl.ERR_UNSUPPORTED
