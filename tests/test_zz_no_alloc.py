"""The allocation-free pressure solve (ifl_pcg_solve_noalloc) against the solver's own PCG.

For callers that cannot allocate device memory while they run, the library
offers one entry point whose scratch is a fixed device array inside the
library.  This file runs last (it checks that the shared array, which keeps the
previous call's contents, is cleared where it must be): two calls in a row on
different grids must each reproduce the regular solver's pressure within the
FP64 tolerance of the other parity tests (1e-10 relative) with the same
iteration count.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
DT = 0.005


def _reference_solve(ifl, w, h, seed):
    """Matrix, right-hand side and pressure of the regular (allocating) solver."""
    g = ifl.FluidSolver(w, h, 0.1)
    rng = np.random.default_rng(seed)
    u = rng.normal(size=(h, w + 1))
    v = rng.normal(size=(h + 1, w))
    u[:, 0] = u[:, w] = 0.0  # closed walls: the Neumann system is consistent
    v[0, :] = v[h, :] = 0.0
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


def test_noalloc_matches_regular_solver_twice_in_a_row(ifl):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    for w, h, seed in ((96, 80, 1), (64, 48, 2)):
        (adiag, ax, ay, rhs), p_ref, it_ref, st_ref = _reference_solve(ifl, w, h, seed)
        d = [torch.tensor(a, dtype=torch.float64, device=dev).contiguous() for a in (adiag, ax, ay, rhs)]
        p = torch.full((h, w), float("nan"), dtype=torch.float64, device=dev)
        stats = torch.zeros(2, dtype=torch.float64, device=dev)  # ifl_pcg_stats: int32, int32, double
        torch.cuda.synchronize()
        rc = ifl.pcg_solve_noalloc(w, h, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), d[3].data_ptr(),
                                   p.data_ptr(), 600, stats.data_ptr())
        torch.cuda.synchronize()
        assert rc == ifl.OK
        raw = stats.cpu().numpy().tobytes()
        it, st = np.frombuffer(raw[:8], dtype=np.int32)
        assert (it, st) == (it_ref, st_ref)
        got = p.cpu().numpy()
        assert np.abs(got - p_ref).max() <= 1e-10 * np.abs(p_ref).max()


def test_noalloc_rejects_grids_beyond_its_scratch(ifl):
    # 1024 x 1024 needs 32 x 1056 strip-diagonals, far beyond the fixed scratch; the
    # size check comes before any device work, so placeholder pointers are never used
    assert ifl.pcg_solve_noalloc(1024, 1024, 1, 1, 1, 1, 1, 600, 1) == ifl.ERR_UNSUPPORTED
