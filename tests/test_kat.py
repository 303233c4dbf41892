"""Known-answer tests of the oracle's scalar kernels, from the mathematics."""
import numpy as np
import pytest

from oracle import oracle as O


def _clip_area(nx, ny, c):
    """Area of {p in [0,1]^2 : nx*px + ny*py + c < 0} by polygon clipping."""
    poly = [(0.0, 0.0), (1.0, 0.0), (1.0, 1.0), (0.0, 1.0)]
    f = lambda p: nx * p[0] + ny * p[1] + c
    out = []
    for i in range(4):
        a, b = poly[i], poly[(i + 1) % 4]
        fa, fb = f(a), f(b)
        if fa < 0:
            out.append(a)
        if (fa < 0) != (fb < 0):
            t = fa / (fa - fb)
            out.append((a[0] + t * (b[0] - a[0]), a[1] + t * (b[1] - a[1])))
    if len(out) < 3:
        return 0.0
    area = 0.0
    for i in range(len(out)):
        x0, y0 = out[i]
        x1, y1 = out[(i + 1) % len(out)]
        area += x0 * y1 - x1 * y0
    return abs(area) / 2


def test_occupancy_of_half_planes():
    """For a linear distance field the reference's triangle/trapezoid formulas are exact."""
    rng = np.random.default_rng(5)
    seen = set()
    for _ in range(4000):
        ang = rng.uniform(0, 2 * np.pi)
        nx, ny = np.cos(ang), np.sin(ang)
        c = rng.uniform(-1.5, 1.5)
        d = {(i, j): nx * i + ny * j + c for i in (0, 1) for j in (0, 1)}
        if min(abs(v) for v in d.values()) < 1e-6:
            continue
        occ = O.occupancy(d[0, 0], d[1, 0], d[0, 1], d[1, 1])
        mask = sum(1 << k for k, key in enumerate([(0, 0), (1, 0), (1, 1), (0, 1)]) if d[key] < 0)
        seen.add(mask)
        assert occ == pytest.approx(_clip_area(nx, ny, c), abs=1e-12)
    # a single line reaches every mask except the two opposed-corner ones and "none/all" both occur
    assert len(seen) == 14


def test_occupancy_opposed_corners():
    # two inside corners on a diagonal: sum of the two corner triangles
    occ = O.occupancy(-0.5, 0.5, 0.5, -0.5)
    assert occ == pytest.approx(2 * 0.5 * 0.25 / (1.0 * 1.0))


def test_cerp_reproduces_constants_and_lines():
    for x in np.linspace(0, 1, 17):
        assert O.cerp(2.5, 2.5, 2.5, 2.5, x) == 2.5
        assert O.cerp(0.0, 1.0, 2.0, 3.0, x) == pytest.approx(1.0 + x, abs=1e-15)


def test_cerp_is_clamped_to_samples():
    rng = np.random.default_rng(1)
    for _ in range(1000):
        a = rng.normal(size=4)
        x = rng.uniform()
        v = O.cerp(*a, x)
        assert a.min() <= v <= a.max()


def test_pcg_solution_satisfies_its_residual():
    """The oracle's pressure solves A p = b to the reported max residual (plain variant)."""
    s = O.OracleSolver(3, 16, 16)
    s.add_inflow(0.3, 0.2, 0.4, 0.3, 1.0, 0.0, 1.0, 3.0)
    s.phase(O.PH_RHS, 0.005)
    b = s.array(0, O.A_R).copy()
    s.phase(O.PH_MATRIX, 0.005)
    s.phase(O.PH_PRECON, 0.005)
    s.phase(O.PH_PROJECT, 0.005)
    it, st, err = s.stats()[0]
    assert st == O.PCG_CONVERGED and err < 1e-5
    d, ax, ay = (s.array(0, k) for k in (O.A_ADIAG, O.A_APLUSX, O.A_APLUSY))
    p = s.array(0, O.A_P)
    Ap = d * p
    Ap[:, 1:] += ax[:, :-1] * p[:, :-1]
    Ap[:, :-1] += ax[:, :-1] * p[:, 1:]
    Ap[1:, :] += ay[:-1, :] * p[:-1, :]
    Ap[:-1, :] += ay[:-1, :] * p[1:, :]
    assert np.abs(Ap - b).max() < 1e-4
    # constant vectors are in the null space of the pure-Neumann matrix
    one = np.ones_like(p)
    A1 = d * one
    A1[:, 1:] += ax[:, :-1]
    A1[:, :-1] += ax[:, :-1]
    A1[1:, :] += ay[:-1, :]
    A1[:-1, :] += ay[:-1, :]
    assert np.abs(A1).max() < 1e-9
