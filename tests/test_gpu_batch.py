"""Batched form (ifl_batch_*): many ragged scenes in one step, through the C ABI.

Bars:
* FP64 batch against the oracle, one oracle per member: pinned to the
  oracle's iteration counts every field stays within 1e-9 relative over the
  run (the same bar as the single-handle trajectory test); unpinned the
  iteration counts agree within one.
* FP64 batch step from the oracle's exact state: pressure and every quantity
  within 1e-10 relative.
* FP32 batch from the oracle's state: pressure (fluid cells, mean-free) and
  velocity within 1e-4 relative of the FP64 oracle after one step.
* Replaying a step as a CUDA graph gives bit-identical fields to issuing its
  launches directly; two identical batches give bit-identical fields; a
  batched scene is bit-identical to the same scene stepped alone.
"""
import numpy as np
import pytest

from oracle import oracle as O
from test_gpu_parity import (BALL, BOX, DT, SPIN, fluid_mask, make_gpu, pressure_err, rel_err, upload,
                             velocity_err)

pytestmark = pytest.mark.gpu

TALL = (1, 0.5, 0.35, 0.16, 0.16, 0.0, 0.0, 0.0, -1.5)
FAR = (1, 0.25, 0.3, 0.16, 0.16, 0.0, 0.1, 0.0, 1.0)  # well clear of SPIN (the curved variants need a gap)
# member: w, h, inflow (x, y, w, h, d, t, u, v), bodies
MEMBERS = [
    (64, 64, (0.45, 0.2, 0.15, 0.05, 1.0, 0.0, 0.0, 3.0), [SPIN, FAR]),
    (72, 40, (0.3, 0.2, 0.4, 0.1, 1.0, 0.0, 0.5, 3.0), [BALL]),
    (40, 70, (0.3, 0.2, 0.6, 0.05, 1.0, 0.0, 0.0, 3.0), []),
    (33, 97, (0.35, 0.15, 0.3, 0.05, 1.0, 0.0, 0.0, 2.0), [TALL]),
    (130, 36, (0.2, 0.3, 0.3, 0.08, 1.0, 0.0, 1.0, 2.0), [BOX]),
]
HEAT_INFLOW = (0.45, 0.2, 0.1, 0.1, 1.0, 700.0, 0.0, 0.0)


def _still(b):
    return b[:6] + (0.0, 0.0, 0.0)


def members_for(variant):
    """The member scenes of a variant.  From 5-curved-boundaries on the bodies
    stand still and the tall member is 48 x 66: with moving bodies, or in
    that narrow tall domain with variable density, the reference's own PCG
    runs into its 2000-iteration cap on these scenes (the oracle shows it),
    which is outside the range a 1e-9 comparison can cover."""
    out = []
    for k, (w, h, inflow, bodies) in enumerate(MEMBERS):
        if variant >= 5:
            bodies = [_still(b) for b in bodies]
        if variant >= 6:
            inflow = HEAT_INFLOW
            if k == 3:
                w, h, bodies = 48, 66, [(1, 0.5, 0.6, 0.16, 0.16, 0.0, 0.0, 0.0, 0.0)]
        out.append((w, h, inflow, bodies if variant >= 4 else []))
    return out


def build(ifl, variant, precision=0, **opts):
    ms = members_for(variant)
    oracles, gpus = [], []
    for w, h, inflow, bodies in ms:
        o = O.OracleSolver(variant, w, h)
        if bodies:
            o.set_bodies(bodies)
        oracles.append(o)
        gpus.append(make_gpu(ifl, variant, w, h, bodies, precision=precision))
    b = ifl.Batch(gpus, **opts)
    for i, (_, _, inflow, _) in enumerate(ms):
        b.set_inflows(i, [inflow])
    return ms, oracles, gpus, b


@pytest.mark.parametrize("variant", [3, 4, 5, 6, 7])
def test_batch_step_fp64_from_oracle_state(ifl, variant):
    """One batch step from the oracle's exact state, iterations pinned to the
    oracle's: pressure (fluid cells) and every quantity within 1e-10 relative.
    7-variable-density: 1e-8.  Its variable-coefficient systems make CG
    sensitive to the rounding of its FP64 sums; the single-handle path (another
    order again) shows the same size on these members (4e-9 in u on the
    40 x 70 member, 4e-10 on the 48 x 66 one, 1e-15 on the others)."""
    tol = 1e-8 if variant == 7 else 1e-10
    ms, oracles, gpus, b = build(ifl, variant)
    for (w, h, inflow, _), o in zip(ms, oracles):
        for _ in range(3):
            o.add_inflow(*inflow)
            o.update(DT)
            o.advance_bodies(DT)
    for o, g in zip(oracles, gpus):
        g.set_bodies(o.bodies())
        upload(ifl, g, o, variant)
    for (w, h, inflow, _), o, g in zip(ms, oracles, gpus):
        o.add_inflow(*inflow)
        o.update(DT)
        (opi, _, _), (ohi, _, _) = o.stats()
        g.set_pinned_iterations(opi, ohi)
    b.update(DT)
    names = [("d", O.QD), ("u", O.QU), ("v", O.QV)] + ([("t", O.QT)] if variant >= 6 else [])
    for i, (o, g) in enumerate(zip(oracles, gpus)):
        assert b.stats()[i][2] & 1 == 0
        assert pressure_err(g, o, variant) < tol, i
        for name, q in names:
            assert rel_err(g.read_field(name), o.array(q, O.A_SRC)) < tol, (i, name)


@pytest.mark.parametrize("variant", [3, 4, 5, 6, 7])
def test_batch_trajectory_fp64_pinned(ifl, variant):
    """Five whole steps from a zero state with the oracle's iteration counts.
    Rounding of the PCG sums (another fixed order than the oracle's) carries
    from step to step; the heat variants amplify it most (see the one-step
    test): 1e-9 up to 5-curved-boundaries, 1e-8 for 6-heat, 1e-6 for
    7-variable-density."""
    tol = {6: 1e-8, 7: 1e-6}.get(variant, 1e-9)
    ms, oracles, gpus, b = build(ifl, variant)
    names = [("d", O.QD), ("u", O.QU), ("v", O.QV)] + ([("t", O.QT)] if variant >= 6 else [])
    for step in range(5):
        pins = []
        for (w, h, inflow, _), o, g in zip(ms, oracles, gpus):
            o.add_inflow(*inflow)
            g.set_bodies(o.bodies())
            o.update(DT)
            (opi, _, _), (ohi, _, _) = o.stats()
            g.set_pinned_iterations(opi, ohi)
            pins.append((opi, ohi))
        b.update(DT)
        for i, ((pi, _, _), (hi, _, _), flags) in enumerate(b.stats()):
            assert flags & 1 == 0
            assert (pi, hi if variant >= 6 else pins[i][1]) == pins[i], (step, i)
        for i, (o, g) in enumerate(zip(oracles, gpus)):
            for name, q in names:
                assert rel_err(g.read_field(name), o.array(q, O.A_SRC)) < tol, (step, i, name)
            o.advance_bodies(DT)


def test_batch_iterations_unpinned_fp64(ifl):
    ms, oracles, gpus, b = build(ifl, 4)
    for step in range(4):
        its = []
        for (w, h, inflow, _), o, g in zip(ms, oracles, gpus):
            o.add_inflow(*inflow)
            g.set_bodies(o.bodies())
            o.update(DT)
            its.append(o.stats()[0][0])
            o.advance_bodies(DT)
        b.update(DT)
        for i, ((pi, _, _), _, flags) in enumerate(b.stats()):
            assert flags & 1 == 0 and abs(pi - its[i]) <= 1, (step, i, pi, its[i])


@pytest.mark.parametrize("variant", [4, 7])
def test_batch_fp32_form_error_vs_fp64_oracle(ifl, variant):
    ms, oracles, gpus, b = build(ifl, variant, precision=ifl.FP32)
    for (w, h, inflow, _), o in zip(ms, oracles):
        for _ in range(4):
            o.add_inflow(*inflow)
            o.update(DT)
            o.advance_bodies(DT)
    for o, g in zip(oracles, gpus):
        g.set_bodies(o.bodies())
        upload(ifl, g, o, variant)
    for (w, h, inflow, _), o in zip(ms, oracles):
        o.add_inflow(*inflow)
        o.update(DT)
    b.update(DT)
    for i, (o, g) in enumerate(zip(oracles, gpus)):
        assert b.stats()[i][2] & 1 == 0
        errs = {"p": mean_free_pressure_err(g, o, variant), "velocity": velocity_err(g, o)}
        assert errs["p"] < 1e-4 and errs["velocity"] < 1e-4, (i, errs)


def mean_free_pressure_err(g, o, variant):
    """The closed domain fixes the pressure only up to a constant; the FP32
    form's rounding moves that constant, the velocity does not see it."""
    m = fluid_mask(o, variant)
    a, r = g.read_field("p")[m], o.array(0, O.A_P)[m]
    return rel_err(a - a.mean(), r - r.mean())


def _run(ifl, precision, steps, **opts):
    ms, oracles, gpus, b = build(ifl, 4, precision=precision, **opts)
    for _ in range(steps):
        b.update(DT)
    return b, [[g.read_field(n) for n in ("d", "u", "v", "p")] for g in gpus]


def test_graph_replay_equals_direct_launches(ifl):
    shape = dict(threads=256, strips_per_block=4, stages=3)
    bg, a = _run(ifl, ifl.FP32, 3, use_graph=True, **shape)
    bd, c = _run(ifl, ifl.FP32, 3, use_graph=False, **shape)
    assert bg.info()["graph"] and not bd.info()["graph"]
    for x, y in zip(a, c):
        for u, v in zip(x, y):
            assert np.array_equal(u, v)
    # and a second identical batch
    _, e = _run(ifl, ifl.FP32, 3, use_graph=True, **shape)
    for x, y in zip(a, e):
        for u, v in zip(x, y):
            assert np.array_equal(u, v)


def test_autotuner_tries_shapes_and_keeps_one(ifl):
    b, _ = _run(ifl, ifl.FP32, 2)
    info = b.info()
    tried = [t for t in info["candidate_ms"] if t > 0]
    assert len(tried) >= 2
    assert info["threads"] in (32, 64, 128, 256) and 1 <= info["strips_per_block"] <= info["threads"] // 32
    assert info["grid"] > 0 and info["steps"] == 2 and info["launches"] > 0


def test_tile_autotuner_keeps_a_candidate_per_phase(ifl):
    b, _ = _run(ifl, ifl.FP32, 2)
    info = b.info()
    assert set(info["tile_ms"]) == {"fill", "bc", "assemble", "advect"}  # variant 4: no heat assembly
    for name, shape in info["tiles"].items():
        assert tuple(shape) in ifl.TILE_SHAPES, (name, shape)
    for name in ("apply", "buoyancy", "mask"):
        assert tuple(info["tiles"][name]) == (32, 8)


@pytest.mark.parametrize("variant", [5, 7])
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_tile_shapes_do_not_change_results(ifl, variant, precision):
    """Every tuned phase on another tile shape than 32 x 8 gives bit-identical
    fields (each cell's arithmetic is independent of the tiling)."""
    forced = {"fill": (16, 16), "bc": (128, 2), "assemble": (64, 4), "heat_assemble": (32, 4),
              "advect": (64, 2)}
    out = []
    for tiles in ("default", forced):
        ms, oracles, gpus, b = build(ifl, variant, precision=precision, tiles=tiles)
        for _ in range(3):
            b.update(DT)
        names = ("d", "u", "v", "p") + (("t",) if variant >= 6 else ())
        out.append([[g.read_field(n) for n in names] for g in gpus])
        if tiles != "default":
            assert {k: tuple(v) for k, v in b.info()["tiles"].items() if k in forced} == forced
    for x, y in zip(*out):
        for u, v in zip(x, y):
            assert np.array_equal(u, v)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_batch_equals_single_handles_bit_for_bit(ifl, precision):
    """Ragged generated scenes (sides 64..320, 0-4 bodies, 1-3 inflows): every
    PCG reduction is summed in per-scene chunks, so a scene's batched step is
    bit-identical to the same scene stepped alone through ifl_update, whatever
    the batch's launch shape."""
    from ifluids import scenes as SC
    sc = SC.batch_scenes(count=12, seed=7, lo=64, hi=320)

    def member(s):
        return ifl.FluidSolver(s.w, s.h, 0.1, list(s.bodies), precision=precision)
    batch_m = [member(s) for s in sc]
    alone = [member(s) for s in sc]
    b = ifl.Batch(batch_m)
    for i, s in enumerate(sc):
        b.set_inflows(i, s.inflows)
    dt = sc[0].dt
    for step in range(3):
        b.update(dt)
        st = b.stats()
        for i, s in enumerate(sc):
            for r in s.inflows:
                alone[i].addInflow(*r[:5], *r[6:])
            alone[i].update(dt)
            assert st[i][2] & 1 == 0
            assert alone[i].stats()[0][0] == st[i][0][0], (step, i)
        for m in batch_m + alone:
            m.set_bodies([_moved(bd, dt) for bd in m.bodies])
    for i in range(len(sc)):
        for n in ("d", "u", "v", "p"):
            assert np.array_equal(batch_m[i].read_field(n), alone[i].read_field(n)), (i, n)


def test_fp32_form_converges_like_fp64(ifl):
    """The FP32 form's pressure solves need about as many iterations as the
    FP64 ones and never reach the cap: its matvec keeps the reference's exact
    zero row sums (an FP32-rounded diagonal made CG stagnate on some scenes)."""
    from ifluids import scenes as SC
    sc = SC.batch_scenes(count=24, seed=11, lo=128, hi=640)
    runs = {}
    for prec in (ifl.FP64, ifl.FP32):
        ms = [ifl.FluidSolver(s.w, s.h, 0.1, list(s.bodies), precision=prec) for s in sc]
        b = ifl.Batch(ms)
        for i, s in enumerate(sc):
            b.set_inflows(i, s.inflows)
        its = []
        for _ in range(4):
            b.update(sc[0].dt)
            its.append([x[0][0] for x in b.stats()])
            assert all(x[0][1] == 0 or x[0][0] == 0 for x in b.stats())  # converged (or nothing to solve)
        runs[prec] = np.array(its)
    assert (runs[ifl.FP32] <= 1.15 * runs[ifl.FP64] + 5).all(), (runs[ifl.FP32] - runs[ifl.FP64])


def _moved(b, dt):
    t, x, y, sx, sy, th, vx, vy, vt = b
    return (t, x + vx * dt, y + vy * dt, sx, sy, th + vt * dt, vx, vy, vt)
