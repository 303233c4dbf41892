"""Parity at the benchmark configurations' own sizes (needs a GB300).

Each comparison starts both sides from an identical state and runs one
update(): the GPU result against the reference's own FP64 solver (compiled on
this host from the staged sources, oracle/_ref) or, where that was not built,
the oracle that is pinned bit-for-bit to it.

* 128 x 128 plain step, FP64 drop-in, 100 steps (3-conjugate-gradients/Fluid.cpp:433-447):
  the configuration's rectangle injects nothing (every field stays zero and
  project() returns on its initial residual); with the reference main's own
  rectangle every one of the 100 steps matches within 1e-10 relative
  (max-norm) with the same PCG iteration count, the GPU taking the oracle's
  state before each step.
* 1024 x 1024, three seeded bodies, FP32 form, 200 steps
  (4-solid-boundaries/Fluid.cpp:869-895): the GPU runs its own 200-step
  trajectory; at steps 1, 50, 100, 150 and 200 its state before the step is
  given to the FP64 reference, and p (fluid cells), u, v and d after the step
  must agree within 1e-4 relative.
* The 512-scene batch at the first timed step of the benchmark (after three
  warm-up steps): a size-stratified sample of eight members, FP32 form, 1e-4.
The reference's CPU solves run in a spawned process pool (about 25 s per 1024^2
update on one core).
"""
import multiprocessing as mp

import numpy as np
import pytest

from oracle import oracle as O
from ifluids import scenes

pytestmark = pytest.mark.gpu
FP32_TOL = 1e-4
FP64_TOL = 1e-10


def ref_kind(variant):
    return "reference" if O.ref_available(variant) else "oracle"


def qs(variant):
    return [O.QD, O.QU, O.QV] + ([O.QT] if variant >= 6 else [])


def gpu_state(ifl, g, variant):
    """Source and target buffers of every advected quantity, as FP64."""
    return {(q, a): np.asarray(g.read_field(ifl.field_id(q, a)), dtype=np.float64)
            for q in qs(variant) for a in (O.A_SRC, O.A_DST)}


def gpu_result(ifl, g, variant):
    out = {q: np.asarray(g.read_field(ifl.field_id(q, O.A_SRC)), dtype=np.float64) for q in qs(variant)}
    out["p"] = np.asarray(g.read_field("p"), dtype=np.float64)
    return out


def body_objs(ifl, sc):
    return [ifl.SolidBox(*b[1:]) if b[0] == 0 else ifl.SolidSphere(b[1], b[2], b[3], *b[5:]) for b in sc.bodies]


def reference_steps(jobs, procs):
    """step_from_state for every job, in a spawned pool (safe after CUDA init)."""
    with mp.get_context("spawn").Pool(max(1, min(procs, len(jobs)))) as pool:
        return pool.starmap(O.step_from_state, jobs)


def test_config0_as_stated_stays_zero(ifl):
    """The configuration's own rectangle selects the row y = 25, whose pulse is zero at 128^2."""
    sc = scenes.config0()
    g = ifl.FluidSolver(128, 128, 0.1)
    x, y, w, h, d, t, u, v = sc.inflows[0]
    for _ in range(sc.steps):
        g.addInflow(x, y, w, h, d, u, v)
        g.update(sc.dt)
        (it, st, _), _, flags = g.stats()
        assert (it, st, flags) == (0, ifl.PCG_INITIAL, 0)
    for name in ("d", "u", "v"):
        assert not np.any(g.read_field(name))


def test_config0b_fp64_every_step_from_the_same_state(ifl):
    sc = scenes.config0b()
    o = O.OracleSolver(O.PLAIN, 128, 128)
    g = ifl.FluidSolver(128, 128, 0.1)
    x, y, w, h, d, t, u, v = sc.inflows[0]
    worst = {}
    for k in range(sc.steps):
        for q in qs(3):
            for a in (O.A_SRC, O.A_DST):
                g.write_field(ifl.field_id(q, a), o.array(q, a).copy())
        o.add_inflow(*sc.inflows[0])
        g.addInflow(x, y, w, h, d, u, v)
        o.update(sc.dt)
        g.update(sc.dt)
        (it, st, _), _, flags = g.stats()
        assert flags & 1 == 0
        assert (it, st) == o.stats()[0][:2], k
        ref = {q: o.array(q, O.A_SRC) for q in qs(3)}
        ref["p"], ref["fluid"] = o.array(0, O.A_P), np.ones((128, 128), dtype=bool)
        for f, e in O.field_errors(gpu_result(ifl, g, 3), ref, 3).items():
            worst[f] = max(worst.get(f, 0.0), e)
            assert e <= FP64_TOL, (k, f, e)
    assert worst["p"] > 0.0 or worst["d"] == 0.0  # the comparison saw real fields


def test_config1_fp32_form_against_fp64_over_200_steps(ifl):
    sc = scenes.config1()
    bodies = body_objs(ifl, sc)
    g = ifl.FluidSolver(sc.w, sc.h, sc.density, bodies, precision=ifl.FP32)
    x, y, w, h, d, t, u, v = sc.inflows[0]
    samples = (1, 50, 100, 150, 200)
    jobs, outs = [], []
    for k in range(1, sc.steps + 1):
        if k in samples:
            jobs.append((4, sc.w, sc.h, gpu_state(ifl, g, 4), [b.as_tuple() for b in bodies], sc.inflows, sc.dt,
                         ref_kind(4)))
        g.addInflow(x, y, w, h, d, u, v)
        g.update(sc.dt)
        if k in samples:
            (it, st, _), _, flags = g.stats()
            assert flags & 1 == 0 and st == ifl.PCG_CONVERGED, (k, it, st)
            outs.append(gpu_result(ifl, g, 4))
        for b in bodies:
            b.update(sc.dt)
    g.close()
    refs = reference_steps(jobs, len(jobs))
    for k, out, ref in zip(samples, outs, refs):
        assert ref["stats"][0][1] == O.PCG_CONVERGED, (k, ref["stats"])
        errs = O.field_errors(out, ref, 4)
        assert max(errs.values()) <= FP32_TOL, (k, errs)


def stratified(scs, k):
    order = sorted(range(len(scs)), key=lambda i: scs[i].cells)
    return [order[int((j + 0.5) * len(order) / k)] for j in range(k)]


def test_batch_sample_at_the_first_timed_step(ifl):
    scs = scenes.batch_scenes(count=512, seed=2)
    bodies = [body_objs(ifl, sc) for sc in scs]
    members = [ifl.FluidSolver(sc.w, sc.h, sc.density, bs, precision=ifl.FP32) for sc, bs in zip(scs, bodies)]
    b = ifl.Batch(members, threads=64, strips_per_block=1, stages=2)
    for i, sc in enumerate(scs):
        b.set_inflows(i, sc.inflows)
    dt = scs[0].dt
    for _ in range(3):  # the benchmark's warm-up steps
        b.update(dt)
        for bs in bodies:
            for x in bs:
                x.update(dt)
    pick = stratified(scs, 8)
    jobs = [(4, scs[i].w, scs[i].h, gpu_state(ifl, members[i], 4), [x.as_tuple() for x in bodies[i]],
             scs[i].inflows, dt, ref_kind(4)) for i in pick]
    b.update(dt)
    stats = b.stats()
    outs = [gpu_result(ifl, members[i], 4) for i in pick]
    b.close()
    refs = reference_steps(jobs, len(jobs))
    for i, out, ref in zip(pick, outs, refs):
        assert stats[i][2] & 1 == 0
        errs = O.field_errors(out, ref, 4)
        assert max(errs.values()) <= FP32_TOL, (scs[i].w, scs[i].h, stats[i][0], ref["stats"][0], errs)


def test_config3_heat_variable_density_prefix(ifl):
    """2048 x 2048, step 7 (heat solve + variable density), FP32 form and FP64 drop-in: at
    updates 1 and 5 of each form's own trajectory the next update is compared with the
    reference's FP64 update from the same state (7-variable-density/Fluid.cpp:995-1034).

    FP32 form: 1e-4 for every field.  FP64 drop-in: 1e-6.  The pressure solve here runs
    about 1400 iterations of a variable-coefficient system; its dot products are summed in
    a fixed parallel order instead of the reference's sequential loop, and CG carries that
    last-bit difference in alpha and beta into the iterates, so the two FP64 solutions
    differ by about 1e-8 relative in p.  The velocity update differences p across each
    face and the pressure field is large against the velocities it corrects, so u and v
    differ by up to about 2e-7 of the largest velocity.  The 1e-10 bar of the smaller
    scenes (128^2 above) cannot hold at this size for any summation order other than the
    reference's own."""
    sc = scenes.config3()
    samples = (1, 5)
    jobs, outs, tols, names = [], [], [], []
    for precision, tol in ((ifl.FP32, FP32_TOL), (ifl.FP64, 1e-6)):
        bodies = body_objs(ifl, sc)
        g = ifl.FluidSolver(sc.w, sc.h, sc.density, sc.density_soot, sc.diffusion, bodies, variant=7,
                            precision=precision)
        for k in range(1, max(samples) + 1):
            if k in samples:
                jobs.append((7, sc.w, sc.h, gpu_state(ifl, g, 7), [b.as_tuple() for b in bodies], sc.inflows,
                             sc.dt, ref_kind(7)))
            g.addInflow(*sc.inflows[0])
            g.update(sc.dt)
            if k in samples:
                assert g.stats()[2] & 1 == 0
                outs.append(gpu_result(ifl, g, 7))
                tols.append(tol)
                names.append(("fp32" if precision == ifl.FP32 else "fp64", k, g.stats()[0][0]))
            for b in bodies:
                b.update(sc.dt)
        g.close()
    refs = reference_steps(jobs, len(jobs))
    errs = [O.field_errors(out, ref, 7) for out, ref in zip(outs, refs)]
    report = [(n, ref["stats"][0][0], e) for n, ref, e in zip(names, refs, errs)]
    print(report)
    for (n, it, e), tol in zip(report, tols):
        assert max(e.values()) <= tol, report
