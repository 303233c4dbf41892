"""Small, reproducible batched-PCG launch for profiler captures.

    python -m ifluids.profile_case [--shape 64,1,2] [--scenes 8] [--iterations 20] [--pool 64]

Builds a batch of the tall scenes (more than 512 rows) among the first `pool`
scenes of the batched-form generator (the class of scenes that dominates a
full step), pins every PCG
solve to a fixed iteration count so that one launch is short and identical
from run to run, and runs three updates.  It prints the PCG time of each
update; it is not a benchmark (bench.py is).
"""
from __future__ import annotations

import argparse

from . import FP32, Batch, FluidSolver
from . import scenes as SC


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--shape", default="64,1,2", help="threads,strips_per_block,stages of the PCG launch")
    ap.add_argument("--scenes", type=int, default=8)
    ap.add_argument("--iterations", type=int, default=20)
    ap.add_argument("--updates", type=int, default=3)
    ap.add_argument("--pool", type=int, default=64, help="generator scenes the tall ones are taken from")
    a = ap.parse_args(argv)
    threads, k, stages = (int(x) for x in a.shape.split(","))
    sc = [s for s in SC.batch_scenes(count=a.pool, seed=2) if s.h > 512][:a.scenes]
    print("scenes", len(sc), "cells", sum(s.w * s.h for s in sc), flush=True)
    members = [FluidSolver(s.w, s.h, s.density, list(s.bodies), precision=FP32) for s in sc]
    for m in members:
        m.set_pinned_iterations(a.iterations, -1)
    b = Batch(members, threads=threads, strips_per_block=k, stages=stages, use_graph=False)
    for i, s in enumerate(sc):
        b.set_inflows(i, s.inflows)
    for u in range(a.updates):
        b.update(sc[0].dt)
        print(u, round(b.info()["last_pcg_ms"], 3), "ms", [x[0][0] for x in b.stats()], flush=True)
    b.close()


if __name__ == "__main__":
    main()
