"""The C++ drop-in header (include/ifluids.hpp) used the way the reference's own
main() uses FluidSolver: it compiles and links against the library here, and on
a GPU it reproduces the oracle's run of the same scene."""
import math
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_main.cpp")
SRC_FLIP = os.path.join(ROOT, "tests", "cpp", "dropin_flip.cpp")


def _compile(ifl, tmp_path_factory, src, name):
    lib_dir = os.path.dirname(ifl.LIB_PATH)
    exe = str(tmp_path_factory.mktemp("cpp") / name)
    cmd = ["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
           "-I/usr/local/cuda/include", src, "-o", exe, "-L" + lib_dir, "-lifluids",
           "-Wl,-rpath," + lib_dir]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


@pytest.fixture(scope="module")
def dropin_exe(ifl, tmp_path_factory):
    return _compile(ifl, tmp_path_factory, SRC, "dropin_main")


@pytest.fixture(scope="module")
def dropin_flip_exe(ifl, tmp_path_factory):
    return _compile(ifl, tmp_path_factory, SRC_FLIP, "dropin_flip")


def test_dropin_program_compiles_and_links(dropin_exe, dropin_flip_exe):
    assert os.path.exists(dropin_exe) and os.path.exists(dropin_flip_exe)


@pytest.mark.gpu
def test_dropin_program_matches_oracle(dropin_exe):
    out = subprocess.run([dropin_exe, "64", "64", "4"], check=True, capture_output=True, text=True).stdout
    rows = [line.split() for line in out.strip().splitlines()]
    o = O.OracleSolver(4, 64, 64)
    o.set_bodies([(0, 0.5, 0.6, 0.7, 0.1, math.pi * 0.25, 0.0, 0.0, 0.0)])
    for it, dsum in rows:
        o.add_inflow(0.45, 0.2, 0.15, 0.03, 1.0, 0.0, 0.0, 3.0)
        o.update(0.005)
        o.advance_bodies(0.005)
        assert abs(int(it) - o.stats()[0][0]) <= 1
        ref = float(o.array(O.QD, O.A_SRC).sum())
        assert abs(float(dsum) - ref) <= 1e-9 * abs(ref)


@pytest.mark.gpu
def test_dropin_flip_program_matches_oracle(dropin_flip_exe):
    """The step-8 program (update() alone adds the reference's built-in inflow):
    particle counts and PCG iterations equal to the oracle's, density sums
    within 1e-9."""
    out = subprocess.run([dropin_flip_exe, "48", "48", "3"], check=True, capture_output=True, text=True).stdout
    rows = [line.split() for line in out.strip().splitlines()]
    o = O.OracleSolver(O.FLIP, 48, 48, 0.1, 0.25, 0.01)
    o.set_bodies([(0, 0.5, 0.6, 0.7, 0.1, math.pi * 0.25, 0.0, 0.0, 0.0)])
    for count, it, dsum in rows:
        o.add_inflow(0.45, 0.2, 0.2, 0.05, 1.0, 294.0, 0.0, 0.0)
        o.update(0.0025)
        assert int(count) == o.particle_count()
        assert abs(int(it) - o.stats()[0][0]) <= 1
        ref = float(o.array(O.QD, O.A_SRC).sum())
        assert abs(float(dsum) - ref) <= 1e-9 * abs(ref)
