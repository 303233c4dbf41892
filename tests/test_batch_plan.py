"""Host logic of the batched PCG launch (no GPU): how the blocks of one
cooperative launch are split into teams, and argument checks of the batch ABI."""
import ctypes as C

import numpy as np
import pytest


def test_every_needed_team_size_gets_a_team(ifl):
    strips = [1, 2, 3, 5, 9, 17, 32]  # K = 4: teams of 1, 1, 1, 2, 4, 8, 8 blocks
    used, teams = ifl.plan_teams(152, 4, strips, [1.0] * len(strips))
    assert teams[0] >= 1 and teams[1] >= 1 and teams[2] >= 1 and teams[3] >= 1
    assert used == sum(t << c for c, t in enumerate(teams)) and used <= 152


def test_blocks_go_where_the_work_is(ifl):
    # 40 tall scenes with much work, 40 short ones with little
    strips = [32] * 40 + [2] * 40
    work = [1000.0] * 40 + [1.0] * 40
    used, teams = ifl.plan_teams(152, 4, strips, work)
    assert teams[3] * 8 >= 100  # most blocks serve the 8-block class
    assert teams[0] >= 1
    assert used <= 152


def test_no_more_teams_than_scenes(ifl):
    used, teams = ifl.plan_teams(1000, 2, [4, 4, 4], [5.0, 5.0, 5.0])
    assert teams[1] == 3 and sum(teams) == 3 and used == 6


def test_finish_bound_by_largest_scene_stops_growth(ifl):
    # one huge scene and many tiny ones of the same class: extra teams cannot
    # finish earlier than the huge scene, so growth stops once the rest fits
    work = [1000.0] + [1.0] * 50
    used, teams = ifl.plan_teams(152, 4, [4] * 51, work)
    assert 1 <= teams[0] <= 51
    assert used < 152


def test_grid_too_small_is_rejected(ifl):
    with pytest.raises(ifl.IflError):
        ifl.plan_teams(8, 4, [32, 1], [1.0, 1.0])  # needs 8 + 1 blocks


@pytest.mark.parametrize("args", [(0, 4, [1], [1.0]), (10, 0, [1], [1.0]), (10, 4, [0], [1.0]),
                                  (10, 4, [1], [-1.0])])
def test_bad_arguments(ifl, args):
    with pytest.raises(ifl.IflError):
        ifl.plan_teams(*args)


def test_random_plans_are_consistent(ifl):
    rng = np.random.default_rng(5)
    for _ in range(50):
        n = int(rng.integers(1, 600))
        strips = rng.integers(1, 33, size=n)
        work = rng.uniform(0, 100, size=n)
        K = int(rng.choice([1, 2, 4]))
        grid = int(rng.choice([152, 304, 456, 608]))
        need = {int(np.ceil(np.log2(max(1, -(-s // K))))) for s in strips}
        if sum(1 << c for c in need) > grid:
            continue
        used, teams = ifl.plan_teams(grid, K, strips.tolist(), work.tolist())
        assert used == sum(t << c for c, t in enumerate(teams)) <= grid
        for c in range(8):
            count = sum(1 for s in strips if int(np.ceil(np.log2(max(1, -(-s // K))))) == c)
            assert (teams[c] >= 1) == (count > 0)
            assert teams[c] <= count


def test_batch_options_defaults(ifl):
    o = ifl.BatchOptions()
    ifl.load_library().ifl_batch_default_options(C.byref(o))
    assert (o.threads, o.use_graph, o.tune_iterations) == (0, 1, 8)
    assert o.tile_tune == 1 and list(o.tile_w) == [32] * 8 and list(o.tile_h) == [8] * 8
    assert C.sizeof(o) == 8 * 4 + 2 * 8 * 4  # the C struct: 6 ints, tile_tune, pad, two int[8]


def test_batch_create_rejects_empty(ifl):
    L = ifl.load_library()
    h = C.c_void_p()
    assert L.ifl_batch_create(None, 0, None, C.byref(h)) == ifl.ERR_ARG
    assert not h.value
    assert L.ifl_batch_update(None, 0.01) == ifl.ERR_ARG
    assert L.ifl_batch_destroy(None) == ifl.ERR_ARG
