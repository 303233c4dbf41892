"""Serving loop on the GPU (ifl_server_*): requests that arrive while others
run join the running batch, and every request's result is bit-identical alone
and in the mix (its arithmetic does not depend on the other members)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = dict(threads=128, strips_per_block=1, stages=3)
SPIN = (0, 0.55, 0.55, 0.3, 0.12, 0.7, 0.0, 0.0, 1.0)
BALL = (1, 0.3, 0.45, 0.2, 0.2, 0.0, 0.1, 0.0, 1.0)
REQS = [  # w, h, steps, bodies, inflows
    (96, 64, 4, [SPIN], [(0.45, 0.2, 0.15, 0.05, 1.0, 0.0, 0.0, 3.0)]),
    (64, 130, 6, [BALL], [(0.3, 0.2, 0.3, 0.05, 1.0, 0.0, 0.0, 2.0), (0.6, 0.3, 0.1, 0.05, 1.0, 0.0, 1.0, 1.0)]),
    (150, 40, 3, [], [(0.2, 0.3, 0.4, 0.08, 1.0, 0.0, 0.5, 2.0)]),
    (33, 97, 5, [BALL], [(0.35, 0.15, 0.3, 0.05, 1.0, 0.0, 0.0, 2.0)]),
    (200, 200, 2, [SPIN, BALL], [(0.45, 0.2, 0.1, 0.02, 1.0, 0.0, 0.0, 3.0)]),
]
FIELDS = ("d", "u", "v", "p")


def run(ifl, reqs, precision, stagger):
    """Submit `reqs` (the k-th after k*stagger steps); return results by index."""
    s = ifl.Server(precision=precision, **SHAPE)
    ids, out, pending, overlap = {}, {}, list(range(len(reqs))), 0
    step = 0
    while pending or len(out) < len(reqs):
        for k in list(pending):
            if k * stagger <= step:
                w, h, n, bodies, inflows = reqs[k]
                ids[s.submit(w, h, n, bodies, inflows)] = k
                pending.remove(k)
        a, _ = s.step()
        overlap = max(overlap, a)
        step += 1
        for c in s.completions():
            k = ids[c["id"]]
            assert c["arrival"] <= c["admitted"] <= c["finished"]
            assert s.stats(c["id"])[2] & 1 == 0
            out[k] = [s.read_field(c["id"], f) for f in FIELDS]
            s.release(c["id"])
        assert step < 100
    s.close()
    return out, overlap


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_results_identical_alone_and_in_the_mix(ifl, precision):
    mix, overlap = run(ifl, REQS, precision, stagger=1)
    assert overlap >= 3  # later arrivals joined while earlier ones were running
    for k, r in enumerate(REQS):
        alone, _ = run(ifl, [r], precision, stagger=0)
        for f, a, b in zip(FIELDS, mix[k], alone[0]):
            assert np.array_equal(a, b), (k, f)


def test_budget_limits_concurrency_on_the_device(ifl):
    one = ifl.device_bytes(4, 128, 128, ifl.FP32)
    s = ifl.Server(precision=ifl.FP32, hbm_budget_bytes=2 * one, **SHAPE)
    for _ in range(4):
        s.submit(128, 128, 2, [], [(0.45, 0.2, 0.15, 0.05, 1.0, 0.0, 0.0, 3.0)])
    peak, done = 0, 0
    for _ in range(20):
        a, q = s.step()
        peak = max(peak, a)
        for c in s.completions():
            s.release(c["id"])
            done += 1
        if done == 4:
            break
    assert done == 4 and peak == 2
    s.close()
