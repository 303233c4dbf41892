"""The serving loop's host logic without a GPU (ifl_server_* in dry-run mode):
first-come-first-served admission under the HBM budget and the member cap,
retirement after the requested steps, release of device state, latency
bookkeeping; and the device-size model (ifl_device_bytes)."""
import pytest


@pytest.fixture
def srv_factory(ifl):
    made = []

    def make(**kw):
        s = ifl.Server(dry_run=True, **kw)
        made.append(s)
        return s
    yield make
    for s in made:
        s.close()


def drain(s, limit=100):
    done = []
    for _ in range(limit):
        a, q = s.step()
        done += s.completions()
        if a == 0 and q == 0:
            break
    return done


def test_device_bytes_grow_with_size_and_precision(ifl):
    b64 = ifl.device_bytes(4, 512, 512, ifl.FP64)
    b32 = ifl.device_bytes(4, 512, 512, ifl.FP32)
    assert 0 < b32 < b64
    assert ifl.device_bytes(4, 1024, 1024, ifl.FP32) > 3.5 * b32
    assert ifl.device_bytes(7, 512, 512, ifl.FP32) > b32  # temperature + densities
    assert ifl.device_bytes(3, 512, 512, ifl.FP32) < b32   # no solid fields


def test_requests_finish_after_their_steps_in_fcfs_order(ifl, srv_factory):
    s = srv_factory()
    ids = [s.submit(64, 64, n) for n in (3, 1, 2)]
    done = drain(s)
    assert [c["id"] for c in done] == [ids[1], ids[2], ids[0]]
    for c in done:
        assert c["arrival"] <= c["admitted"] <= c["finished"]
    assert s.info()["cell_steps"] == 64 * 64 * 6
    assert s.info()["steps"] == 3


def test_budget_admits_in_arrival_order_and_release_frees_it(ifl, srv_factory):
    one = ifl.device_bytes(4, 128, 128, ifl.FP32)
    s = srv_factory(hbm_budget_bytes=2 * one + one // 2)
    ids = [s.submit(128, 128, 1) for _ in range(4)]
    a, q = s.step()
    assert (a, q) == (0, 2)  # two admitted, both done after one step, still holding memory
    done = s.completions()
    assert [c["id"] for c in done] == ids[:2]
    a, q = s.step()
    assert q == 2  # nothing released yet: the head of the queue waits
    for c in done:
        s.release(c["id"])
    a, q = s.step()
    assert q == 0
    assert [c["id"] for c in s.completions()] == ids[2:]


def test_head_of_line_waits_even_if_a_later_one_fits(ifl, srv_factory):
    small = ifl.device_bytes(4, 64, 64, ifl.FP32)
    big = ifl.device_bytes(4, 512, 512, ifl.FP32)
    s = srv_factory(hbm_budget_bytes=big + small)
    first = s.submit(512, 512, 5)
    second = s.submit(512, 512, 1)   # does not fit next to the first
    third = s.submit(64, 64, 1)      # would fit, but arrives after the second
    s.step()
    assert s.info()["active"] == 1 and s.info()["queued"] == 2
    done = []
    for _ in range(20):
        s.step()
        for c in s.completions():
            done.append(c["id"])
            s.release(c["id"])
    assert done == [first, second, third]


def test_member_cap(ifl, srv_factory):
    s = srv_factory(max_active=2)
    for _ in range(5):
        s.submit(32, 32, 2)
    a, q = s.step()
    assert (a, q) == (2, 3)


def test_oversized_request_is_refused(ifl, srv_factory):
    s = srv_factory(hbm_budget_bytes=ifl.device_bytes(4, 64, 64, ifl.FP32))
    with pytest.raises(ifl.IflError):
        s.submit(1024, 1024, 1)


@pytest.mark.parametrize("bad", [dict(w=1, h=64, steps=1), dict(w=64, h=64, steps=0),
                                 dict(w=64, h=64, steps=1, inflows=[(0, 0, 1, 1, 1, 0, 0)] * 9)])
def test_bad_requests(ifl, srv_factory, bad):
    s = srv_factory()
    with pytest.raises(ifl.IflError):
        s.submit(**bad)


def test_latency_bookkeeping_uses_caller_arrival(ifl, srv_factory):
    s = srv_factory()
    t = s.now()
    rid = s.submit(64, 64, 1, arrival=t - 5.0)  # arrived five seconds ago
    done = drain(s)
    assert done[0]["id"] == rid and done[0]["finished"] - done[0]["arrival"] >= 5.0
