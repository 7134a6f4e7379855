"""Host logic of the serving loop (no GPU): batching order, per-patch frame order, busy
patches, admission by free device memory with eviction and shrinking."""
import random

import pytest

from mesolf_gb300.serve import Request, Scheduler


def make(n=4, max_batch=2, free=10**12, plan=lambda key: 100 * len(key), evict=lambda: False):
    return Scheduler(n, max_batch, plan, lambda: free if not callable(free) else free(), evict)


def test_oldest_first_and_max_batch():
    s = make(max_batch=2)
    s.add(Request(2, 0, None, 1.0))
    s.add(Request(0, 0, None, 3.0))
    s.add(Request(1, 0, None, 2.0))
    reqs = s.pick(lambda k: False)
    assert sorted(r.patch for r in reqs) == [1, 2]
    assert s.busy == {1, 2}
    assert [r.patch for r in s.pick(lambda k: False)] == [0]
    assert s.pick(lambda k: False) == []


def test_busy_patch_waits_and_frames_stay_in_order():
    s = make(max_batch=4)
    s.add(Request(0, 0, None, 0.0))
    s.add(Request(0, 1, None, 0.1))
    a = s.pick(lambda k: False)
    assert [(r.patch, r.frame) for r in a] == [(0, 0)]
    assert s.pick(lambda k: False) == []          # frame 1 waits for frame 0
    s.done([0])
    assert [(r.patch, r.frame) for r in s.pick(lambda k: False)] == [(0, 1)]
    with pytest.raises(ValueError):
        s.add(Request(0, 1, None, 0.2))           # frames must increase per patch


def test_admission_evicts_then_shrinks():
    evicted = []
    free = {"v": 250}

    def evict():
        if not evicted:
            evicted.append(1)
            free["v"] += 50
            return True
        return False

    s = Scheduler(4, 4, lambda key: 100 * len(key), lambda: free["v"], evict, reserve_bytes=0)
    for p in range(4):
        s.add(Request(p, 0, None, float(p)))
    reqs = s.pick(lambda k: False)
    # 400 > 250 -> evict (300) -> shrink to 3 patches (300 fits)
    assert evicted == [1]
    assert [r.patch for r in reqs] == [0, 1, 2]
    assert s.pending() == 1


def test_cached_composition_needs_no_memory():
    s = make(free=0)
    s.add(Request(0, 0, None, 0.0))
    s.add(Request(1, 0, None, 0.0))
    assert s.pick(lambda k: False) == []
    assert [r.patch for r in s.pick(lambda k: k == (0, 1))] == [0, 1]


def test_simulated_lanes_process_everything_once_in_order():
    rnd = random.Random(3)
    s = make(n=6, max_batch=3)
    t = 0.0
    for f in range(5):
        for p in range(6):
            t += rnd.random()
            s.add(Request(p, f, None, t))
    seen = {p: [] for p in range(6)}
    inflight = []
    while s.pending() or inflight:
        if inflight and (len(inflight) == 2 or rnd.random() < 0.5 or not s.ready()):
            done = inflight.pop(rnd.randrange(len(inflight)))
            s.done([r.patch for r in done])
            continue
        reqs = s.pick(lambda k: False)
        for r in reqs:
            seen[r.patch].append(r.frame)
        if reqs:
            inflight.append(reqs)
        assert len({r.patch for b in inflight for r in b}) == sum(len(b) for b in inflight)
    assert all(v == list(range(5)) for v in seen.values())


def test_drop_stale_takes_the_newest_frame():
    s = Scheduler(2, 2, lambda key: 0, lambda: 1, lambda: False, drop_stale=True)
    for f in range(3):
        s.add(Request(0, f, None, float(f)))
    s.add(Request(1, 0, None, 0.5))
    reqs = s.pick(lambda k: True)
    assert [(r.patch, r.frame) for r in reqs] == [(0, 2), (1, 0)]
    assert [(r.patch, r.frame) for r in s.dropped] == [(0, 0), (0, 1)]
    assert s.pending() == 0


def test_remove_queued_request():
    s = make()
    s.add(Request(0, 0, None, 0.0))
    s.add(Request(0, 1, None, 0.1))
    r = s.remove(0, 1)
    assert r is not None and r.frame == 1
    assert s.remove(0, 5) is None
    assert [(x.patch, x.frame) for x in s.pick(lambda k: True)] == [(0, 0)]
    assert s.pending() == 0
