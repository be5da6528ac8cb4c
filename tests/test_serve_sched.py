"""Admission and batching policy of the render server (host logic, no GPU)."""
from dataclasses import dataclass

import pytest

from ubs.serve import Request, Scheduler, ServeConfig


@dataclass
class Cam:
    width: int
    height: int


def make(cfg, per_pixel=1.0, bytes_per_isect=10):
    est = lambda scene, cams: per_pixel * sum(c.width * c.height for c in cams)  # noqa: E731
    cost = lambda scene, cams, cap: cap * bytes_per_isect  # noqa: E731
    return Scheduler(cfg, est, cost)


def reqs(spec):
    return [Request(i, sc, Cam(w, h), 0.01 * i) for i, (sc, w, h) in enumerate(spec)]


def test_batches_take_the_oldest_scene_in_arrival_order():
    s = make(ServeConfig(max_slots=4, max_batch_views=3, mem_budget=1 << 40, margin=1.0))
    s.arrive(reqs([("a", 10, 10), ("b", 10, 10), ("a", 20, 20), ("a", 5, 5), ("a", 5, 5)]))
    scene, chosen, cap, nbytes = s.next_batch()
    assert scene == "a" and [r.rid for r in chosen] == [0, 2, 3]  # capped at 3 views
    assert cap == 100 + 400 + 25 + 4096 and nbytes == cap * 10
    scene, chosen, _, _ = s.next_batch()
    assert scene == "b" and [r.rid for r in chosen] == [1]
    scene, chosen, _, _ = s.next_batch()
    assert scene == "a" and [r.rid for r in chosen] == [4]
    assert s.next_batch() is None and s.slots_busy == 3


def test_slots_bound_admission():
    cfg = ServeConfig(max_slots=2, max_batch_views=1, mem_budget=1 << 40, margin=1.0)
    s = make(cfg)
    s.arrive(reqs([("a", 10, 10)] * 4))
    b1, b2 = s.next_batch(), s.next_batch()
    assert b1 and b2 and s.slots_busy == 2
    assert s.next_batch() is None  # no free slot
    s.release(b1[3])
    assert s.next_batch() is not None and len(s.waiting) == 1


def test_memory_bound_admission():
    # one 100x100 view: (10000 + 4096) * 10 bytes; two fit in the budget, three do not
    cfg = ServeConfig(max_slots=4, max_batch_views=8, mem_budget=300_000, margin=1.0)
    s = make(cfg)
    s.arrive(reqs([("a", 100, 100)] * 5))
    b1 = s.next_batch()
    assert len(b1[1]) == 2 and b1[3] == (20000 + 4096) * 10
    assert s.next_batch() is None  # the next view does not fit beside b1
    s.release(b1[3])
    b2 = s.next_batch()
    assert [r.rid for r in b2[1]] == [2, 3]


def test_oversized_request_waits_for_memory_then_runs_alone():
    cfg = ServeConfig(max_slots=4, max_batch_views=8, mem_budget=50_000, margin=1.0)
    s = make(cfg)
    s.arrive(reqs([("a", 10, 10), ("b", 100, 100)]))
    b1 = s.next_batch()
    assert b1[0] == "a"
    assert s.next_batch() is None  # b does not fit while a is in flight
    s.release(b1[3])
    b2 = s.next_batch()
    assert b2[0] == "b" and s.in_flight_bytes > cfg.mem_budget  # alone, over budget


def test_every_request_is_served_exactly_once():
    import random
    rnd = random.Random(0)
    cfg = ServeConfig(max_slots=3, max_batch_views=4, mem_budget=200_000, margin=1.3)
    s = make(cfg)
    spec = [(rnd.choice("abc"), rnd.choice([8, 16, 32]), rnd.choice([8, 16])) for _ in range(200)]
    s.arrive(reqs(spec))
    served, inflight = [], []
    while s.waiting or inflight:
        b = s.next_batch()
        if b is None:
            done = inflight.pop(0)
            s.release(done[3])
            continue
        assert len({r.scene for r in b[1]}) == 1 and len(b[1]) <= 4
        served += [r.rid for r in b[1]]
        inflight.append(b)
    assert sorted(served) == list(range(200)) and s.in_flight_bytes == 0


def test_intersection_bound_caps_a_batch_but_never_starves_it():
    # 1 intersection per pixel: 100x100 views of 10,000 each; a 25,000 bound
    # takes two views per batch, and a lone view larger than the bound still goes
    cfg = ServeConfig(max_slots=4, max_batch_views=8, mem_budget=1 << 40, margin=1.0,
                      max_batch_isects=25_000)
    s = make(cfg)
    s.arrive(reqs([("a", 100, 100)] * 3 + [("b", 300, 300)]))
    assert [r.rid for r in s.next_batch()[1]] == [0, 1]
    assert [r.rid for r in s.next_batch()[1]] == [2]
    assert [r.rid for r in s.next_batch()[1]] == [3]
    assert s.next_batch() is None
