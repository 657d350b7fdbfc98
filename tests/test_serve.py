"""CPU tests of the serving loop's host logic (hephaestus_gb300/serve.py):
Poisson stream generation, HBM-footprint admission, size-class ordering and
the worker loop, driven by a fake executor (no GPU)."""
import threading
import time

import numpy as np
import pytest

from hephaestus_gb300 import serve as S


def test_stream_is_seeded_and_within_ranges():
    a = S.make_stream(200, rate=50.0, seed=3)
    b = S.make_stream(200, rate=50.0, seed=3)
    assert [(r.n, r.p, r.steps, r.seed) for r in a] == [(r.n, r.p, r.steps, r.seed) for r in b]
    t = np.array([r.arrival for r in a])
    assert np.all(np.diff(t) > 0)
    # mean inter-arrival ~ 1/rate
    assert 0.6 / 50 < np.diff(t).mean() < 1.5 / 50
    assert all(r.p in (1, 2, 3) for r in a)
    assert all(r.ndof <= 2e6 for r in a)
    assert min(r.ndof for r in a) < 5e4 and max(r.ndof for r in a) > 5e5
    assert {r.steps for r in a} == {1, 5}


def test_scheduler_respects_budget_slots_and_classes():
    fp = lambda n, p: n * 10  # noqa: E731  (fake footprint: 10 bytes per element row)
    sch = S.Scheduler(budget_bytes=1000, slots=3, footprint=fp)
    small = [S.Request(i, 0.0, 4, 1, 1, i) for i in range(3)]        # class 0, 40 B each
    big = [S.Request(10 + i, 0.0, 60, 3, 1, i) for i in range(2)]    # class 2, 600 B each
    for r in big + small:
        sch.enqueue(r)
    got = []
    while True:
        r = sch.next_admissible()
        if r is None:
            break
        got.append(r.rid)
    # round-robin over classes: a small one, then a big one, then a small one; slots = 3
    assert got == [0, 10, 1]
    assert sch.in_use == 40 + 600 + 40 and sch.running == 3
    sch.release(small[0])
    # the second big request does not fit (680 + 600 > 1000): the next small one is admitted instead
    assert sch.next_admissible().rid == 2
    with pytest.raises(ValueError):
        sch.enqueue(S.Request(99, 0.0, 200, 1, 1, 0))


def test_run_stream_with_fake_executor():
    reqs = S.make_stream(60, rate=400.0, seed=1, dof_range=(1e4, 4e5))
    budget = 3 * max(S.footprint_bytes(r.n, r.p) for r in reqs)
    live = {"bytes": 0, "peak": 0, "conc": 0, "peak_conc": 0}
    lk = threading.Lock()

    def fake(req, w):
        with lk:
            live["bytes"] += S.footprint_bytes(req.n, req.p)
            live["conc"] += 1
            live["peak"] = max(live["peak"], live["bytes"])
            live["peak_conc"] = max(live["peak_conc"], live["conc"])
        time.sleep(1e-3 + req.ndof * 2e-9 * req.steps)
        with lk:
            live["bytes"] -= S.footprint_bytes(req.n, req.p)
            live["conc"] -= 1
        return {"status": "OK", "w": w}

    out, wall = S.run_stream(reqs, fake, budget_bytes=budget, slots=4)
    assert len(out) == 60 and all(r.finish >= r.start >= r.arrival - 1e-3 for r in out)
    assert live["peak"] <= budget
    assert live["peak_conc"] <= 4
    st = S.latency_stats(out)
    assert 0 < st["p50_s"] <= st["p99_s"] <= st["max_s"]
    assert wall >= max(r.arrival for r in reqs)
