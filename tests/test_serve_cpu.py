"""Scheduling logic of the solve server (rrlbm.serve) on a host-only fake
device, and the seeded workload generators (rrlbm.workloads)."""
import numpy as np
import pytest

import rrlbm
from rrlbm import serve, workloads


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 0.0)


class FakeBackend:
    """Resident domains on their own 'streams': a chunk of n steps of a domain
    takes n * nodes / (rate / resident domains) seconds of the fake clock
    (the device's aggregate rate, shared)."""

    def __init__(self, clock, rate=1e9, bad=()):
        self.clock = clock
        self.rate = rate
        self.members = []
        self.bad = set(bad)  # request ids whose watchdog fires
        self.starts = []
        self.used = 0
        self.peak = 0

    def bytes_for(self, d):
        return 100 * d.nodes

    def start(self, d):
        h = {"d": d, "steps": 0, "pending": 0, "until": self.clock.t}
        self.members.append(h)
        self.starts.append(d.rid)
        self.used += self.bytes_for(d)
        self.peak = max(self.peak, self.used)
        return h

    def advance(self, h, n):
        share = self.rate / max(1, len(self.members))
        h["until"] = max(h["until"], self.clock.t) + n * h["d"].nodes / share
        h["pending"] += n

    def ready(self, h):
        if self.clock.t < h["until"]:
            return False
        h["steps"] += h["pending"]
        h["pending"] = 0
        return True

    def healthy(self, h):
        return h["d"].rid not in self.bad

    def finish(self, h, on_result=None):
        res = on_result(h) if on_result else None
        self.members.remove(h)
        self.used -= self.bytes_for(h["d"])
        return res


def _stream(n=40, rate=200.0, seed=1):
    return workloads.request_stream(n, rate=rate, seed=seed, sizes=(8, 24), steps=(10, 200))


def test_all_served_in_order_within_budget():
    clock = FakeClock()
    be = FakeBackend(clock, rate=2e8)
    reqs = _stream()
    budget = 100 * 3 * 24 ** 3
    srv = serve.Server(be, budget, max_chunk=64, on_result=lambda h: h["steps"], clock=clock, sleep=clock.sleep)
    recs = srv.run(reqs)
    assert all(not r.error for r in recs)
    for r, d in zip(recs, reqs):
        assert r.result == d.steps  # exactly its step count, no more
        assert r.arrival <= r.admit <= r.done
    assert be.starts == [d.rid for d in sorted(reqs, key=lambda d: d.arrival)]  # FIFO admission
    assert be.peak <= budget and srv.peak_bytes <= budget
    assert srv.peak_active > 1  # batching happened
    s = serve.summarize(recs)
    assert s["completed"] == len(reqs) and s["latency_p99_s"] >= s["latency_p50_s"] > 0


def test_one_at_a_time_is_sequential_and_slower_to_drain():
    reqs = _stream(30)
    out = {}
    for slots in (None, 1):
        clock = FakeClock()
        be = FakeBackend(clock, rate=2e8)
        srv = serve.Server(be, 10 ** 12, max_chunk=1000, max_active=slots, clock=clock, sleep=clock.sleep)
        recs = srv.run(reqs)
        out[slots] = serve.summarize(recs)
        if slots == 1:
            order = sorted(recs, key=lambda r: r.admit)
            for a, b in zip(order, order[1:]):
                assert b.admit >= a.done
    # a fixed aggregate rate: the same total work, but queueing dominates one-at-a-time
    assert out[1]["latency_p50_s"] >= out[None]["latency_p50_s"]


def test_oversized_request_rejected_and_watchdog_isolated():
    clock = FakeClock()
    reqs = _stream(12)
    big = workloads.Domain("tg", 64, 50, arrival=0.0, rid=999)
    be = FakeBackend(clock, bad={reqs[3].rid})
    srv = serve.Server(be, 100 * 30 ** 3, max_chunk=32, clock=clock, sleep=clock.sleep)
    recs = srv.run(reqs + [big])
    byid = {r.rid: r for r in recs}
    assert "budget" in byid[999].error
    assert "watchdog" in byid[reqs[3].rid].error
    assert sum(1 for r in recs if not r.error) == len(reqs) - 1


def test_request_stream_seeded_and_in_range():
    a = workloads.request_stream(200, seed=7)
    b = workloads.request_stream(200, seed=7)
    assert [(d.kind, d.n, d.steps, d.storage, d.arrival) for d in a] == \
           [(d.kind, d.n, d.steps, d.storage, d.arrival) for d in b]
    t = np.array([d.arrival for d in a])
    assert np.all(np.diff(t) > 0)
    assert 100 < len(a) / t[-1] < 400  # mean rate 200/s
    assert all(32 <= d.n <= 192 and 1000 <= d.steps <= 20000 for d in a)
    assert {d.kind for d in a} == {"tg", "cavity", "channel"} and {d.storage for d in a} == {"f16", "f32"}
    e = workloads.ensemble(256)
    assert len(e) == 256 and {d.kind for d in e} == {"tg", "cavity"}
    for d in e:
        assert (32 <= d.n <= 128) if d.kind == "tg" else (32 <= d.n <= 96)
        if d.kind == "tg":
            assert 0.52 <= d.tau <= 0.8 and 0.01 <= d.Ma <= 0.1
        else:
            assert 100 <= d.Re <= 1000


@pytest.mark.parametrize("kind", ["tg", "cavity", "channel"])
def test_params_of_valid(kind):
    d = workloads.Domain(kind, 40, 100, "f16", tau=0.6, Ma=0.05, Re=500)
    p = workloads.params_of(d)
    assert rrlbm.bytes_for(p) >= 2 * 27 * 40 ** 3 * 2  # validated by the library
    assert rrlbm.bytes_for(workloads.params_of(d, "f64")) > rrlbm.bytes_for(p)
    assert p.tau > 0.5
