"""Continuous-batching solve server.

Requests (workloads.Domain: kind, size, step count, storage) arrive over
time.  The server keeps every admitted domain's state resident on the
device and admits queued requests in arrival order as soon as the HBM budget
and the slot limit allow.  Each resident domain advances on its own CUDA
stream in chunks of steps; the GPU runs the chunks of all resident domains
concurrently, and the host never waits for the whole set: it polls each
domain's stream, enqueues the next chunk of a domain whose chunk has
finished (so a small solve is never held back by a large one), hands a
finished domain's result to on_result and frees its memory for the queue.
Admission (the upload of a new domain's start state, asynchronous on its
stream) runs while the other domains' chunks are on the GPU.  Each domain's
arithmetic is the same as when it runs alone.

The device side is a backend object (GpuBackend here; tests substitute a
host-only fake), so the scheduling logic runs and is tested without a GPU.
"""
import collections
import time
from dataclasses import dataclass

import numpy as np


@dataclass
class Record:
    rid: int
    arrival: float
    nodes: int
    steps: int
    admit: float = float("nan")
    done: float = float("nan")
    error: str = ""
    result: object = None

    @property
    def queued(self):
        return self.admit - self.arrival

    @property
    def device(self):
        return self.done - self.admit

    @property
    def latency(self):
        return self.done - self.arrival


class _Member:
    """a resident domain: its solver and the start fields its asynchronous
    upload still reads"""

    def __init__(self, solver, keep):
        self.solver = solver
        self.keep = keep


class GpuBackend:
    """Resident domains as rr_solver objects, each on its own stream."""

    READOUT_BYTES_PER_NODE = 40  # FP64 rho, u, tau_t scratch a readout allocates

    def __init__(self, device=0):
        import rrlbm

        self._rr = rrlbm
        self.device = device
        self.members = []

    def bytes_for(self, d):
        from .workloads import params_of

        return self._rr.bytes_for(params_of(d)) + self.READOUT_BYTES_PER_NODE * d.nodes

    def start(self, d):
        """create the domain and enqueue its state upload (asynchronous)"""
        from .workloads import macros_on_device, params_of

        s = self._rr.Solver(params_of(d))
        # generated on torch's stream, read by the solver's upload on its own
        # stream after an event: no host synchronisation with the other
        # resident domains' work
        fields = macros_on_device(d, f"cuda:{self.device}", stream=s.stream)
        s.init_state(*fields)
        h = _Member(s, fields)
        self.members.append(h)
        return h

    def advance(self, h, n):
        """enqueue n steps of h on its stream"""
        h.solver.step(n)

    def ready(self, h):
        """h's enqueued work has finished (does not wait)"""
        if h.solver.busy():
            return False
        h.keep = None  # the upload has read the start fields
        return True

    def healthy(self, h):
        """h's watchdog has not fired (call once h is ready)"""
        try:
            h.solver.sync()
            return True
        except self._rr.RRError as e:
            if e.code != 5:
                raise
            return False

    def finish(self, h, on_result=None):
        res = on_result(h.solver) if on_result else None
        self.members.remove(h)
        h.solver.close()
        return res

    def close(self):
        for h in list(self.members):
            self.finish(h)


class Server:
    def __init__(self, backend, budget_bytes, max_chunk=2000, max_active=None, on_result=None,
                 clock=time.perf_counter, sleep=time.sleep, poll_s=2e-4):
        self.backend = backend
        self.budget = int(budget_bytes)
        self.max_chunk = int(max_chunk)
        self.max_active = max_active
        self.on_result = on_result
        self.clock = clock
        self.sleep = sleep
        self.poll_s = poll_s
        self.chunks = 0
        self.peak_bytes = 0
        self.peak_active = 0

    def run(self, requests):
        """Serve requests (sorted by arrival, seconds from the start);
        returns one Record per request, in request order."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        recs = {r.rid: Record(r.rid, r.arrival, r.nodes, r.steps) for r in reqs}
        queue = collections.deque()
        active = []  # [request, handle, bytes, steps not yet enqueued, steps of the chunk in flight]
        used = 0
        i = 0
        t0 = self.clock()

        def enqueue(a):
            n = min(self.max_chunk, a[3])
            self.backend.advance(a[1], n)
            a[3] -= n
            a[4] = n
            self.chunks += 1

        while i < len(reqs) or queue or active:
            now = self.clock() - t0
            while i < len(reqs) and reqs[i].arrival <= now:
                queue.append(reqs[i])
                i += 1
            # admission in arrival order, by memory budget and slot limit; a
            # new domain's upload and first chunk go in behind the others'
            while queue and (self.max_active is None or len(active) < self.max_active):
                r = queue[0]
                b = self.backend.bytes_for(r)
                if b > self.budget:
                    queue.popleft()
                    recs[r.rid].error = f"needs {b} bytes, budget {self.budget}"
                    recs[r.rid].admit = recs[r.rid].done = self.clock() - t0
                    continue
                if used + b > self.budget:
                    break
                queue.popleft()
                h = self.backend.start(r)
                used += b
                a = [r, h, b, r.steps, 0]
                active.append(a)
                recs[r.rid].admit = self.clock() - t0
                enqueue(a)
            self.peak_bytes = max(self.peak_bytes, used)
            self.peak_active = max(self.peak_active, len(active))
            # completions: per domain, without waiting for the others
            progressed = False
            for a in list(active):
                if not self.backend.ready(a[1]):
                    continue
                progressed = True
                rec = recs[a[0].rid]
                if not self.backend.healthy(a[1]):
                    # the domain that blew up leaves with an error; the others go on
                    self.backend.finish(a[1])
                    rec.error = "watchdog: density out of range or NaN"
                elif a[3] > 0:
                    enqueue(a)
                    continue
                else:
                    rec.result = self.backend.finish(a[1], self.on_result)
                rec.done = self.clock() - t0
                used -= a[2]
                active.remove(a)
            if progressed:
                continue
            # nothing finished: wait a poll interval, or until the next arrival
            # when nothing is resident
            wait = self.poll_s
            if not active and i < len(reqs):
                wait = max(reqs[i].arrival - (self.clock() - t0), 0.0)
            if wait > 0:
                self.sleep(wait)
        return [recs[r.rid] for r in requests]


def summarize(records):
    """solves/s, LUP/s and latency percentiles of a finished run"""
    ok = [r for r in records if not r.error]
    if not ok:
        return {"completed": 0, "failed": len(records)}
    t_first = min(r.arrival for r in records)
    t_last = max(r.done for r in ok)
    span = t_last - t_first
    lat = np.array([r.latency for r in ok])
    q = np.array([r.queued for r in ok])
    dev = np.array([r.device for r in ok])
    lups = float(sum(r.nodes * r.steps for r in ok))
    pct = lambda a, p: float(np.percentile(a, p))
    return {
        "completed": len(ok),
        "failed": len(records) - len(ok),
        "makespan_s": span,
        "solves_per_s": len(ok) / span if span > 0 else float("inf"),
        "mlups": lups / span / 1e6 if span > 0 else float("inf"),
        "latency_p50_s": pct(lat, 50),
        "latency_p99_s": pct(lat, 99),
        "queue_p50_s": pct(q, 50),
        "queue_p99_s": pct(q, 99),
        "device_p50_s": pct(dev, 50),
        "device_p99_s": pct(dev, 99),
        "by_size": by_size(ok),
    }


SIZE_CLASSES = ((0, 48 ** 3, "n <= 48"), (48 ** 3, 96 ** 3, "48 < n <= 96"), (96 ** 3, float("inf"), "n > 96"))


def by_size(records):
    """latency percentiles per cube-size class (n^3 nodes)"""
    out = {}
    for lo, hi, name in SIZE_CLASSES:
        sel = [r.latency for r in records if lo < r.nodes <= hi]
        if sel:
            out[name] = {"count": len(sel), "latency_p50_s": float(np.percentile(sel, 50)),
                         "latency_p99_s": float(np.percentile(sel, 99))}
    return out
