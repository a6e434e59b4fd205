"""Continuous-batching solve server.

Requests (workloads.Domain: kind, size, step count, storage) arrive over
time.  The server keeps every admitted domain's state resident on the
device, admits queued requests in arrival order as soon as the HBM budget
and the slot limit allow, and advances all resident domains together in
chunks of steps (one rr_batch_step per chunk).  A chunk ends when the
first resident domain reaches its step count (or after max_chunk steps, so
that arrivals never wait longer than one chunk to join); finished domains
hand their result to on_result and leave, freeing their memory for the
queue.  Each domain's arithmetic is the same as when it runs alone.

The device side is a backend object (GpuBackend here; tests substitute a
host-only fake), so the scheduling logic runs and is tested without a GPU.
"""
import collections
import re
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


class GpuBackend:
    """Resident domains as rr_solver members of one rr_batch."""

    READOUT_BYTES_PER_NODE = 40  # FP64 rho, u, tau_t scratch a readout allocates

    def __init__(self, device=0, mode=1, chains=16):
        """mode 1 (default): the members' own launches fanned over `chains`
        parallel graph branches; mode 0: one persistent batch kernel per step
        (rr_batch_set_mode)"""
        import rrlbm

        self._rr = rrlbm
        self.device = device
        self.batch = rrlbm.Batch(device)
        self.batch.set_mode(mode, chains)
        self.members = []  # handles in order of addition (the batch's member order)

    def bytes_for(self, d):
        from .workloads import params_of

        return self._rr.bytes_for(params_of(d)) + self.READOUT_BYTES_PER_NODE * d.nodes

    def start(self, d):
        from .workloads import macros_on_device, params_of

        s = self._rr.Solver(params_of(d))
        rho, ux, uy, uz = macros_on_device(d, f"cuda:{self.device}")
        s.init_state(rho, ux, uy, uz)
        self.batch.add(s)  # waits for the solver's upload: the fields may go
        self.members.append(s)
        return s

    def step(self, n):
        self.batch.step(n)

    def sync(self):
        """None, or the index (order of addition) of a member whose watchdog fired"""
        try:
            self.batch.sync()
            return None
        except self._rr.RRError as e:
            if e.code != 5:
                raise
            m = re.search(r"member (\d+)", str(e))
            return int(m.group(1)) if m else 0

    def finish(self, h, on_result=None):
        res = on_result(h) if on_result else None
        self.batch.remove(h)
        self.members.remove(h)
        h.close()
        return res

    def close(self):
        for h in list(self.members):
            self.finish(h)
        self.batch.close()


class Server:
    def __init__(self, backend, budget_bytes, max_chunk=500, max_active=None, on_result=None,
                 clock=time.perf_counter, sleep=time.sleep):
        self.backend = backend
        self.budget = int(budget_bytes)
        self.max_chunk = int(max_chunk)
        self.max_active = max_active
        self.on_result = on_result
        self.clock = clock
        self.sleep = sleep
        self.chunks = 0
        self.peak_bytes = 0
        self.peak_active = 0

    def run(self, requests):
        """Serve requests (sorted by arrival, seconds from the start);
        returns one Record per request, in request order."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        recs = {r.rid: Record(r.rid, r.arrival, r.nodes, r.steps) for r in reqs}
        queue = collections.deque()
        active = []  # [request, handle, bytes, remaining steps]
        used = 0
        i = 0
        t0 = self.clock()
        while i < len(reqs) or queue or active:
            now = self.clock() - t0
            while i < len(reqs) and reqs[i].arrival <= now:
                queue.append(reqs[i])
                i += 1
            # admission in arrival order, by memory budget and slot limit
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
                active.append([r, h, b, r.steps])
                recs[r.rid].admit = self.clock() - t0
            self.peak_bytes = max(self.peak_bytes, used)
            self.peak_active = max(self.peak_active, len(active))
            if not active:
                if i < len(reqs):
                    wait = reqs[i].arrival - (self.clock() - t0)
                    if wait > 0:
                        self.sleep(wait)
                continue
            chunk = min(self.max_chunk, min(a[3] for a in active))
            self.backend.step(chunk)
            self.chunks += 1
            for a in active:
                a[3] -= chunk
            bad = self.backend.sync()
            now = self.clock() - t0
            while bad is not None:
                # the member that blew up leaves with an error; the others go on
                a = next(x for x in active if x[1] is self.backend.members[bad])
                self.backend.finish(a[1])
                recs[a[0].rid].error = "watchdog: density out of range or NaN"
                recs[a[0].rid].done = now
                used -= a[2]
                active.remove(a)
                bad = self.backend.sync()
            for a in [x for x in active if x[3] == 0]:
                recs[a[0].rid].result = self.backend.finish(a[1], self.on_result)
                recs[a[0].rid].done = self.clock() - t0
                used -= a[2]
                active.remove(a)
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
    }
