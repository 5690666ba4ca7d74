"""Continuous-batching request server for the GPU inverses.

Requests (one sinogram each, of any supported N) queue per size. Each size has a lane: a device pipeline with a fixed
number of slots (its batch) captured in a CUDA graph, on its own CUDA stream, so batches of different sizes run
concurrently on the GPU. Whenever a lane is idle and requests of its size wait, up to `slots` of them are packed into
its pinned staging buffer, copied in, the graph is replayed and the results are copied back, all stream-ordered; the
lane is busy until its completion event fires, and requests that arrive meanwhile are admitted into the next batch
as soon as the slots free up (a batch never waits to fill). A lane for a new size is created only if its device
memory (estimated before anything is allocated) fits the HBM budget beside the lanes that exist; idle lanes with no
waiting requests are evicted, least recently used first, to make room, and otherwise the new size waits. A batch's
state (sinograms, packed rows, iterates) stays on the device for its whole inverse.

make_inverse(n) builds (or loads) the inverse of size 2^n; its plan setup runs on the first request of that size,
so a caller that cannot afford it in the request path builds the inverses before serving.
"""

import time
from collections import deque

import numpy as np
import torch

from .device import Pipeline


class Request:
    __slots__ = ("rid", "n", "b", "t_arrival", "t_start", "t_done", "result", "error")

    def __init__(self, rid, n, b, t_arrival=0.0):
        self.rid, self.n, self.b, self.t_arrival = rid, n, b, t_arrival
        self.t_start = self.t_done = None
        self.result = None
        self.error = None  # set when the batch's device work reported a failure (result is then None)


class Lane:
    """One size: captured pipeline, stream, pinned staging buffers, the batch in flight."""

    def __init__(self, inverse, slots, device):
        self.inv, self.slots = inverse, int(slots)
        self.N = inverse.N
        self.stream = torch.cuda.Stream(device=device)
        with torch.cuda.stream(self.stream):  # the lane's own pipeline: nothing shared with inverse.apply()
            self.pipe = Pipeline(inverse.plan, self.slots, inverse.precision, device, inverse.stencil_precision).capture()
        self.stream.synchronize()
        self.stage_in = torch.zeros((self.slots, 4, 2 * self.N - 1, self.N), dtype=torch.float64, pin_memory=True)
        self.stage_out = torch.empty((self.slots, self.N, self.N), dtype=torch.float64, pin_memory=True)
        self.batch = None
        self.event = None

    @staticmethod
    def estimate_bytes(inverse, slots):
        return Pipeline.estimate_bytes(inverse.plan, slots, inverse.precision, inverse.stencil_precision)

    def device_bytes(self):
        return self.pipe.device_bytes()

    def launch(self, reqs):
        """Start one batch: each sinogram is copied into the graph's input slot (directly from a pinned tensor,
        otherwise through the lane's pinned staging buffer), the graph replays, and the results of the used slots
        are copied back, all on the lane's stream. Unused slots keep the previous batch's (finite) data and their
        results are dropped."""
        with torch.cuda.stream(self.stream):
            for i, r in enumerate(reqs):
                b = r.b
                if isinstance(b, torch.Tensor):
                    # device tensors and pinned host tensors copy straight in (copy_ casts the dtype); pageable host
                    # tensors too, synchronously
                    self.pipe.b_in[i].copy_(b, non_blocking=b.is_cuda or b.is_pinned())
                    continue
                self.stage_in[i].copy_(torch.from_numpy(np.ascontiguousarray(b, dtype=np.float64)))
                self.pipe.b_in[i].copy_(self.stage_in[i], non_blocking=True)
            x = self.pipe.replay()
            k = len(reqs)
            self.stage_out[:k].copy_(x[:k], non_blocking=True)
            self.event = torch.cuda.Event()
            self.event.record(self.stream)
        self.batch = reqs

    def done(self):
        return self.batch is not None and self.event.query()

    def collect(self, keep=None):
        """The finished batch; each request's result is copied out of the staging buffer unless keep(r) is false.
        If the batch's tensor-core dense-row launch gave up on a bounded wait (the library's error flag, read here
        after the completion event, so without an extra synchronisation), no result is delivered: every request
        of the batch gets result None and its error set."""
        out = self.batch
        self.batch = None
        try:
            self.pipe.tables.raise_if_error()
        except RuntimeError as e:
            for r in out:
                r.result, r.error = None, str(e)
            return out
        for i, r in enumerate(out):
            r.result = self.stage_out[i].clone() if keep is None or keep(r) else None
        return out

    def release(self):
        """Drop the captured graph and the pipeline's buffers."""
        self.pipe = None


class InverseServer:
    """make_inverse(key) -> FastHybridGpu / FastLpGpu for a request key (its size n, or any hashable class such as
    (n, method, p)); slots(key) -> batch slots of that key's lane. Request.n holds the key."""

    lane_cls = Lane

    def __init__(self, make_inverse, slots, hbm_budget_bytes=120e9, device="cuda", keep_result=None):
        self.make_inverse, self.slots, self.budget = make_inverse, slots, float(hbm_budget_bytes)
        self.keep_result = keep_result  # keep_result(request) -> bool; None keeps every result
        self.device = torch.device(device)
        self.inverses, self.lanes, self.queues, self.last_used = {}, {}, {}, {}
        self.finished = []
        self.clock = time.perf_counter
        self.evictions = 0
        self.max_busy = 0  # most lanes seen with a batch in flight at once

    def memory_in_use(self):
        return sum(l.device_bytes() for l in self.lanes.values())

    def _admit_lane(self, n):
        """The lane of size n, created if the budget allows (evicting idle lanes without waiting requests); None
        while it does not fit."""
        if n in self.lanes:
            return self.lanes[n]
        if n not in self.inverses:
            self.inverses[n] = self.make_inverse(n)
        inv = self.inverses[n]
        need = self.lane_cls.estimate_bytes(inv, self.slots(n))
        if need > self.budget:
            raise MemoryError(f"a lane for n={n} needs {need} bytes, above the budget of {self.budget:.0f}")
        victims = sorted((self.last_used[m], m) for m, l in self.lanes.items() if l.batch is None and not self.queues.get(m))
        while self.memory_in_use() + need > self.budget and victims:
            _, m = victims.pop(0)
            self.lanes.pop(m).release()
            self.evictions += 1
        if self.memory_in_use() + need > self.budget:
            return None
        self.lanes[n] = self.lane_cls(inv, self.slots(n), self.device)
        return self.lanes[n]

    def submit(self, req):
        self.queues.setdefault(req.n, deque()).append(req)

    def pending(self):
        return sum(len(q) for q in self.queues.values()) + sum(len(l.batch) for l in self.lanes.values() if l.batch)

    def step(self):
        """Collect finished batches and start new ones on idle lanes; returns the number of requests waiting or
        in flight."""
        for n, lane in self.lanes.items():
            if lane.done():
                t = self.clock()
                for r in lane.collect(self.keep_result):
                    r.t_done = t
                    self.finished.append(r)
        for n, q in self.queues.items():
            if not q:
                continue
            lane = self._admit_lane(n)
            if lane is None or lane.batch is not None:
                continue
            take = [q.popleft() for _ in range(min(lane.slots, len(q)))]
            t = self.clock()
            for r in take:
                r.t_start = t
            lane.launch(take)
            self.last_used[n] = t
        self.max_busy = max(self.max_busy, sum(1 for l in self.lanes.values() if l.batch is not None))
        return self.pending()

    def run(self, arrivals, poll_sleep=5e-5):
        """Serve (t_offset_seconds, Request) pairs in real time, each submitted at its arrival offset; returns the
        finished requests once all are done."""
        arrivals = sorted(arrivals, key=lambda a: a[0])
        t0 = self.clock()
        i = 0
        while i < len(arrivals) or self.pending():
            now = self.clock() - t0
            while i < len(arrivals) and arrivals[i][0] <= now:
                r = arrivals[i][1]
                r.t_arrival = t0 + arrivals[i][0]
                self.submit(r)
                i += 1
            if not self.step() and i < len(arrivals):
                time.sleep(min(poll_sleep, max(0.0, arrivals[i][0] - (self.clock() - t0))))
        return self.finished

    @staticmethod
    def stats(done):
        lat = np.array([r.t_done - r.t_arrival for r in done])
        span = max(r.t_done for r in done) - min(r.t_arrival for r in done)
        return {"requests": len(done), "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3), "throughput_rps": len(done) / span}


def poisson_arrivals(rate, duration, sizes, probs, seed=0):
    """Arrival offsets of a Poisson process of `rate` per second over `duration` seconds, each with a size drawn
    from `sizes` with probabilities `probs`: [(t, n)]."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            return out
        out.append((t, int(rng.choice(sizes, p=probs))))
