"""Continuous-batching request server for the GPU inverses.

Requests (one sinogram each, of any supported N) queue per size. Each size has a lane on its own CUDA stream, so the
lanes of different sizes run concurrently on the GPU. Two kinds of lane:

  SlotLane (the default, slot-level batching): a pipeline of B slots that advances one outer Chebyshev step at a
    time for all slots together, each slot at its own outer iteration (per-slot coefficients on the device). A
    request is admitted into any free slot between two steps: its sinogram is back-projected into the slot (a
    batch-1 pipeline on the lane's stream) and the slot's iterates are cleared; after D steps its result is copied
    out and the slot is free again. So a request never waits for another request's whole inverse, only for one
    step (about D times shorter), and requests of one size overlap on the device at different iterations. Each
    step is a CUDA graph (one per phase of the three rotating iterate buffers).
  Lane (batch-level): the whole inverse of up to B requests as one CUDA graph; new requests wait until the batch in
    flight has finished.

A lane for a new size is created only if its device memory (estimated before anything is allocated) fits the HBM
budget beside the lanes that exist and the memory the device can still give (the driver's free memory plus what the
caching allocator holds unused); idle lanes with no waiting requests are evicted, least recently used first, to
make room, and otherwise the new size waits. A request's state (sinogram, packed rows, iterates) stays on the device
for its whole inverse.

make_inverse(n) builds (or loads) the inverse of size 2^n; its plan setup runs on the first request of that size,
so a caller that cannot afford it in the request path builds the inverses before serving.
"""

import time
from collections import deque

import numpy as np
import torch

from .device import Pipeline, graph_capture
from .plan import outer_coeffs


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

    # the server's lane interface
    def free_slots(self):
        return self.slots if self.batch is None else 0

    def admit(self, reqs):
        self.launch(reqs)

    def poll(self, keep=None):
        return self.collect(keep) if self.done() else []

    def advance(self):
        pass

    def in_flight(self):
        return len(self.batch) if self.batch else 0


class SlotLane:
    """One size with slot-level batching: `slots` images step through the outer Chebyshev iteration together, each
    at its own iteration k (0 .. D); a slot at k = D is free (its iterate is frozen: both per-slot coefficients
    are zero). The step is x_{k+1} = x_k + om_a(k) P(y - G x_k) + om_1(k) (x_k - x_{k-1}) with x_0 = x_{-1} = 0 and
    (om_a(0), om_1(0)) = (a, 0), the reference's outer loop (fastops.py:247-258) written uniformly, so that a slot
    admitted between two steps starts at k = 0 while the others go on."""

    def __init__(self, inverse, slots, device):
        self.inv, self.slots = inverse, int(slots)
        self.N = N = inverse.N
        plan = inverse.plan
        self.D = D = int(plan.outer_deg)
        self.device = torch.device(device)
        self.stream = torch.cuda.Stream(device=self.device)
        # step pipelines over prefixes of the slots (B/8, B/4, B/2, B): a step costs in proportion to the highest
        # occupied slot, and admission fills the lowest free slot, so a lightly loaded lane runs small steps
        self.sizes = sorted({max(1, self.slots >> k) for k in range(4)})
        with torch.cuda.stream(self.stream):
            self.pipe = Pipeline(plan, self.slots, inverse.precision, self.device, inverse.stencil_precision)
            self.sub = {b: (self.pipe if b == self.slots else self.pipe.prefix(b)) for b in self.sizes}
            self.bp = Pipeline(plan, 1, inverse.precision, self.device, inverse.stencil_precision)
            a, _, steps = outer_coeffs(plan.lo, plan.hi, D)
            tab = [(a, 0.0)] + [tuple(st) for st in steps] + [(0.0, 0.0)]
            self.coef_tab = torch.tensor(tab, dtype=torch.float64, device=self.device)  # row D: a frozen slot
            self.k = torch.full((self.slots,), D, dtype=torch.int64, device=self.device)
            self.om = torch.zeros((self.slots, 2), dtype=torch.float64, device=self.device)
            for x in self.pipe.xs:
                x.zero_()
            self.pipe.y.zero_()
            self.b1 = torch.zeros((1, 4, 2 * N - 1, N), dtype=torch.float64, device=self.device)
            for b in self.sizes:  # builds every table and kernel attribute before the capture
                self._step_eager(0, b)
                self._step_eager(1, b)
            self.bp.backproject_into(self.b1, self.pipe.y[:1])
            self.pipe.y.zero_()
        self.stream.synchronize()
        self.graphs = {}
        for b in self.sizes:
            for ph in range(3):
                g = torch.cuda.CUDAGraph()
                with graph_capture(g, self.stream):
                    self._step_eager(ph, b)
                self.graphs[(b, ph)] = g
        self.s = 0  # global step counter (the buffer rotation phase is s % 3)
        self.hk = [D] * self.slots  # host mirror of the per-slot iteration counters
        self.req = [None] * self.slots
        # pinned staging per slot: a slot's staging is written again only at its next admission, after its previous
        # request's result (and so its input copy) has completed
        self.stage_in = torch.zeros((self.slots, 4, 2 * N - 1, N), dtype=torch.float64, pin_memory=True)
        self.stage_out = torch.empty((self.slots, N, N), dtype=torch.float64, pin_memory=True)
        self.out_events = []  # (slot, request, event) of result copies in flight
        self.step_events = deque()  # completion events of the steps in flight (at most `depth`)
        self.depth = 2  # steps queued ahead: the GPU never waits for the host, an admission waits at most 2 steps
        self.steps_run = 0
        self.step_sizes = {}  # prefix size -> steps run at it

    @staticmethod
    def estimate_bytes(inverse, slots):
        """The slot pipeline, the batch-1 back-projection pipeline, the prefix pipelines' dense-row staging and the
        per-slot coefficient state."""
        p = inverse.plan
        N, nd = p.N, 2 * len(p.dense_freqs)
        rs = 4 if inverse.precision == "fp32" else 8
        prefixes = sum(max(1, int(slots) >> k) for k in range(1, 4) if max(1, int(slots) >> k) < int(slots))
        return (Pipeline.estimate_bytes(p, slots, inverse.precision, inverse.stencil_precision, captured=False) +
                Pipeline.estimate_bytes(p, 1, inverse.precision, inverse.stencil_precision, captured=True) +
                nd * prefixes * N * 2 * rs + int(slots) * 24 + (int(p.outer_deg) + 1) * 16)

    def device_bytes(self):
        zd = sum(q.tables._zd.numel() * q.tables._zd.element_size() for b, q in self.sub.items()
                 if q is not self.pipe and q.tables._zd is not None)
        return (self.pipe.device_bytes() + self.bp.device_bytes() + self.b1.numel() * 8 + self.k.numel() * 8 +
                self.om.numel() * 8 + self.coef_tab.numel() * 8 + zd)

    def _bufs(self, ph, xs=None):
        xs = self.pipe.xs if xs is None else xs
        return xs[ph % 3], xs[(ph + 2) % 3], xs[(ph + 1) % 3]  # cur, prev, new

    def _step_eager(self, ph, b):
        """One step of the first b slots (the others keep their state)."""
        q = self.sub[b]
        cur, prev, new = self._bufs(ph, q.xs)
        torch.index_select(self.coef_tab, 0, self.k[:b], out=self.om[:b])
        q.G(cur)
        q.step_all(q.y, cur, prev, new, self.om[:b])
        self.k[:b].add_(1).clamp_(max=self.D)

    # the server's lane interface
    def free_slots(self):
        return sum(1 for r in self.req if r is None)

    def in_flight(self):
        return sum(1 for r in self.req if r is not None) + len(self.out_events)

    def admit(self, reqs):
        """Each request into a free slot, stream-ordered before the next step: its sinogram back-projected into the
        slot's y, the slot's two live iterates cleared, its counter set to 0."""
        free = [i for i, r in enumerate(self.req) if r is None]
        assert len(reqs) <= len(free)
        cur, prev, _ = self._bufs(self.s)
        with torch.cuda.stream(self.stream):
            for i, r in zip(free, reqs):
                b = r.b
                if isinstance(b, torch.Tensor):
                    self.b1[0].copy_(b, non_blocking=b.is_cuda or b.is_pinned())
                else:
                    self.stage_in[i].copy_(torch.from_numpy(np.ascontiguousarray(b, dtype=np.float64)))
                    self.b1[0].copy_(self.stage_in[i], non_blocking=True)
                self.bp.backproject_into(self.b1, self.pipe.y[i:i + 1])
                cur[i].zero_()
                prev[i].zero_()
                self.k[i:i + 1].fill_(0)
                self.req[i] = r
                self.hk[i] = 0

    def advance(self):
        """Queue the next step while some slot is active and fewer than `depth` steps are in flight; the results
        of slots that reach k = D are copied out right after their last step."""
        if not any(r is not None for r in self.req):
            return
        while self.step_events and self.step_events[0].query():
            self.step_events.popleft()
        if len(self.step_events) >= self.depth:
            return
        top = max(i for i, r in enumerate(self.req) if r is not None) + 1
        b = next(sz for sz in self.sizes if sz >= top)
        with torch.cuda.stream(self.stream):
            self.graphs[(b, self.s % 3)].replay()
            self.step_sizes[b] = self.step_sizes.get(b, 0) + 1
            _, _, new = self._bufs(self.s)
            self.s += 1
            self.steps_run += 1
            for i, r in enumerate(self.req):
                if r is None:
                    continue
                self.hk[i] += 1
                if self.hk[i] == self.D:
                    res = self.pipe.result(new[i:i + 1], None if self.pipe.x64 is None else self.pipe.x64[i:i + 1])
                    self.stage_out[i].copy_(res[0], non_blocking=True)
                    ev = torch.cuda.Event()
                    ev.record(self.stream)
                    self.out_events.append((i, r, ev))
                    self.req[i] = None
            ev = torch.cuda.Event()
            ev.record(self.stream)
            self.step_events.append(ev)

    def poll(self, keep=None):
        """Requests whose result copies have completed (device error flags checked first)."""
        done, rest = [], []
        for i, r, ev in self.out_events:
            if ev.query():
                done.append((i, r))
            else:
                rest.append((i, r, ev))
        self.out_events = rest
        if not done:
            return []
        err = None
        try:
            self.pipe.tables.raise_if_error()
            self.bp.tables.raise_if_error()
        except RuntimeError as e:
            err = str(e)
        out = []
        for i, r in done:
            if err is not None:
                r.result, r.error = None, err
            else:
                r.result = self.stage_out[i].clone() if keep is None or keep(r) else None
            out.append(r)
        return out

    def release(self):
        self.graphs = {}
        self.pipe = self.bp = None
        self.sub = {}


class InverseServer:
    """make_inverse(key) -> FastHybridGpu / FastLpGpu for a request key (its size n, or any hashable class such as
    (n, method, p)); slots(key) -> batch slots of that key's lane. Request.n holds the key."""

    lane_cls = SlotLane

    def __init__(self, make_inverse, slots, hbm_budget_bytes=120e9, device="cuda", keep_result=None, lane_cls=None):
        if lane_cls is not None:
            self.lane_cls = lane_cls
        self.make_inverse, self.slots, self.budget = make_inverse, slots, float(hbm_budget_bytes)
        self.keep_result = keep_result  # keep_result(request) -> bool; None keeps every result
        self.device = torch.device(device)
        self.inverses, self.lanes, self.queues, self.last_used = {}, {}, {}, {}
        self.finished = []
        self.clock = time.perf_counter
        self.evictions = 0
        self.max_busy = 0  # most lanes seen with a batch in flight at once
        self.device_free = self._device_free  # bytes the device can still give (replaceable for host tests)

    def memory_in_use(self):
        return sum(l.device_bytes() for l in self.lanes.values())

    def _device_free(self):
        """Free device memory as the driver reports it plus what torch's caching allocator holds unused."""
        if self.device.type != "cuda":
            return float("inf")
        free, _ = torch.cuda.mem_get_info(self.device)
        return free + torch.cuda.memory_reserved(self.device) - torch.cuda.memory_allocated(self.device)

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
        victims = sorted((self.last_used.get(m, 0.0), m) for m, l in self.lanes.items()
                         if not l.in_flight() and not self.queues.get(m))
        # admission by the HBM budget and by what the device can actually still give (other users of the GPU,
        # other allocations of this process)
        def fits():
            return self.memory_in_use() + need <= self.budget and need <= self.device_free()

        while not fits() and victims:
            _, m = victims.pop(0)
            self.lanes.pop(m).release()
            self.evictions += 1
            if self.device.type == "cuda":
                torch.cuda.empty_cache()
        if not fits():
            return None
        self.lanes[n] = self.lane_cls(inv, self.slots(n), self.device)
        return self.lanes[n]

    def submit(self, req):
        self.queues.setdefault(req.n, deque()).append(req)

    def pending(self):
        return sum(len(q) for q in self.queues.values()) + sum(l.in_flight() for l in self.lanes.values())

    def step(self):
        """Collect finished requests, admit waiting ones into free slots, advance the lanes; returns the number of
        requests waiting or in flight."""
        for n, lane in self.lanes.items():
            got = lane.poll(self.keep_result)
            if got:
                t = self.clock()
                for r in got:
                    r.t_done = t
                    self.finished.append(r)
        for n, q in self.queues.items():
            if not q:
                continue
            lane = self._admit_lane(n)
            if lane is None:
                continue
            k = min(lane.free_slots(), len(q))
            if not k:
                continue
            take = [q.popleft() for _ in range(k)]
            t = self.clock()
            for r in take:
                r.t_start = t
            lane.admit(take)
            self.last_used[n] = t
        for lane in self.lanes.values():
            lane.advance()
        self.max_busy = max(self.max_busy, sum(1 for l in self.lanes.values() if l.in_flight()))
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
