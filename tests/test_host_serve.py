"""Host logic of the request server (admission by memory budget, eviction, batching, latency statistics) with a
fake lane in place of the captured GPU pipeline."""
import numpy as np
import pytest


class FakeInverse:
    def __init__(self, n):
        self.n, self.N = n, 1 << n


class FakeLane:
    created = []

    def __init__(self, inv, slots, device):
        self.inv, self.slots, self.batch = inv, slots, None
        FakeLane.created.append(inv.n)
        self.released = False

    @staticmethod
    def estimate_bytes(inv, slots):
        return slots * inv.N * inv.N

    def device_bytes(self):
        return self.slots * self.inv.N * self.inv.N

    def launch(self, reqs):
        assert len(reqs) <= self.slots
        self.batch = reqs

    def done(self):
        return self.batch is not None

    def collect(self, keep=None):
        out, self.batch = self.batch, None
        for r in out:
            r.result = ("x", r.rid, self.inv.n)
        return out

    def release(self):
        self.released = True

    # the server's lane interface (batch-level)
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


class FakeSlotLane(FakeLane):
    """Slot-level: each admitted request finishes D advance() calls later; free slots take new requests at once."""

    D = 3

    def __init__(self, inv, slots, device):
        super().__init__(inv, slots, device)
        self.req = [None] * slots
        self.k = [0] * slots
        self.out = []
        self.steps = 0

    def free_slots(self):
        return sum(r is None for r in self.req)

    def admit(self, reqs):
        free = [i for i, r in enumerate(self.req) if r is None]
        assert len(reqs) <= len(free)
        for i, r in zip(free, reqs):
            self.req[i], self.k[i] = r, 0

    def advance(self):
        if not any(self.req):
            return
        self.steps += 1
        for i, r in enumerate(self.req):
            if r is not None:
                self.k[i] += 1
                if self.k[i] == self.D:
                    r.result = ("x", r.rid, self.inv.n)
                    self.out.append(r)
                    self.req[i] = None

    def poll(self, keep=None):
        out, self.out = self.out, []
        return out

    def in_flight(self):
        return sum(r is not None for r in self.req) + len(self.out)


def _server(pkg, budget, slots=lambda n: 4, lane=FakeLane):
    from adrt_pinv_gb300 import serve

    FakeLane.created = []
    return serve.InverseServer(FakeInverse, slots, hbm_budget_bytes=budget, device="cpu", lane_cls=lane), serve


def test_batches_and_results(pkg):
    S, serve = _server(pkg, budget=1e12)
    reqs = [serve.Request(i, 5 + i % 2, None) for i in range(11)]
    for r in reqs:
        S.submit(r)
    S.step()  # first batches launch: 4 of n=5, 4 of n=6
    assert sorted(len(l.batch) for l in S.lanes.values()) == [4, 4]
    while S.step():
        pass
    assert len(S.finished) == 11
    for r in S.finished:
        assert r.result == ("x", r.rid, r.n)
        assert r.t_start <= r.t_done


def test_budget_admission_and_eviction(pkg):
    # budget fits one lane at a time: the second size waits until the first lane is idle with an empty queue
    S, serve = _server(pkg, budget=4 * 64 * 64 + 1)
    for i in range(6):
        S.submit(serve.Request(i, 5, None))
    S.submit(serve.Request(100, 6, None))
    S.step()
    assert list(S.lanes) == [5] and 6 not in S.lanes
    while S.step():
        pass
    assert len(S.finished) == 7
    assert S.evictions == 1 and FakeLane.created == [5, 6]


def test_lane_over_budget_raises(pkg):
    S, serve = _server(pkg, budget=10)
    S.submit(serve.Request(0, 5, None))
    with pytest.raises(MemoryError):
        S.step()


def test_run_and_stats(pkg):
    S, serve = _server(pkg, budget=1e12)
    arr = serve.poisson_arrivals(2000.0, 0.02, [5, 6], [0.5, 0.5], seed=3)
    assert 10 < len(arr) < 80 and all(0 <= t < 0.02 for t, _ in arr)
    done = S.run([(t, serve.Request(i, n, None)) for i, (t, n) in enumerate(arr)])
    st = serve.InverseServer.stats(done)
    assert st["requests"] == len(arr) and st["p50_ms"] <= st["p99_ms"] and st["throughput_rps"] > 0


def test_pipeline_estimate_matches_buffers(pkg):
    # the estimate counts the same buffers as device_bytes (CPU tensors stand in for device ones)
    import torch
    from adrt_pinv_gb300.device import Pipeline
    from adrt_pinv_gb300.plan import Plan

    plan = Plan("hybrid", 5, np.full(64, 2000.0), 0.2, 0.1, 1e-10, dense_cap=8)
    est = Pipeline.estimate_bytes(plan, 3, "fp32", captured=False)
    N, L, B = 32, 64, 3
    nd = 2 * len(plan.dense_freqs)
    assert nd > 0
    expect = B * 2 * L * N * 8 + 3 * B * N * N * 4 + 4 * B * N * N * 8 + 4 * B * N * N * 4
    expect += 2 * nd * N * N * 8 + nd * B * N * 8 + L * 8 + 3 * L * 4 + plan.coef.size * 4
    assert est == expect
    assert Pipeline.estimate_bytes(plan, 3, "fp32") - est == 2 * B * 4 * (2 * N - 1) * N * 8


def test_slot_level_admission_between_steps(pkg):
    """A request that arrives while a slot lane is busy starts at the next step in a free slot, without waiting for
    the requests ahead of it to finish."""
    S, serve = _server(pkg, budget=1e12, slots=lambda n: 2, lane=FakeSlotLane)
    a, b, c = (serve.Request(i, 5, None) for i in range(3))
    S.submit(a)
    S.step()  # a admitted and one step run
    lane = S.lanes[5]
    assert lane.req[0] is a and lane.k[0] == 1
    S.submit(b)
    S.submit(c)
    S.step()  # b takes the free slot while a is mid-way; c waits for a slot
    assert lane.req[1] is b and lane.k == [2, 1] and len(S.queues[5]) == 1
    S.step()  # a finishes (k = 3); its slot frees
    assert a.result == ("x", 0, 5) and lane.req[0] is None
    S.step()  # a collected, c admitted into slot 0 and stepped together with b's last step
    assert lane.req[0] is c and lane.k[0] == 1 and b.result == ("x", 1, 5)
    while S.step():
        pass
    assert {r.rid for r in S.finished} == {0, 1, 2}
    assert lane.steps == 6  # a: steps 1-3, b: 2-4, c: 4-6, overlapping


def test_admission_by_device_free_memory(pkg):
    """A lane that fits the budget but not the memory the device can still give waits (the queue keeps its
    requests) until memory frees up."""
    S, serve = _server(pkg, budget=1e12)
    free = {"bytes": 100}  # far less than one lane (4 slots x 64 x 64)
    S.device_free = lambda: free["bytes"]
    S.submit(serve.Request(0, 6, None))
    assert S.step() == 1 and not S.lanes
    free["bytes"] = 1e9
    while S.step():
        pass
    assert len(S.finished) == 1 and 6 in S.lanes
