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


def _server(pkg, budget, slots=lambda n: 4):
    from adrt_pinv_gb300 import serve

    class S(serve.InverseServer):
        lane_cls = FakeLane

    FakeLane.created = []
    return S(FakeInverse, slots, hbm_budget_bytes=budget, device="cpu"), serve


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
    assert Pipeline.estimate_bytes(plan, 3, "fp32") - est == B * 4 * (2 * N - 1) * N * 8
