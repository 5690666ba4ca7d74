"""CUDA-graph replay and the continuous-batching server on the GPU: every served result equals the same sinogram
inverted alone (same kernels, per-image arithmetic; tolerance 1e-6 relative), with sizes mixed, lanes running
concurrently and lanes evicted under a small memory budget."""

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _inverses(pkg, golden):
    return {
        4: pkg.FastHybridGpu(4, lam_max=golden["inv_lam_hyb_4"], outer=tuple(golden["inv_outer_hyb_4"])),
        5: pkg.FastLpGpu(5, dense_cap=8),
        6: pkg.FastHybridGpu(6, lam_max=golden["inv_lam_hybd8_6"], outer=tuple(golden["inv_outer_hybd8_6"]),
                             dense_cap=8),
    }


def _sinos(pkg, n, count, seed):
    from adrt_pinv_gb300 import adrtcore, phantoms

    return [adrtcore.adrt(n, phantoms.ellipse_phantom(1 << n, seed=seed + i)) for i in range(count)]


def test_graph_replay_matches_eager(pkg, golden):
    import torch

    inv = _inverses(pkg, golden)[6]
    bs = np.stack(_sinos(pkg, 6, 3, 10))
    eager = inv.apply(bs)
    pipe = inv.pipeline(3).capture()
    x = pipe.replay(torch.from_numpy(bs).cuda()).cpu().numpy()
    assert np.array_equal(x, eager)
    pipe.replay(torch.from_numpy(bs[::-1].copy()).cuda())
    assert np.array_equal(pipe.x_out.cpu().numpy(), eager[::-1])
    from adrt_pinv_gb300.device import Pipeline

    assert pipe.device_bytes() == Pipeline.estimate_bytes(inv.plan, 3, "fp32")


def _serve(pkg, golden, budget, seed, lane="slot"):
    from adrt_pinv_gb300 import serve

    invs = _inverses(pkg, golden)
    cls = serve.SlotLane if lane == "slot" else serve.Lane
    S = serve.InverseServer(lambda n: invs[n], slots=lambda n: 4, hbm_budget_bytes=budget, lane_cls=cls)
    rng = np.random.default_rng(seed)
    sizes = rng.choice([4, 5, 6], size=30)
    sinos = {n: _sinos(pkg, n, int((sizes == n).sum()), 100 * n) for n in (4, 5, 6)}
    reqs, k = [], {4: 0, 5: 0, 6: 0}
    for i, n in enumerate(sizes):
        reqs.append((0.002 * i, serve.Request(i, int(n), sinos[n][k[n]])))
        k[n] += 1
    done = S.run(reqs)
    assert len(done) == len(reqs)
    for r in done:
        alone = invs[r.n].apply(r.b)
        assert rel_err(r.result.numpy(), alone) < 1e-6
    st = serve.InverseServer.stats(done)
    assert st["p50_ms"] <= st["p99_ms"]
    return S, invs


@pytest.mark.parametrize("lane", ["slot", "batch"])
def test_served_mix_equals_alone(pkg, golden, lane):
    S, _ = _serve(pkg, golden, 120e9, 0, lane)
    assert S.max_busy >= 2  # lanes of different sizes were in flight together
    assert S.evictions == 0
    if lane == "slot":  # requests of one size overlapped on the device at different outer iterations
        assert any(l.steps_run < sum(1 for r in S.finished if r.n == n) * l.D for n, l in S.lanes.items())


@pytest.mark.parametrize("lane", ["slot", "batch"])
def test_served_mix_under_small_budget(pkg, golden, lane):
    from adrt_pinv_gb300 import serve

    invs = _inverses(pkg, golden)
    cls = serve.SlotLane if lane == "slot" else serve.Lane
    big = max(cls.estimate_bytes(invs[n], 4) for n in invs)
    S, _ = _serve(pkg, golden, big + 1, 1, lane)
    assert S.evictions >= 1 and S.memory_in_use() <= big + 1


def test_slot_lane_device_bytes_match_estimate(pkg, golden):
    from adrt_pinv_gb300 import serve

    inv = _inverses(pkg, golden)[6]
    lane = serve.SlotLane(inv, 4, "cuda")
    assert lane.device_bytes() <= serve.SlotLane.estimate_bytes(inv, 4)


def test_public_apply_graph_replay(pkg, golden):
    """apply() runs eagerly on the first call of a batch size and replays a CUDA graph from the second: the results
    and the level-row count per call stay the same."""
    inv = _inverses(pkg, golden)[6]
    bs = np.stack(_sinos(pkg, 6, 2, 40))
    outs, counts = [], []
    for _ in range(3):
        c0 = inv.eng.count[0]
        outs.append(inv.apply(bs))
        counts.append(inv.eng.count[0] - c0)
    assert inv.pipeline(2).graph is not None
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[1], outs[2])
    assert counts[0] == counts[1] == counts[2] > 0


def test_autotuned_pipeline_same_results(pkg, golden):
    """The autotuner times every candidate launch configuration on the GPU and keeps the fastest; the tuned pipeline
    gives the same inverse (within FP32 rounding of the dense kernels, 1e-6)."""
    import torch

    from adrt_pinv_gb300 import tune
    from adrt_pinv_gb300.device import Pipeline

    inv = _inverses(pkg, golden)[6]
    bs = torch.from_numpy(np.stack(_sinos(pkg, 6, 3, 70))).cuda()
    ref = inv.pipeline(3).apply(bs).clone()
    pipe = Pipeline(inv.plan, 3, "fp32", "cuda")
    res = tune.Tuner(reps=1).tune(pipe, bs)
    stage1 = tune.candidates(pipe)
    assert len(res["ms"]) >= len(stage1) >= 2
    assert {k: res["config"][k] for k in ("dense", "row_grid")} in stage1
    out = pipe.apply(bs)
    assert float((out - ref).norm() / ref.norm()) < 1e-6


def test_pipelined_host_calls_match_eager(pkg, golden):
    """apply(pinned host batch, out=pinned host buffer) alternates two captured graphs and input buffers so that a
    batch's copy overlaps the previous batch's graph; a run of such calls with different inputs gives, call by call,
    the eager results, and check() reports no dense-kernel failure."""
    import torch

    inv = _inverses(pkg, golden)[6]
    batches = [np.stack(_sinos(pkg, 6, 3, 200 + 10 * k)) for k in range(4)]
    eager = [inv.pipeline(3).apply(torch.from_numpy(bb).cuda()).cpu().numpy().copy() for bb in batches]
    inv.apply(batches[0])  # the second call of this batch size captures the graphs
    inv.apply(batches[0])
    outs = [torch.empty((3, 64, 64), dtype=torch.float64, pin_memory=True) for _ in batches]
    hosts = [torch.from_numpy(bb).pin_memory() for bb in batches]
    for _ in range(2):
        for hb, o in zip(hosts, outs):
            inv.apply(hb, out=o)
        inv.check()
        torch.cuda.synchronize()
        for o, e in zip(outs, eager):
            assert rel_err(o.numpy(), e) < 1e-12
