"""Autotuner logic (candidate set, selection, cache) with a fake timer and a stand-in pipeline on the CPU."""
import json
import types

import numpy as np


def _pipe(torch, B, dense, real):
    plan = types.SimpleNamespace(N=256, method="hybrid", deg_cap=32, dense_cap=16,
                                 dense_freqs=np.arange(3) if dense else np.zeros(0))
    tables = types.SimpleNamespace(stream_dense=False, use_tc=False, row_grid=0, dense_tile=0, _dense_dev={})
    return types.SimpleNamespace(plan=plan, B=B, precision="fp32", real=real, device="cpu", tables=tables, band=0,
                                 fused_outer_ok=lambda: True)


def test_candidates_and_choice(pkg, monkeypatch, tmp_path):
    import torch

    from adrt_pinv_gb300 import tune

    monkeypatch.setattr(tune, "device_info", lambda d: ("FakeGPU", 152))
    p = _pipe(torch, 8, True, torch.float32)
    cands = tune.candidates(p)
    assert {c["dense"] for c in cands} == {"tc", "simt", "stream"} and {c["row_grid"] for c in cands} == {152, 304}
    assert {c["dense"] for c in tune.candidates(_pipe(torch, 64, True, torch.float32))} == {"tc", "simt"}
    assert {c["dense"] for c in tune.candidates(_pipe(torch, 4, False, torch.float32))} == {"none"}
    assert {c["dense"] for c in tune.candidates(_pipe(torch, 4, True, torch.float64))} == {"simt"}

    cost = {"tc": 3.0, "simt": 5.0, "stream": 2.0}
    calls = []

    def timer(pipe, b):
        calls.append(1)
        t = pipe.tables
        mode = "stream" if t.stream_dense else ("tc" if t.use_tc else "simt")
        return cost[mode] + (0.5 if t.row_grid == 304 else 0.0) - (0.1 if pipe.band == 16 else 0.0) - \
            (0.2 if t.dense_tile == 32 else 0.0)

    path = tmp_path / "tune.json"
    T = tune.Tuner(path=str(path), timer=timer)
    p.tables._dense_dev = {(0, 1, 1, 1, True): "t", (0, 1, 1, 1, False): "f"}
    res = T.tune(p, None)
    assert res["config"] == {"dense": "stream", "row_grid": 152, "band": 16}  # tile shapes tuned after the kernels
    assert p.tables.stream_dense and not p.tables.use_tc and p.tables.row_grid == 152 and p.band == 16
    assert list(p.tables._dense_dev) == [(0, 1, 1, 1, True)]  # the other layout's tables are dropped
    n = len(calls)
    T2 = tune.Tuner(path=str(path), timer=timer)  # cached on disk: no timing
    q = _pipe(torch, 8, True, torch.float32)
    assert T2.tune(q, None)["config"] == res["config"] and len(calls) == n
    assert json.load(open(path))


def test_tile_shapes_of_the_tensor_core_kernel(pkg, monkeypatch):
    import torch

    from adrt_pinv_gb300 import tune

    monkeypatch.setattr(tune, "device_info", lambda d: ("FakeGPU", 152))
    p = _pipe(torch, 64, True, torch.float32)

    def timer(pipe, b):
        t = pipe.tables
        base = 1.0 if t.use_tc else 4.0
        return base - {0: 0.0, 16: 0.05, 32: 0.3, 64: 0.1}[t.dense_tile] + (0.2 if pipe.band == 16 else 0.0)

    res = tune.Tuner(timer=timer).tune(p, None)
    assert res["config"] == {"dense": "tc", "row_grid": 152, "dense_tile": 32}  # band: no gain over the default
    assert p.tables.dense_tile == 32 and p.band == 0
    assert tune.tile_dimensions(p, {"dense": "tc"}) == {"dense_tile": [16, 32, 64], "band": [16, 32],
                                                        "fft_cols": [16, 4]}
    assert [tune.fft_cols_default(1 << n, torch.float32) for n in (2, 5, 8, 9, 10, 11)] == [4, 16, 16, 8, 4, 2]
