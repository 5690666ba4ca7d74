"""Autotuner for the launch configuration and tile shapes of a device pipeline.

Per (plan, batch, precision) the tuner times the candidate configurations of the choices that depend on the
workload's shape, on the GPU and with the pipeline's own data, and keeps the fastest:
  * the dense-row kernel: tensor cores (3xTF32 tcgen05), the streaming CUDA-core kernel (batches of at most 16; the
    operators stored transposed) or the tiled CUDA-core kernel, crossed with the grid of the row programs (one or
    two persistent CTAs per SM);
  * then, one dimension at a time with the others held at the best so far, the tile shapes: images per CTA of the
    tensor-core dense kernel (16, 32, 64), rows per CTA of the fused outer step's bands (16 or 32, which also
    sets the cluster size, N/16 or N/32 CTAs per image) and strip columns per CTA of the offset FFTs (the default
    or a quarter of it).
Each candidate is timed with CUDA events over `reps` applies after one warm-up apply. Results are cached per
(N, method, degree cap, dense cap, batch, precision, GPU name) in memory and, when a path is given, in a JSON file.
"""

import itertools
import json
import os

import torch


def device_info(device):
    """(name, SM count) of the GPU."""
    return torch.cuda.get_device_name(device), torch.cuda.get_device_properties(device).multi_processor_count


def candidates(pipe):
    """The configurations worth timing for this pipeline: [{"dense": mode, "row_grid": g}]."""
    sms = device_info(pipe.device)[1]
    dense = ["none"]
    if len(pipe.plan.dense_freqs):
        if pipe.real == torch.float32:
            dense = ["tc", "simt"] + (["stream"] if pipe.B <= 16 else [])
        else:
            dense = ["simt"]
    return [{"dense": d, "row_grid": g} for d, g in itertools.product(dense, (sms, 2 * sms))]


def tile_dimensions(pipe, cfg):
    """The tile-shape choices worth timing for this pipeline once the kernels are chosen: {name: [values]}."""
    dims = {}
    if cfg.get("dense") == "tc":
        dims["dense_tile"] = [16, 32, 64]
    N = pipe.plan.N
    if pipe.fused_outer_ok() and N >= 32 and N // 16 <= 16:
        dims["band"] = [16, 32]
    wide = fft_cols_default(N, pipe.real)
    if wide >= 4:
        dims["fft_cols"] = [wide, wide // 4]
    return dims


def fft_cols_default(N, real):
    """The offset FFTs' default strip columns per CTA (csrc/fft.cu fft_cols): up to 16 (FP32) / 8 (FP64), at most
    1024 threads (8 points each along the 2N-long axis), at most N/2, and within 227 KB of shared memory."""
    L = 2 * N
    elem = 8 if real == torch.float32 else 16
    tpc = L // 8 if L >= 8 else 1  # threads per column: 8 points each
    c = max(1, min(16 if real == torch.float32 else 8, 1024 // tpc, N))
    pad = lambda c: c + 1 if c > 1 else 1
    while c > 1 and (L + (L + L // 2) * pad(c)) * elem > 227 * 1024:
        c >>= 1
    return c


def apply_config(pipe, cfg):
    t = pipe.tables
    t.stream_dense = cfg["dense"] == "stream"
    t.use_tc = cfg["dense"] == "tc"
    t.row_grid = int(cfg["row_grid"])
    t.dense_tile = int(cfg.get("dense_tile", 0))
    pipe.band = int(cfg.get("band", 0))
    pipe.fft_cols = int(cfg.get("fft_cols", 0))


def key_of(pipe):
    p = pipe.plan
    name = device_info(pipe.device)[0]
    return f"{name}|N={p.N}|{p.method}|cap={p.deg_cap}|dense={p.dense_cap}|B={pipe.B}|{pipe.precision}"


class Tuner:
    def __init__(self, path=None, reps=3, timer=None):
        self.path, self.reps = path, int(reps)
        self.cache = {}
        if path and os.path.exists(path):
            with open(path) as f:
                self.cache = json.load(f)
        self.timer = timer or self._time

    def _time(self, pipe, b):
        pipe.apply(b)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(self.reps):
            pipe.apply(b)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / self.reps

    def tune(self, pipe, b):
        """Pick and apply the fastest configuration for pipe on sinograms b (on the device); returns
        {"config": ..., "ms": {...}}. Must run before the pipeline is captured in a graph."""
        k = key_of(pipe)
        if k not in self.cache:
            times = {}

            def run(cfg):
                key = json.dumps(cfg, sort_keys=True)
                if key not in times:
                    apply_config(pipe, cfg)
                    times[key] = self.timer(pipe, b)
                return times[key]

            for cfg in candidates(pipe):
                run(cfg)
            best = json.loads(min(times, key=times.get))
            for name, values in tile_dimensions(pipe, best).items():
                for v in values:
                    cfg = dict(best, **{name: v})
                    if run(cfg) < run(best):
                        best = cfg
            self.cache[k] = {"config": best, "ms": times}
            if self.path:
                with open(self.path, "w") as f:
                    json.dump(self.cache, f, indent=1)
        apply_config(pipe, self.cache[k]["config"])
        t = pipe.tables  # keep only the dense tables of the chosen layout
        t._dense_dev = {kk: v for kk, v in t._dense_dev.items() if kk[4] == t.stream_dense}
        return self.cache[k]
