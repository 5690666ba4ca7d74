"""Uneven batches in one CUDA graph.

A batch of sinograms of different sizes N, inner degree caps p and methods (L_p / hybrid) is split into classes,
one inverse (plan) per class. Each class gets a device pipeline sized to its share of the batch, and the applies of
all classes are recorded into ONE CUDA graph, each class on its own stream forked from the capture stream and joined
back into it, so that the whole uneven batch is one graph launch whose classes run concurrently on the GPU (the
kernels of a small class fill the SMs a large class leaves idle). Every class keeps its own buffers, tables and work
counter, so the classes share nothing but the GPU.
"""

import torch


class UnevenBatch:
    def __init__(self, groups, device="cuda", tuner=None, sinos=None):
        """groups: [(inverse, count)], one entry per class; an inverse may appear more than once (a large class split
        into several concurrent parts), each entry getting its own pipeline. With a tuner (tune.Tuner) and the
        classes' sinograms, every class's launch configuration is autotuned on its own data before the capture."""
        from .device import Pipeline

        self.groups = [(inv, int(c)) for inv, c in groups if int(c) > 0]
        self.device = torch.device(device)
        self.pipes = [Pipeline(inv.plan, c, inv.precision, self.device, inv.stencil_precision) for inv, c in self.groups]
        self.inputs = [torch.zeros((c, 4, 2 * inv.N - 1, inv.N), dtype=torch.float64, device=self.device)
                       for inv, c in self.groups]
        self.tuning = []
        if tuner is not None and sinos is not None:
            for pipe, x in zip(self.pipes, sinos):
                self.tuning.append(tuner.tune(pipe, x.to(self.device)))
        self.streams = [torch.cuda.Stream(device=self.device) for _ in self.groups]
        cap = torch.cuda.Stream(device=self.device)
        cap.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(cap):
            for pipe, x in zip(self.pipes, self.inputs):  # eager run: builds tables, sets kernel attributes
                pipe.apply(x)
            cap.synchronize()
            self.graph = torch.cuda.CUDAGraph()
            self.outputs = []
            with torch.cuda.graph(self.graph, stream=cap):
                for st, pipe, x in zip(self.streams, self.pipes, self.inputs):
                    st.wait_stream(cap)
                    with torch.cuda.stream(st):
                        self.outputs.append(pipe.apply(x))
                for st in self.streams:
                    cap.wait_stream(st)
        torch.cuda.current_stream(self.device).wait_stream(cap)

    def set_inputs(self, sinos):
        """sinos: one (count, 4, 2N-1, N) tensor per class (device or pinned host), copied into the graph inputs."""
        for dst, src in zip(self.inputs, sinos):
            dst.copy_(src, non_blocking=True)

    def replay(self):
        """One launch of the whole uneven batch on the current stream; returns the per-class result buffers. The
        results are valid once the stream has reached this point and check() has passed."""
        self.graph.replay()
        return self.outputs

    def check(self):
        """Raise if a tensor-core dense-row launch of any class gave up on a bounded wait since the last check (its
        dense rows were not written). Reads each class's error flag, a device synchronisation: call it after
        synchronising on the replay, before the results are used."""
        for pipe in self.pipes:
            pipe.tables.raise_if_error()

    def device_bytes(self):
        return sum(p.device_bytes() for p in self.pipes)
