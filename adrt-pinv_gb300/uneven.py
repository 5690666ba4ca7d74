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
        from .device import Pipeline, graph_capture

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
            with graph_capture(self.graph, cap):
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


class PersistentUnevenBatch:
    """Uneven batch whose polynomial rows run in ONE persistent launch per outer step.

    All classes step through the outer iteration together (class c takes D_c steps; it drops out once they are
    done): at every step each class packs its images (or, at step 0, its sinograms) on its own stream, then one
    persistent row-engine launch (adrt_rows_run_multi) processes the polynomial rows of every active class from a
    single work queue (classes ordered by the cost of their rows, rows within a class by degree), then each class
    finishes its pass (dense or compensated rows, inverse FFT, unpack) and its outer step on its own stream. The
    whole batch is recorded once as a CUDA graph; replay() is one launch. Classes must be FP32 with N = 64..512
    (the sizes whose rows fit one warp); results are per class as in UnevenBatch."""

    def __init__(self, groups, device="cuda", tuner=None, sinos=None):
        import ctypes

        import numpy as np

        from . import _lib as C
        from .device import Pipeline, graph_capture
        from .plan import outer_coeffs

        self.groups = [(inv, int(c)) for inv, c in groups if int(c) > 0]
        self.device = torch.device(device)
        for inv, _ in self.groups:
            if inv.precision != "fp32" or not 6 <= inv.n <= 9:
                raise ValueError("the persistent uneven batch takes FP32 classes with N = 64..512")
        self.pipes = [Pipeline(inv.plan, c, inv.precision, self.device, inv.stencil_precision) for inv, c in self.groups]
        self.inputs = [torch.zeros((c, 4, 2 * inv.N - 1, inv.N), dtype=torch.float64, device=self.device)
                       for inv, c in self.groups]
        self.tuning = []
        if tuner is not None and sinos is not None:
            for pipe, x in zip(self.pipes, sinos):
                self.tuning.append(tuner.tune(pipe, x.to(self.device)))
        self.coeffs = [outer_coeffs(p.plan.lo, p.plan.hi, p.plan.outer_deg) for p in self.pipes]
        self.D = [p.plan.outer_deg for p in self.pipes]
        lib = C.load()
        # cost order: level-rows of one G pass per class, costliest first
        cost = [p.tables.main_level_rows(p.ops["G"]) * p.B for p in self.pipes]
        self.order = sorted(range(len(self.pipes)), key=lambda i: -cost[i])

        def job_set(kind, classes):
            jobs, codes, starts = [], [], [0]
            for i in classes:
                p = self.pipes[i]
                j = p.tables.main_job(p.Y, p.ops[kind])
                code = lib.adrt_rows_multi_code(ctypes.byref(j))
                if code < 0:
                    raise ValueError(f"class {i}: its row program cannot join the persistent launch")
                gpw = 32 // lib.adrt_rows_lanes_per_row(p.plan.n)
                jobs.append(j)
                codes.append(code)
                starts.append(starts[-1] + -(-(j.nimg * j.nsel) // gpw))
            arr = (C.RowJob * len(jobs))(*jobs)
            raw = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).to(self.device)
            return (raw, torch.tensor(codes, dtype=torch.int32, device=self.device),
                    torch.tensor(starts, dtype=torch.int32, device=self.device), len(jobs))

        self.counter = torch.zeros(4, dtype=torch.int32, device=self.device)
        self.job_sets = {("BP", None): job_set("BP", self.order)}
        for s in range(1, max(self.D)):
            act = tuple(i for i in self.order if self.D[i] > s)
            if ("G", act) not in self.job_sets:
                self.job_sets[("G", act)] = job_set("G", act)
        self.streams = [torch.cuda.Stream(device=self.device) for _ in self.pipes]
        cap = torch.cuda.Stream(device=self.device)
        cap.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(cap):
            for pipe, x in zip(self.pipes, self.inputs):  # eager run: builds tables, sets kernel attributes
                pipe.apply(x)
            self._run(cap)  # and one eager run of the lock-step schedule
            cap.synchronize()
            self.graph = torch.cuda.CUDAGraph()
            with graph_capture(self.graph, cap):
                self.outputs = self._run(cap)
        torch.cuda.current_stream(self.device).wait_stream(cap)
        self.launches_per_step = None

    def _rows(self, key, cap):
        from . import _lib as C

        raw, codes, starts, nj = self.job_sets[key]
        C.call("adrt_rows_run_multi", C.ptr(raw), C.ptr(codes), C.ptr(starts), nj, C.ptr(self.counter), 0,
               C.stream_handle())

    def _fork(self, cap, classes, fn):
        for i in classes:
            st = self.streams[i]
            st.wait_stream(cap)
            with torch.cuda.stream(st):
                fn(i)
        for i in classes:
            cap.wait_stream(self.streams[i])

    def _run(self, cap):
        """The lock-step schedule on the current (capture) stream; returns the per-class result buffers."""
        allc = list(self.order)
        state = {}  # class -> (x, x_prev, free buffers)

        def pack_bp(i):
            self.pipes[i].pack(self.inputs[i], sino=True)

        def finish_bp(i):
            p = self.pipes[i]
            p.finish_pass(p.ops["BP"])
            p.sum_parts(p.y)
            a = self.coeffs[i][0]
            p.first_step(p.y, p.xs[0], a)
            state[i] = [p.xs[0], None, [p.xs[1], p.xs[2]]]

        self._fork(cap, allc, pack_bp)
        self._rows(("BP", None), cap)
        self._fork(cap, allc, finish_bp)
        for s in range(1, max(self.D)):
            act = tuple(i for i in self.order if self.D[i] > s)

            def pack_g(i):
                self.pipes[i].pack(state[i][0], sino=False)

            def finish_g(i, s=s):
                p = self.pipes[i]
                x, xp, free = state[i]
                p.finish_pass(p.ops["G"])
                om_a, om_1 = self.coeffs[i][2][s - 1]
                xn = free.pop(0)
                p.next_step(p.y, x, xp, xn, om_a, om_1)
                if xp is not None:
                    free.append(xp)
                state[i] = [xn, x, free]

            self._fork(cap, act, pack_g)
            self._rows(("G", act), cap)
            self._fork(cap, act, finish_g)
        return [self.pipes[i].result(state[i][0]) for i in range(len(self.pipes))]

    def set_inputs(self, sinos):
        for dst, src in zip(self.inputs, sinos):
            dst.copy_(src, non_blocking=True)

    def replay(self):
        """One launch of the whole uneven batch on the current stream; returns the per-class result buffers (valid
        once the stream has reached this point and check() has passed)."""
        self.graph.replay()
        return self.outputs

    def check(self):
        for pipe in self.pipes:
            pipe.tables.raise_if_error()

    def device_bytes(self):
        return sum(p.device_bytes() for p in self.pipes)
