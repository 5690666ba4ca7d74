"""The synchronisation protocol of the warp-specialised dense-row kernel (csrc/dense.cu, dense_cx_kernel), modelled on
the CPU: four roles (operator copies, image tiles, MMA issue, fold) over a ring of S stages and two accumulator sets,
connected by mbarriers whose waits use a phase parity, run under many random interleavings with asynchronous copy
and MMA completion.

Checked: every role finishes (no deadlock); no parity wait targets a phase two or more behind the barrier (on the
hardware such a wait would see the parity of a later phase and block); the MMAs of a chunk read a stage holding
that chunk's operator and image tiles; a stage is refilled only after the MMAs that read it completed; an
accumulator set is rewritten only after its previous chunk was folded, and every fold reads the chunk it expects."""

import random

import pytest


class Barrier:
    def __init__(self, count):
        self.count, self.pending, self.tx, self.completed = count, count, 0, 0

    def _maybe_complete(self):
        if self.pending == 0 and self.tx == 0:
            self.completed += 1
            self.pending = self.count

    def arrive(self, expect_tx=0):
        self.tx += expect_tx
        self.pending -= 1
        self._maybe_complete()

    def complete_tx(self, nbytes):
        self.tx -= nbytes
        self._maybe_complete()

    def ready(self, phase):
        """A wait for (0-based) phase `phase`: true once it completed; aliasing if the barrier is already two ahead."""
        assert self.completed <= phase + 1, f"parity alias: waiting for phase {phase}, {self.completed} completed"
        return self.completed == phase + 1


def run_protocol(NC, S, seed, faults=()):
    """faults: waits to leave out ("stage_free" in the operator-copy role, "acc_free" in the MMA role), to show that
    the model catches them."""
    rng = random.Random(seed)
    a_full = [Barrier(1) for _ in range(S)]
    x_full = [Barrier(1) for _ in range(S)]  # the image-tile warps' arrivals, modelled as one
    stage_free = [Barrier(1) for _ in range(S)]
    acc_full = [Barrier(1) for _ in range(2)]
    acc_free = [Barrier(1) for _ in range(2)]
    stage_a = [None] * S  # chunk whose operator tiles the stage holds
    stage_x = [None] * S
    stage_reader_done = [True] * S  # the MMAs that read the stage's current content completed
    acc = [None, None]  # chunk whose partial sums the accumulator set holds
    acc_folded = [True, True]
    folded = []
    async_events = []  # (kind, arguments): copies landing, MMA groups completing (in issue order)

    def producer():
        for kc in range(NC):
            s, u = kc % S, kc // S
            if u > 0 and "stage_free" not in faults:
                while not stage_free[s].ready(u - 1):
                    yield
            assert stage_reader_done[s], "operator tiles overwrite a stage still being read"
            a_full[s].arrive(expect_tx=1)
            async_events.append(("copy", s, kc))
            yield

    def image_tiles():
        for kc in range(NC):
            s, u = kc % S, kc // S
            if u > 0:
                while not stage_free[s].ready(u - 1):
                    yield
            assert stage_reader_done[s], "image tiles overwrite a stage still being read"
            stage_x[s] = kc
            x_full[s].arrive()
            yield

    def mma():
        for kc in range(NC):
            s, u, be, v = kc % S, kc // S, kc & 1, kc >> 1
            while not (a_full[s].ready(u) and x_full[s].ready(u)):
                yield
            if v > 0 and "acc_free" not in faults:
                while not acc_free[be].ready(v - 1):
                    yield
            assert stage_a[s] == kc and stage_x[s] == kc, "MMAs read a stage holding another chunk"
            assert acc_folded[be], "accumulator set rewritten before its chunk was folded"
            stage_reader_done[s] = False
            acc_folded[be] = False
            async_events.append(("mma", s, be, kc))  # completes later, after the MMAs issued before it
            yield

    def fold():
        for kc in range(NC):
            be, v = kc & 1, kc >> 1
            while not acc_full[be].ready(v):
                yield
            assert acc[be] == kc, "fold reads an accumulator set of another chunk"
            folded.append(kc)
            acc_folded[be] = True
            acc_free[be].arrive()
            yield

    roles = [producer(), image_tiles(), mma(), fold()]
    live = list(range(len(roles)))
    steps = 0
    while live or async_events:
        steps += 1
        assert steps < 100000, "deadlock"
        mma_events = [e for e in async_events if e[0] == "mma"]
        if async_events and (not live or rng.random() < 0.3):
            # an asynchronous completion: any copy, or the oldest MMA group (tcgen05 completes in issue order)
            cands = [e for e in async_events if e[0] == "copy"] + mma_events[:1]
            ev = rng.choice(cands)
            async_events.remove(ev)
            if ev[0] == "copy":
                _, s, kc = ev
                stage_a[s] = kc
                a_full[s].complete_tx(1)
            else:
                _, s, be, kc = ev
                acc[be] = kc
                stage_reader_done[s] = True
                stage_free[s].arrive()  # the commit to the stage's barrier
                acc_full[be].arrive()   # the commit to the accumulator set's barrier
            continue
        if not live:
            continue
        i = rng.choice(live)
        try:
            next(roles[i])
        except StopIteration:
            live.remove(i)
    assert folded == list(range(NC))


@pytest.mark.parametrize("NC", [8, 16, 32, 64])
def test_dense_pipeline_protocol(NC):
    """The kernel's ring of 4 stages at the chunk counts of N = 128..1024 (16 input columns per chunk)."""
    for seed in range(200):
        run_protocol(NC, 4, seed)


@pytest.mark.parametrize("fault", ["stage_free", "acc_free"])
def test_protocol_model_detects_a_missing_wait(fault):
    """The model can fail: with either wait left out, some interleaving overwrites data still in use."""
    caught = 0
    for seed in range(200):
        try:
            run_protocol(16, 4, seed, faults=(fault,))
        except AssertionError:
            caught += 1
    assert caught > 0
