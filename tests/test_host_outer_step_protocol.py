"""The split cluster barrier of the register-resident outer step (csrc/outer_step.cu, outer_step_reg_kernel), modelled
on the CPU: the CTAs of one image's cluster publish their strip-boundary rows into one of two buffer copies, arrive,
compute the next step without the boundary terms, wait, and then read their neighbours' boundary rows. Under many
random interleavings every boundary read must see exactly the previous step's values (never a copy already
overwritten by a step ahead), every CTA must finish, and no CTA may leave while a neighbour can still read its
buffers."""

import random

import pytest


def run_cluster(CL, steps, seed, copies=2):
    rng = random.Random(seed)
    buf = [[None] * copies for _ in range(CL)]  # buf[cta][copy] = step whose boundary rows it holds
    arrived = [0] * CL  # arrivals per CTA (one per phase)
    exited = [False] * CL

    def completed(phase):  # the cluster barrier's phase is complete once every CTA arrived for it
        return all(a > phase for a in arrived)

    def cta(i):
        buf[i][0] = 0  # publish the first iterate (step 0), arrive for phase 0
        arrived[i] += 1
        yield
        for k in range(1, steps + 1):
            yield  # the step's interior work, no shared data
            while not completed(k - 1):
                yield
            for j in (i - 1, i + 1):  # the neighbours' boundary rows of step k - 1
                if 0 <= j < CL:
                    assert not exited[j], "read of an exited CTA's shared memory"
                    assert buf[j][(k - 1) % copies] == k - 1, f"step {k} read copy of step {buf[j][(k - 1) % copies]}"
            yield
            buf[i][k % copies] = k  # publish step k, arrive for phase k
            arrived[i] += 1
            yield
        while not completed(steps):  # the last arrival's wait before leaving
            yield
        exited[i] = True

    live = {i: cta(i) for i in range(CL)}
    n = 0
    while live:
        n += 1
        assert n < 200000, "deadlock"
        i = rng.choice(list(live))
        try:
            next(live[i])
        except StopIteration:
            del live[i]


@pytest.mark.parametrize("CL,steps", [(2, 12), (4, 12), (8, 12), (16, 12), (8, 1), (8, 2)])
def test_split_barrier_two_copies(CL, steps):
    """Clusters of 2..16 CTAs (N = 64..512 at 32-row bands, 16-row bands up to 16 CTAs), 12 stencil steps (degree 13),
    and the shortest degrees."""
    for seed in range(150):
        run_cluster(CL, steps, seed)


def test_one_copy_is_not_enough():
    """With a single buffer copy a fast CTA overwrites boundary rows a slow neighbour has not read yet: the model
    catches it, so the second copy is what makes one barrier per step sufficient."""
    caught = 0
    for seed in range(150):
        try:
            run_cluster(4, 12, seed, copies=1)
        except AssertionError:
            caught += 1
    assert caught > 0
