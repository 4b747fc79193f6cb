"""Host model of the producer/consumer protocol of the double 3-D pipeline
kernel (stencil3d_stream_kernel in csrc/kernel3d_tile.cuh): NS stages, each
with a "full" mbarrier (one arrival + the copy's bytes) and an "empty"
mbarrier (one arrival per consumer warp). The producer issues plane n into
stage n % NS after waiting for phase n/NS - 1 of empty[n % NS] (n >= NS);
consumer warps wait for phase n/NS of full[n % NS], read, then arrive on
empty[n % NS]; past the block's last plane they neither wait nor arrive.
Random interleavings (copies land late, warps run at different speeds)
check that every wait ends, that a consumer always reads the plane it asked
for, and that a parity wait is never satisfied by a later phase (the
producer is never two phases ahead of a stage's readers). CPU only."""
import numpy as np
import pytest


class Barrier:
    """mbarrier: `count` arrivals (and any pending copy) complete a phase;
    try_wait(parity) succeeds once the phase of that parity has completed,
    i.e. while the current phase's parity differs from it."""

    def __init__(self, count):
        self.count, self.arrived, self.pending_tx, self.completed = count, 0, 0, 0

    def arrive(self, tx=0):
        self.arrived += 1
        self.pending_tx += tx
        self._check()

    def land(self, tx):
        self.pending_tx -= tx
        self._check()

    def _check(self):
        if self.arrived == self.count and self.pending_tx == 0:
            self.arrived = 0
            self.completed += 1

    def try_wait(self, parity):
        return (self.completed & 1) != parity


def simulate(NS, NW, nplanes, extra_steps, seed):
    rng = np.random.default_rng(seed)
    full = [Barrier(1) for _ in range(NS)]
    empty = [Barrier(NW) for _ in range(NS)]
    stage = [None] * NS       # plane held by each stage
    in_flight = []            # (stage, plane) copies issued and not landed
    prod_n = 0
    cons = [0] * NW           # next step of each consumer warp
    last_step = nplanes + extra_steps
    for _ in range(200000):
        if prod_n >= nplanes and all(c >= last_step for c in cons) and not in_flight:
            return True
        actor = int(rng.integers(NW + 2))
        if actor == NW:       # producer
            if prod_n < nplanes:
                st = prod_n % NS
                if prod_n < NS or empty[st].try_wait(((prod_n // NS) - 1) & 1):
                    # the stage's previous plane has been released by every warp
                    assert prod_n < NS or empty[st].completed == prod_n // NS
                    full[st].arrive(tx=1)
                    in_flight.append((st, prod_n))
                    prod_n += 1
        elif actor == NW + 1:  # a copy lands
            if in_flight:
                st, pl = in_flight.pop(int(rng.integers(len(in_flight))))
                stage[st] = pl
                full[st].land(1)
        else:                 # consumer warp
            n = cons[actor]
            if n >= last_step:
                continue
            st = n % NS
            if n < nplanes:
                if not full[st].try_wait((n // NS) & 1):
                    continue
                # the wait ends in the phase that delivered plane n, not a later one
                assert full[st].completed == n // NS + 1
                assert stage[st] == n
                empty[st].arrive()
            cons[actor] = n + 1
    return False


@pytest.mark.parametrize("NS", [2, 3, 4])
@pytest.mark.parametrize("NW", [1, 4, 8])
@pytest.mark.parametrize("nplanes", [1, 3, 7, 20])
def test_pipeline_protocol(NS, NW, nplanes):
    for seed in range(8):
        assert simulate(NS, NW, nplanes, extra_steps=2, seed=seed), "a wait never ended"
