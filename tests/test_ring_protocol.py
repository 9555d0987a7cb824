"""The hand-off protocol of the tcgen05 operator kernel's stage ring
(``pyfr_gb300/csrc/mul_umma.cu``), modelled on the host with mbarrier
parity semantics and random completion orders (no GPU).

A producer loads chunk j into stage j mod NS once the stage's previous
chunk has been consumed (FREE), a converter group waits for the stage's
LOADED phase of parity (j / NS) & 1 and converts it, and the MMA thread
waits, in order, for CONVERTED and releases the stage.  An mbarrier wait on
parity P returns as soon as the barrier's current phase has the other
parity -- so a waiter that comes two phases early is let through, and
every waiter must be at most one phase ahead of the stage.  With the
converter groups owning the even and the odd stages (the kernel's scheme)
that holds for a ring of any length; with the groups taking alternate
chunks it fails for an odd ring, where a stage's consecutive chunks belong
to different groups.
"""
import random

import pytest


class Barrier:
    """An mbarrier: phases complete after ``count`` arrivals (and, for a
    loaded stage, the data's arrival); try_wait(P) is true when the
    current phase's parity differs from P."""

    def __init__(self, count=1):
        self.count, self.pending, self.phase = count, 0, 0

    def arrive(self):
        self.pending += 1
        if self.pending == self.count:
            self.pending = 0
            self.phase += 1

    def try_wait(self, parity):
        return (self.phase & 1) != parity


def simulate(ns, nchunks, owner, seed):
    """Run the protocol to completion with random interleavings; returns
    the chunks each consumer saw (which must be the ones it asked for)."""
    rng = random.Random(seed)
    loaded = [Barrier() for _ in range(ns)]
    converted = [Barrier() for _ in range(ns)]
    free = [Barrier() for _ in range(ns)]
    content = [None]*ns             # the chunk whose data is in the stage
    inflight = []                   # (stage, chunk) loads not yet landed

    prod = 0
    conv = {0: 0, 1: 0}             # next chunk index each group looks at
    mma = 0
    seen = []

    def next_for(g):
        j = conv[g]
        while j < nchunks and owner(j, j % ns) != g:
            j += 1
        conv[g] = j
        return j

    busy_conv = {0: None, 1: None}
    busy_mma = None
    for _ in range(100*nchunks):
        acts = []
        if prod < nchunks:
            s = prod % ns
            if prod < ns or free[s].try_wait(((prod // ns) & 1) ^ 1):
                acts.append('prod')
        if inflight:
            acts.append('land')
        for g in (0, 1):
            if busy_conv[g] is not None:
                acts.append(('convdone', g))
                continue
            j = next_for(g)
            if j < nchunks and loaded[j % ns].try_wait((j // ns) & 1):
                acts.append(('conv', g))
        if busy_mma is not None:
            acts.append('mmadone')
        elif mma < nchunks and converted[mma % ns].try_wait((mma // ns) & 1):
            acts.append('mma')
        if not acts:
            break
        a = rng.choice(acts)
        if a == 'prod':
            inflight.append((prod % ns, prod))
            prod += 1
        elif a == 'land':
            s, j = inflight.pop(rng.randrange(len(inflight)))
            content[s] = j
            loaded[s].arrive()
        elif a[0] == 'conv':
            g = a[1]
            j = conv[g]
            seen.append(('conv', j, content[j % ns]))
            busy_conv[g] = j
            conv[g] += 1
        elif a[0] == 'convdone':
            g = a[1]
            converted[busy_conv[g] % ns].arrive()
            busy_conv[g] = None
        elif a == 'mma':
            seen.append(('mma', mma, content[mma % ns]))
            busy_mma = mma
            mma += 1
        else:
            free[busy_mma % ns].arrive()
            busy_mma = None
    return seen, mma


def stage_owner(j, s):
    return s & 1


def chunk_owner(j, s):
    return j & 1


@pytest.mark.parametrize('ns', range(4, 11))
def test_stage_owned_groups_any_ring(ns):
    for seed in range(60):
        seen, done = simulate(ns, 12*ns, stage_owner, seed)
        assert done == 12*ns
        bad = [x for x in seen if x[1] != x[2]]
        assert not bad, (ns, seed, bad[:3])


def test_chunk_alternating_groups_fail_on_odd_rings():
    """The scheme the kernel replaced: alternate chunks per group is safe
    on even rings only."""
    for ns in (4, 6, 8):
        for seed in range(40):
            seen, _ = simulate(ns, 12*ns, chunk_owner, seed)
            assert all(x[1] == x[2] for x in seen)
    failures = 0
    for seed in range(200):
        seen, _ = simulate(5, 60, chunk_owner, seed)
        failures += any(x[1] != x[2] for x in seen)
    assert failures > 0
