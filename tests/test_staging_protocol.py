"""Model check, on the CPU, of the barrier-free staging protocol of the deposit
(owned-cell launches), histogram and one-pass placement kernels: 32 (or 16)
warps stream batches through two shared-memory buffers, each filled by one bulk
copy that completes one phase of
the buffer's mbarrier.  Batch q (counted over all passes of a CTA) sits in
buffer q % 2 and completes phase q // 2 there.  A warp waits for it with a
parity wait (true once the barrier's current phase has the other parity), reads
its records, and adds one to the buffer's release counter; the warp that brings
the counter to a multiple of the warp count issues the copy of batch q + 2 of the same pass
into that buffer.  Passes (bins, grids, float32 redos) follow one another after
a block barrier; each starts with thread 0 issuing its first two copies.

Random interleavings, with copies landing at random later times, check that no
parity wait succeeds on any phase but its own, that no warp reads a buffer
that is being refilled, that each copy is issued once and only after every
warp has left the buffer, and that every run ends."""
import numpy as np
import pytest

WARPS = 32


def run(passes, seed, last=None, warps=WARPS):
    """warps: warps of the CTA (32, or 16 for the 512-thread placement kernels);
    last: the release count, modulo warps, whose warp issues the refill."""
    rng = np.random.default_rng(seed)
    last = warps - 1 if last is None else last
    phases = [0, 0]                 # completed phases per buffer
    content = [None, None]          # batch held by each buffer (None: copy in flight)
    in_flight = []                  # (buffer, batch) copies not yet landed
    rel = [0, 0]                    # release counters, never reset
    issued = {}                     # batch -> times its copy was issued
    q0 = 0
    steps = 0

    def issue(q):
        b = q & 1
        issued[q] = issued.get(q, 0) + 1
        content[b] = None
        in_flight.append((b, q))

    def land():
        b, q = in_flight.pop(int(rng.integers(len(in_flight))))
        content[b] = q
        phases[b] += 1
        assert phases[b] == q // 2 + 1

    for nb in passes:
        for j in range(min(2, nb)):             # thread 0, then the pass-start barrier
            issue(q0 + j)
        left = [set() for _ in range(nb)]
        pos = [0] * warps
        waiting = [True] * warps
        while any(p < nb for p in pos):
            steps += 1
            assert steps < 400 * (sum(passes) + 1) * warps, 'no progress: deadlock'
            if in_flight and rng.random() < 0.3:
                land()
            w = int(rng.integers(warps))
            j = pos[w]
            if j >= nb:
                continue
            q = q0 + j
            b, phase = q & 1, q // 2
            if waiting[w]:
                if (phases[b] & 1) != (phase & 1):     # mbarrier.try_wait.parity
                    assert phases[b] == phase + 1, 'parity wait passed on another phase'
                    assert content[b] == q, 'read a buffer that is being refilled'
                    waiting[w] = False
            else:
                left[j].add(w)
                done = rel[b]
                rel[b] += 1
                if (done & (warps - 1)) == last and j + 2 < nb:
                    assert len(left[j]) == warps, 'refilled before every warp left'
                    issue(q + 2)
                waiting[w] = True
                pos[w] += 1
        assert not in_flight                    # every copy of the pass was waited for
        assert rel[0] % warps == 0 and rel[1] % warps == 0
        q0 += nb
    assert sorted(issued) == list(range(q0)) and set(issued.values()) <= {1}
    return steps


@pytest.mark.parametrize('warps', [32, 16])
@pytest.mark.parametrize('nb', [0, 1, 2, 3, 7, 16])
def test_one_pass(nb, warps):
    for seed in range(30):
        run([nb], seed, warps=warps)


@pytest.mark.parametrize('passes', [[5, 2, 9], [1, 1, 1, 1], [3, 0, 4, 4], [16, 16]])
def test_passes_share_counters_and_barriers(passes):
    for seed in range(20):
        run(passes, seed)


def test_model_catches_an_early_refill():
    """The same model with the refill issued by the 31st warp out instead of the
    32nd: some interleaving must trip an assertion."""
    caught = 0
    for seed in range(20):
        try:
            run([8], seed, last=30)
        except AssertionError:
            caught += 1
    assert caught > 0
