"""The claim protocol of the batched integrators' work queue
(gala_gb300/csrc/gx_queue.cuh, queue_next), restated step for step in Python
and run with warps interleaved at random: every 32-orbit block of the order is
integrated exactly once, at most one lead block goes to each SM sub-partition
while lead warps exist, and after a cancellation at any point the blocks taken
are the ones BatchIntegrator._taken_slots reports from the two counters."""
import numpy as np
import pytest


class Queue:
    """queue[0] main claims, queue[1] lead claims, one flag per sub-partition."""

    def __init__(self, n_chunks, subs, n_slots):
        self.main = 0
        self.lead = 0
        self.flags = [0] * n_slots
        self.n_chunks = n_chunks
        self.subs = subs
        self.n_lead = min(n_chunks, n_slots // subs)   # queue_lead_chunks

    def next(self, warp):
        """queue_next for one warp: (chunk, sub) or None; warp['phase'] persists."""
        n_lead_blocks = self.n_lead * self.subs
        if warp["phase"] == 0:
            warp["phase"] = 1
            s = warp["slot"]
            if self.flags[s] == 0:          # atomicCAS(flag, 0, 1) == 0
                self.flags[s] = 1
                l, self.lead = self.lead, self.lead + 1
                if l < n_lead_blocks:
                    return l // self.subs, l % self.subs
        if warp["phase"] == 1:
            m, self.main = self.main, self.main + 1
            if m < self.n_chunks - self.n_lead:
                return self.n_lead + m, -1
            warp["phase"] = 2
        l, self.lead = self.lead, self.lead + 1
        if l < n_lead_blocks:
            return l // self.subs, l % self.subs
        return None


def _taken_blocks(q, chunk, n_chunks):
    """The slot ranges of BatchIntegrator._taken_slots, as block indices."""
    subs = chunk // 32
    lead = min(q.lead, q.n_lead * subs)
    main = min(q.main, n_chunks - q.n_lead)
    blocks = set(range(lead))
    blocks |= set(range(q.n_lead * subs, (q.n_lead + main) * subs))
    return blocks


@pytest.mark.parametrize("chunk", [32, 64, 128])
@pytest.mark.parametrize("n_chunks", [1, 7, 300, 2000])
@pytest.mark.parametrize("warps_per_slot", [1, 2, 3])
def test_every_block_once_and_lead_spread(chunk, n_chunks, warps_per_slot):
    rng = np.random.default_rng(chunk * 7919 + n_chunks * 31 + warps_per_slot)
    n_slots = 64                                   # 16 SMs x 4 sub-partitions
    subs = chunk // 32
    q = Queue(n_chunks, subs, n_slots)
    warps = [{"slot": s, "phase": 0, "busy": 0} for s in range(n_slots) for _ in range(warps_per_slot)]
    seen = []
    lead_by_slot = {}
    running = list(range(len(warps)))
    while running:
        i = running[rng.integers(len(running))]
        got = q.next(warps[i])
        if got is None:
            running.remove(i)
            continue
        c, sub = got
        blocks = [c * subs + sub] if sub >= 0 else [c * subs + b for b in range(subs)]
        seen.extend(blocks)
        if sub >= 0 and warps[i]["phase"] == 1:   # a lead block taken at the warp's start
            lead_by_slot[warps[i]["slot"]] = lead_by_slot.get(warps[i]["slot"], 0) + 1
    assert sorted(seen) == list(range(n_chunks * subs))
    assert all(v == 1 for v in lead_by_slot.values())
    assert _taken_blocks(q, chunk, n_chunks) == set(seen)


@pytest.mark.parametrize("chunk", [32, 64])
def test_cancelled_run_takes_what_the_counters_say(chunk):
    rng = np.random.default_rng(11 + chunk)
    for trial in range(50):
        n_chunks = int(rng.integers(1, 400))
        subs = chunk // 32
        q = Queue(n_chunks, subs, 64)
        warps = [{"slot": s % 64, "phase": 0} for s in range(128)]
        stop = int(rng.integers(0, 3 * n_chunks + 10))   # claims before the flag is seen
        seen = set()
        claims = 0
        running = list(range(len(warps)))
        while running and claims < stop:
            i = running[rng.integers(len(running))]
            got = q.next(warps[i])
            claims += 1
            if got is None:
                running.remove(i)
                continue
            c, sub = got
            seen |= {c * subs + sub} if sub >= 0 else {c * subs + b for b in range(subs)}
        assert _taken_blocks(q, chunk, n_chunks) == seen, trial
