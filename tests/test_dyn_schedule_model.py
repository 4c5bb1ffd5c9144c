"""A CPU model of the dynamic batched schedule's work distribution
(qed3_gb300/csrc/batched_dyn.cu): warps take work items step * ntiles + tile
in increasing order from one counter (each warp holding one prefetched item),
an item waits until its system has completed the previous step, the last tile
of a system's step advances the system (epoch + 1, or done after its final
step), tiles of finished systems are skipped by moving the counter past them,
and a warp leaves once every system is done.  The model runs warps with random
durations as a discrete-event simulation and checks that it always ends (no
warp waits forever), that every step of a system starts only after all tiles
of its previous step finished, and that every tile of every live step is
processed exactly once."""
import heapq

import numpy as np
import pytest


def simulate(tiles, steps, nwarps, seed):
    rng = np.random.default_rng(seed)
    nsys = len(tiles)
    ch0 = np.concatenate([[0], np.cumsum(tiles)])[:-1]
    ntiles = int(np.sum(tiles))
    sys_of_tile = np.repeat(np.arange(nsys), tiles)
    epoch = [0] * nsys           # steps completed
    done = [False] * nsys
    cnt = [0] * nsys             # tiles of the current step finished
    counter = [0]
    processed = {}               # (sys, step, tile) -> start time
    step_end = {}                # (sys, step) -> time its last tile finished

    def take():
        v = counter[0]
        counter[0] += 1
        return v

    # events: (time, seq, kind, warp); kind 0 = look at the held item, 1 = the held item's work ends
    held = {w: take() for w in range(nwarps)}
    nxt = {}
    ev = [(0.0, w, 0, w) for w in range(nwarps)]
    heapq.heapify(ev)
    seq = nwarps
    waiting = {}                 # warp -> system it waits on
    guard = 0
    while ev:
        guard += 1
        assert guard < 10_000_000, "simulation does not end"
        t, _, kind, w = heapq.heappop(ev)
        step, g = divmod(held[w], ntiles)
        s = sys_of_tile[g]
        if kind == 1:            # work done: count the tile; the last one of the step advances the system
            cnt[s] += 1
            if cnt[s] == tiles[s]:
                cnt[s] = 0
                step_end[(s, step)] = t
                if step + 1 == steps[s]:
                    done[s] = True
                epoch[s] = step + 1
                for w2, s2 in list(waiting.items()):
                    if s2 == s:
                        del waiting[w2]
                        heapq.heappush(ev, (t, seq, 0, w2))
                        seq += 1
            held[w] = nxt.pop(w)
            heapq.heappush(ev, (t, seq, 0, w))
            seq += 1
            continue
        if w not in nxt:
            nxt[w] = take()      # the next item, fetched before this one is looked at
        if done[s]:
            counter[0] = max(counter[0], step * ntiles + ch0[s] + tiles[s])  # skip its other tiles
            if all(done):
                continue         # this warp leaves
            held[w] = nxt.pop(w)
            heapq.heappush(ev, (t, seq, 0, w))
            seq += 1
            continue
        if epoch[s] < step:      # its previous step is not complete: wait until it is
            waiting[w] = s
            continue
        assert (s, step, g) not in processed
        processed[(s, step, g)] = t
        if step > 0:
            assert step_end[(s, step - 1)] <= t
        heapq.heappush(ev, (t + rng.exponential(1.0), seq, 1, w))
        seq += 1
    assert not waiting, "warps left waiting"
    assert all(done)
    for s in range(nsys):
        for k in range(steps[s]):
            for g in range(ch0[s], ch0[s] + tiles[s]):
                assert (s, k, g) in processed, (s, k, g)
    return t


@pytest.mark.parametrize("seed", range(24))
def test_dynamic_schedule_model_ends_and_orders_steps(seed):
    rng = np.random.default_rng(100 + seed)
    nsys = int(rng.integers(1, 9))
    tiles = rng.integers(1, 12, size=nsys)
    steps = rng.integers(1, 15, size=nsys)
    nwarps = int(rng.integers(1, 40))
    simulate(tiles, steps, nwarps, seed)


def test_dynamic_schedule_model_uneven_systems():
    # one long system among short ones: the short ones finish, the long one keeps every warp busy
    simulate(np.array([4, 4, 4, 16]), np.array([5, 5, 5, 40]), 24, 7)
