"""Host replay of the grid barriers of the cooperative kernels, checked on the
CPU before any GPU run.

The barriers wait on a count that only grows (zero at the launch):
* grid_barrier (dynemol_gb300/csrc/grid_sync.cuh; the Chebyshev row kernels,
  Taylor, Lanczos): a CTA arrives by an add that returns the arrivals before
  it, prev, and waits until the count reaches (prev // G + 1) G;
* oz_cheb_kernel's barrier (dynemol_gb300/csrc/ozaki.cu): the CTA's arrival at
  barrier e (the one after order_zero is e = 0) waits until the count reaches
  G (e + 1).
For any interleaving of the CTAs' arrivals, no CTA may leave a barrier before
all G have arrived at it, and all must leave once they have."""

import os
import random

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _src(name):
    return open(os.path.join(ROOT, "dynemol_gb300", "csrc", name)).read()


def test_barrier_sources_match_replay():
    gs = _src("grid_sync.cuh")
    assert "atom.add.release.gpu.global.u64 %0, [%1], 1;" in gs
    assert "const unsigned long long target = (prev / nblocks + 1) * nblocks;" in gs
    assert "ld.relaxed.gpu.global.u64" in gs and "__threadfence();  // acquire" in gs
    oz = _src("ozaki.cu")
    assert "red.release.gpu.global.add.u32 [%0], 1;" in oz
    assert "grid_barrier_sub(L.bar_count, (unsigned)G, L.error, bar_ns)" in oz
    assert "grid_barrier_sub(L.bar_count, (unsigned)G * (unsigned)(k + 1), L.error, bar_ns)" in oz


def _simulate(G, nbar, rng, target_of):
    """Event-driven replay: each CTA arrives at barriers 0 .. nbar - 1 in turn; a
    waiting CTA leaves once the count reaches its target.  Returns, per barrier,
    the number of CTAs that had arrived when each CTA left."""
    count = 0
    state = [("run", 0)] * G  # (phase, barrier index)
    waiting = {}
    left_at = [[] for _ in range(nbar)]
    arrived = [0] * nbar
    done = 0
    while done < G:
        # CTAs free to move: running ones arrive; waiting ones may leave
        ready = [c for c in range(G) if state[c][0] == "run" and state[c][1] < nbar]
        leavers = [c for c, t in waiting.items() if count >= t]
        choices = [("arrive", c) for c in ready] + [("leave", c) for c in leavers]
        assert choices, "deadlock: no CTA can move"
        kind, c = rng.choice(choices)
        e = state[c][1]
        if kind == "arrive":
            prev = count
            count += 1
            arrived[e] += 1
            waiting[c] = target_of(prev, e)
            state[c] = ("wait", e)
        else:
            left_at[e].append(arrived[e])
            del waiting[c]
            state[c] = ("run", e + 1)
            if e + 1 == nbar:
                done += 1
    return left_at, count


@pytest.mark.parametrize("G", [1, 2, 3, 7, 152])
def test_monotonic_barriers_release_only_complete_epochs(G):
    rng = random.Random(G)
    nbar = 6
    replays = {
        "grid_barrier": lambda prev, e: (prev // G + 1) * G,
        "oz_cheb_kernel": lambda prev, e: G * (e + 1),
    }
    for name, target in replays.items():
        for trial in range(20 if G < 100 else 3):
            left_at, count = _simulate(G, nbar, rng, target)
            assert count == G * nbar, name
            for e in range(nbar):
                assert len(left_at[e]) == G, (name, e)
                assert all(a == G for a in left_at[e]), (name, e)  # nobody left before all arrived


def test_epoch_of_an_arrival():
    """The grid_barrier target from the returned prev: every arrival of barrier e
    (prev in [G e, G (e + 1))) waits for G (e + 1); a 64-bit count keeps this
    exact far past any launch's barrier count."""
    for G in (1, 5, 152):
        for e in (0, 1, 17, 10 ** 9):
            for prev in (G * e, G * e + G // 2, G * (e + 1) - 1):
                assert (prev // G + 1) * G == G * (e + 1)
    assert (2 ** 63 - 1) // 152 > 10 ** 15  # barriers before a 64-bit count could wrap
