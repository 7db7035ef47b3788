"""The paste trick's settling rule, on the host: the frontier rounds that
aggregate.cu's paste_* kernels run (count killers; groups without killers are
processed; a popped processed group switches its victims off, a popped
switched-off group counts them down, the last one settles a victim as
processed) give the same processed set as the reference's sequential mask
walk (nldct.cpp:2302-2322), on random switch-off graphs with repeated edges."""
import numpy as np
import pytest


def sequential(n, victims):
    alive = np.zeros(n, bool)
    off = np.zeros(n, bool)
    for g in range(n):
        if off[g]:
            continue
        alive[g] = True
        for v in victims[g]:
            off[v] = True
    return alive


def frontier_rounds(n, victims, rng):
    pending = np.zeros(n, int)
    for g in range(n):
        for v in victims[g]:
            pending[v] += 1
    state = np.where(pending == 0, 1, 0)      # 0 undecided, 1 processed, 2 switched off
    frontier = list(np.nonzero(state == 1)[0])
    rounds = 0
    while frontier:
        rounds += 1
        rng.shuffle(frontier)                  # pops within a round run in any order
        nxt = []
        for g in frontier:
            for v in victims[g]:
                if state[g] == 1:
                    if state[v] == 0:
                        state[v] = 2
                        nxt.append(v)
                else:
                    pending[v] -= 1
                    if pending[v] == 0 and state[v] == 0:
                        state[v] = 1
                        nxt.append(v)
        frontier = nxt
    assert (state != 0).all()
    return state == 1, rounds


@pytest.mark.parametrize("seed", range(8))
def test_frontier_rounds_match_the_sequential_walk(seed):
    rng = np.random.default_rng(seed)
    n = 400
    victims = []
    for g in range(n):
        k = rng.integers(0, 12)
        # later groups nearby (as switch-offs are: neighbours of the members),
        # with repeats
        vs = [int(v) for v in g + 1 + rng.integers(0, 30, size=k) if v < n]
        victims.append(vs)
    alive, rounds = frontier_rounds(n, victims, rng)
    assert np.array_equal(alive, sequential(n, victims))
    assert rounds <= n + 1
