"""A model of the persistent kernel's schedule (step_kernel_persist in
tile_kernel.cuh), on the CPU: CTAs take work items w = level * n_tiles + tile
from one counter, in order, only while they run; an item starts when its own
tile and its neighbour tiles in the same run have finished the previous
level. The model runs random interleavings with fewer resident slots than
CTAs (CTAs that start only when another has exited, as an ordinary launch
may do) and checks that every item finishes (no deadlock) and starts only
after its dependencies, and that the dependencies are exactly the tiles
whose outputs its window overlaps when a halo is at most half an output
range."""
import random

import pytest


def neighbours(runs_of_tiles):
    """Per tile: (left, right) neighbour in its run, itself if none (the
    engine's build_tiles)."""
    nb = []
    for i, r in enumerate(runs_of_tiles):
        left = i - 1 if i > 0 and runs_of_tiles[i - 1] == r else i
        right = i + 1 if i + 1 < len(runs_of_tiles) and \
            runs_of_tiles[i + 1] == r else i
        nb.append((left, right))
    return nb


def simulate(runs_of_tiles, levels, ctas, slots, seed):
    rng = random.Random(seed)
    n = len(runs_of_tiles)
    nb = neighbours(runs_of_tiles)
    total = levels * n
    prog = [0] * n
    counter = 0
    waiting_to_start = list(range(ctas))
    running = {}          # cta -> item or None (needs to fetch)
    exited = set()
    started = []
    steps = 0
    while len(exited) < ctas:
        steps += 1
        assert steps < 100 * total * ctas + 10000, "no progress (deadlock)"
        while waiting_to_start and len(running) < slots:
            running[waiting_to_start.pop(0)] = None
        cta = rng.choice(sorted(running))
        item = running[cta]
        if item is None:                       # fetch (atomicAdd)
            if counter >= total:
                del running[cta]
                exited.add(cta)
                continue
            running[cta] = ("wait", counter)
            counter += 1
            continue
        state, w = item
        k, i = divmod(w, n)
        deps = {i, nb[i][0], nb[i][1]}
        if state == "wait":
            if all(prog[j] >= k for j in deps):
                running[cta] = ("work", w)
                started.append(w)
                for j in deps:                 # dependencies really done
                    assert prog[j] >= k
            continue
        # finish the item: progress mark, fetch the next one
        assert prog[i] == k
        prog[i] = k + 1
        running[cta] = None
    assert counter >= total
    assert all(p == levels for p in prog)
    assert sorted(started) == list(range(total))


@pytest.mark.parametrize("seed", range(12))
def test_schedule_completes_without_deadlock(seed):
    rng = random.Random(100 + seed)
    runs = []
    for r in range(rng.randint(1, 6)):
        runs += [r] * rng.randint(1, 9)
    levels = rng.randint(1, 7)
    slots = rng.randint(1, 8)
    ctas = slots + rng.randint(0, 6)          # more CTAs than slots
    simulate(runs, levels, ctas, slots, seed)


def test_window_overlaps_only_neighbour_outputs():
    """With out >= 2 halo (the engine refuses a halo above a quarter of
    the tile width W = out + 2 halo), a tile's window [start - halo,
    start + out_len + halo) meets only its own output and its neighbours'
    (the last tile of a run may be short; nothing lies beyond the run)."""
    for width in (128, 256, 512, 1024, 2048):
        for halo in (8, 16, 24, 32, 64):
            if halo * 4 > width:
                continue
            out = width - 2 * halo
            for nx in (1, 7, out - 1, out, out + 1, 3 * out + 5, 7 * out):
                starts = list(range(0, nx, out))
                rng = [(s, min(out, nx - s)) for s in starts]
                for i, (s, ln) in enumerate(rng):
                    w0, w1 = s - halo, s + ln + halo
                    for j, (s2, ln2) in enumerate(rng):
                        if abs(i - j) <= 1:
                            continue
                        assert s2 + ln2 <= w0 or s2 >= w1, \
                            (width, halo, nx, i, j)
