"""The schedule of the single-launch radix sort (physim_gb300/csrc/bh.cu:
radix_sort_kernel), restated and run as a progress model on the CPU: block b
of a grid of G resident blocks sorts tiles b, b + G, b + 2G, ... of every
pass in that order; a tile's look-back can finish only once tile t - 1 has
published its inclusive prefix; after each pass but the last every block adds
one to the barrier counter and waits for (pass + 1) * G.  Checked for grids
smaller than, equal to and larger than the tile count: every tile is sorted
exactly once per pass, no block waits forever (every wait is on a lower tile
that a resident block reaches after lower tiles only), and the barrier
targets match the arrivals.  The GPU sort itself is checked against the CPU
model and against the one-launch-per-pass form in test_bh_gpu.py."""
from __future__ import annotations

import pytest

PASSES = 7  # kSortPasses


def run_schedule(tiles: int, grid: int) -> list[list[int]]:
    """Completion order of the tiles of each pass under the model; raises if
    the blocks can make no progress."""
    done_order = []
    barrier = 0
    for p in range(PASSES):
        queues = [list(range(b, tiles, grid)) for b in range(grid)]
        published = [False] * tiles
        order = []
        while any(queues):
            progressed = False
            for q in queues:
                if q and (q[0] == 0 or published[q[0] - 1]):
                    t = q.pop(0)
                    published[t] = True
                    order.append(t)
                    progressed = True
            if not progressed:
                raise RuntimeError(f"no progress in pass {p}")
        if p + 1 < PASSES:
            barrier += grid  # every block arrives once
            assert barrier == (p + 1) * grid  # the kernel's wait target
        done_order.append(order)
    return done_order


@pytest.mark.parametrize("tiles,grid", [(1, 1), (1, 152), (5, 152), (128, 152), (152, 152),
                                        (196, 152), (305, 152), (1000, 7), (64, 1)])
def test_every_tile_once_and_every_wait_ends(tiles, grid):
    grid = min(grid, tiles)  # the host launches min(tiles, blocks per SM x SMs)
    for order in run_schedule(tiles, grid):
        assert sorted(order) == list(range(tiles))


def test_a_wait_on_an_unresident_block_would_not_end():
    """The model does detect a stuck schedule: if tile 1's block never runs
    (a grid larger than the resident blocks, which the cooperative launch
    rules out), tile 2's look-back cannot finish."""
    queues = [[0], [], [2]]  # tile 1 missing
    published = [False] * 3
    stuck = False
    while any(queues):
        progressed = False
        for q in queues:
            if q and (q[0] == 0 or published[q[0] - 1]):
                published[q.pop(0)] = True
                progressed = True
        if not progressed:
            stuck = True
            break
    assert stuck
