"""The window questions of the Barnes-Hut level-mask pass
(physim_gb300/csrc/bh.cu: mask_kernel), restated and checked against the
direct loops they replace, on random tiles of key-prefix lengths L (values
-1 .. D, long runs of deep values, "no boundary" markers at either end) and
every leaf size 1..64:

  * the minimum of L over the next `leaf` boundaries, from two overlapping
    entries of the window-minimum tables;
  * the consecutive boundaries at or below a level before and after a body,
    up to `leaf` each, by binary lifting over the tables;
  * the consecutive boundaries at or below a level after a body up to the
    tile's end (the leaf's length), by 64-boundary steps then lifting.

The GPU trees built this way are checked bit for bit against the CPU model in
test_bh_gpu.py."""
from __future__ import annotations

import numpy as np
import pytest

BLOCK, HALO = 1024, 72  # kTreeBlock, kTreeHalo
TILE = BLOCK + 2 * HALO  # kTreeTile
TABLES = 7  # kMinTables: windows of 1, 2, 4, ..., 64 boundaries


def window_tables(sl: np.ndarray) -> list[np.ndarray]:
    """tab[q][t] = min of sl[t .. t + 2^q - 1], clipped at the tile's end."""
    tab = [sl.astype(np.int64)]
    for q in range(1, TABLES):
        h = 1 << (q - 1)
        prev = tab[-1]
        cur = prev.copy()
        cur[:TILE - h] = np.minimum(prev[:TILE - h], prev[h:])
        tab.append(cur)
    return tab


def leaf_window_min(tab, s: int, leaf: int) -> int:
    q = leaf.bit_length() - 1
    return int(min(tab[q][s + 1], tab[q][s + leaf + 1 - (1 << q)]))


def runs_either_side(tab, s: int, leaf: int, level: int) -> tuple[int, int]:
    lft = rgt = 0
    for q in range(TABLES - 1, -1, -1):
        k = 1 << q
        if lft + k <= leaf and tab[q][s - lft - k] >= level:
            lft += k
        if rgt + k <= leaf and tab[q][s + rgt + 1] >= level:
            rgt += k
    return lft, rgt


def run_to_tile_end(tab, s: int, level: int) -> int:
    room = TILE - 1 - s
    run = 0
    while run + 64 <= room and tab[6][s + 1 + run] >= level:
        run += 64
    for q in range(TABLES - 2, -1, -1):
        k = 1 << q
        if run + k <= room and tab[q][s + 1 + run] >= level:
            run += k
    return run


def random_tile(rng, depth: int) -> np.ndarray:
    sl = rng.integers(0, depth + 1, TILE)
    if rng.random() < 0.5:  # mostly deep boundaries: long runs
        sl = np.where(rng.random(TILE) < 0.85, rng.integers(depth - 3, depth + 1, TILE), sl)
    if rng.random() < 0.3:  # the state ends inside the tile
        sl[int(rng.integers(HALO, TILE)):] = -1
    if rng.random() < 0.3:  # the tile starts before body 1
        sl[:int(rng.integers(1, HALO + 8))] = -1
    return sl


@pytest.mark.parametrize("seed", range(4))
def test_window_tables_answer_as_the_loops_do(seed):
    rng = np.random.default_rng(seed)
    for trial in range(64):
        depth = int(rng.choice([10, 21]))  # quadtree and octree key depths
        leaf = 1 + (trial + 16 * seed) % 64
        sl = random_tile(rng, depth)
        tab = window_tables(sl)
        for tid in rng.integers(0, BLOCK, 48):
            s = int(tid) + HALO
            if (sl[s + 1:s + leaf + 1] >= 0).all():
                want = min([depth] + [int(v) for v in sl[s + 1:s + leaf + 1]])
                assert leaf_window_min(tab, s, leaf) == want
            level = int(sl[s])
            if level >= 0:
                lft = 0
                while lft < leaf and sl[s - lft - 1] >= level:
                    lft += 1
                rgt = 0
                while rgt < leaf and sl[s + rgt + 1] >= level:
                    rgt += 1
                assert runs_either_side(tab, s, leaf, level) == (lft, rgt)
            lf = int(rng.integers(0, depth + 1))
            t = s + 1
            while t < TILE and sl[t] >= lf:
                t += 1
            assert s + 1 + run_to_tile_end(tab, s, lf) == t


def test_queries_stay_inside_the_tile():
    """Every table entry a query reads covers boundaries inside the tile,
    for the extreme slots and the largest leaf."""
    for leaf in (1, 63, 64):
        for s in (HALO, HALO + BLOCK - 1):
            q = leaf.bit_length() - 1
            assert s + leaf + 1 - (1 << q) + (1 << q) - 1 <= TILE - 1
            assert s - leaf >= 0 and s + leaf <= TILE - 1
