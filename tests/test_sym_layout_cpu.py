"""The slot layout of the each-pair-once sum's cluster schedule
(physim_gb300/csrc/direct_sym.cu: sym_iside_base, sym_jside_base,
sym_clusters and the kernels' write and read pattern), restated and checked
exhaustively over tile counts: every pair of tiles (I, J), I <= J, is
evaluated by exactly one cluster; every i-side and j-side slot is written by
exactly one (cluster, tile) and belongs to the tile whose bodies it holds; the
reduce reads exactly the slots written for each tile; and the slot counts are
the closed forms the allocation uses (3T^2/32 for large T).  The GPU results of
both schedules are checked in test_direct_sym_gpu.py."""
from __future__ import annotations

import pytest

C, R = 8, 16  # kSymCluster, kSymRun


def iside_base(k: int, runs: int) -> int:
    q, rem = divmod(k, R)
    return k * runs - (R * q * (q - 1) // 2 + q * rem)


def jside_base(k: int) -> int:
    q, rem = divmod(k, C)
    return k + C * q * (q - 1) // 2 + q * rem


def clusters(t: int) -> list[tuple[int, int]]:
    """(group g, run r) of every cluster, in launch order."""
    groups, runs = -(-t // C), -(-t // R)
    return [(g, r) for g in range(groups) for r in range((g * C) // R, runs)]


@pytest.mark.parametrize("t", list(range(1, 70)) + [129, 257, 1025, 2049])
def test_cluster_layout_covers_every_pair_and_slot_once(t):
    runs = -(-t // R)
    pairs = set()
    written_i, written_j = {}, {}
    for g, r in clusters(t):
        j0, j1 = r * R, min(r * R + R, t)
        for rank in range(C):
            i = g * C + rank
            if i >= t:
                continue
            for j in range(j0, j1):
                if i <= j:
                    assert (i, j) not in pairs
                    pairs.add((i, j))
            if j1 - 1 >= i:  # the block's tile I gets its run's i-side slot
                slot = iside_base(i, runs) + (r - i // R)
                assert slot not in written_i
                written_i[slot] = i
        for j in range(j0, j1):
            if g * C <= j:  # some tile of the group reaches J: one j-side slot
                slot = jside_base(j) + g
                assert slot not in written_j
                written_j[slot] = j
    assert len(pairs) == t * (t + 1) // 2
    for k in range(t):
        read_i = [iside_base(k, runs) + u for u in range(runs - k // R)]
        read_j = [jside_base(k) + u for u in range(k // C + 1)]
        assert all(written_i.get(s) == k for s in read_i)
        assert all(written_j.get(s) == k for s in read_j)
    assert len(written_i) == iside_base(t, runs)
    assert len(written_j) == jside_base(t)


def test_slot_bytes_at_a_million_bodies():
    t = 1025  # 1,048,580 bodies in 1,024-body tiles
    runs = -(-t // R)
    slots = iside_base(t, runs) + jside_base(t)
    assert slots * 3 * 1024 * 4 == 1_234_722_816  # against 12 t n = 12.9e9 for tile pairs
    assert abs(slots / (3 * t * t / 32) - 1) < 0.03
