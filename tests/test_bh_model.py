"""The CPU model of the GPU tree build (oracle/bh_model.c) against the
reference's pointer trees (octree.rs / quadtree.rs restated in the oracle).

With leaf size 1 the level-by-level tree over Morton keys has exactly the
reference tree's cells: same geometric centres and half-widths (bit for bit)
and the same number of children per cell.  CPU only."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest


def reference_cells(oracle_mod, state, nchild):
    X = oracle_mod.load().oracle_state_extent(state.ctypes.data, len(state))
    t = oracle_mod.Tree(nchild, (0.0, 0.0, 0.0), X)
    for e in state:
        assert t.push(e) == 0
    n = t.node_count()
    geom = np.zeros(4 * n)
    kids = np.zeros(n, np.int32)
    oracle_mod.load().oracle_tree_dump(C.c_void_p(t.h), geom.ctypes.data, kids.ctypes.data, n)
    return geom.reshape(n, 4), kids


def model_cells(oracle_mod, state, nchild, leaf=1):
    m = oracle_mod.bh_model(state, nchild, leaf)
    return m["centre"].T.copy(), m["nchild"].astype(np.int32), m


def _canon(geom, kids):
    rec = np.concatenate([geom, kids[:, None].astype(np.float64)], axis=1)
    return rec[np.lexsort(rec.T[::-1])]


def _states():
    from physim_gb300 import ics
    rng = np.random.default_rng(8)
    out = {"cube": ics.cube_with_stars(5000, seed=81, stars=ics.STARS_4),
           "plummer": ics.plummer(5000, seed=82, a=0.05)}
    s = ics.cube_with_stars(800, seed=83)
    # bodies exactly on cell boundaries at several levels
    X = np.abs(np.stack([s["x"], s["y"], s["z"]])).max()
    seen = set()
    k = 0
    while k < 40:  # distinct (x, y): the reference quadtree cannot separate equal x, y
        lvl = 1 + k % 6
        x = X * (rng.integers(-(2 ** lvl) + 1, 2 ** lvl) / 2 ** lvl)
        y = X * (rng.integers(-(2 ** lvl) + 1, 2 ** lvl) / 2 ** lvl)
        if (x, y) in seen:
            continue
        seen.add((x, y))
        s[k]["x"], s[k]["y"] = x, y
        k += 1
    out["boundaries"] = s
    return out


@pytest.mark.parametrize("name", ["cube", "plummer", "boundaries"])
@pytest.mark.parametrize("nchild", [8, 4])
def test_leaf1_model_equals_reference_tree(oracle_mod, name, nchild):
    s = _states()[name]
    rg, rk = reference_cells(oracle_mod, s, nchild)
    mg, mk, _ = model_cells(oracle_mod, s, nchild)
    assert len(rg) == len(mg)
    assert np.array_equal(_canon(rg, rk), _canon(mg, mk))


def test_keys_follow_reference_octants(oracle_mod):
    """Level-1 digit of every key is the reference's octant id at the root."""
    from physim_gb300 import ics
    s = ics.cube_with_stars(2000, seed=84)
    m = oracle_mod.bh_model(s, 8, 16)
    keys = np.zeros(len(s), np.uint64)
    oracle_mod.load().bh_model_keys(s.ctypes.data, len(s), 8, keys.ctypes.data)
    oct_id = (s["x"] > 0).astype(int) | ((s["y"] > 0).astype(int) << 1) | ((s["z"] > 0).astype(int) << 2)
    assert np.array_equal((keys >> np.uint64(60)).astype(int), oct_id)
    assert np.all(np.diff(m["keys"].astype(np.float64)) >= 0)
    assert np.array_equal(np.sort(m["order"]), np.arange(len(s)))


def test_leaf_sizes_and_ranges(oracle_mod):
    from physim_gb300 import ics
    s = ics.cube_with_stars(10000, seed=85, stars=ics.STARS_2)
    for leaf in (1, 4, 16, 64):
        m = oracle_mod.bh_model(s, 8, leaf)
        leaves = m["child"] < 0
        keys = m["keys"]
        for b, c in zip(m["begin"][leaves], m["count"][leaves]):
            assert c <= leaf or keys[b] == keys[b + c - 1]
        # children partition their parent's range
        for i in np.nonzero(~leaves)[0][:200]:
            f, k = m["child"][i], m["nchild"][i]
            assert m["begin"][f] == m["begin"][i]
            assert m["count"][f:f + k].sum() == m["count"][i]
