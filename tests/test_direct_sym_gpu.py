"""simple_astro with every unordered pair evaluated once (the symmetric plan)
against the oracle (astro/src/transformers.rs:219-244) and against the
one-pair kernels, under both of its schedules: one block per tile pair (the
default up to ~600,000 bodies) and thread-block clusters (the default above;
forced here at every size with physim_gpu_set_symmetric_pairs_limit).

Tolerances: per-body relative error 1e-5 against the f64 oracle (as for the
one-pair kernels); 2e-6 against the one-pair kernels (both FP32 pair
arithmetic, differently grouped sums); NaN, fixed and untouched entries
exact; repeated passes bit-identical (the slot sums run in a fixed order)."""
from __future__ import annotations

import numpy as np
import pytest

from test_direct_gpu import RTOL, _vec, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True, params=["pairs", "clusters"])
def schedule(request):
    import physim_gb300 as pg
    pg.set_symmetric_pairs_limit(1 if request.param == "clusters" else 0)
    yield request.param
    pg.set_symmetric_pairs_limit(0)


def _sim_acc(state, e, symmetric=True, **plan):
    import physim_gb300 as pg
    with pg.Simulation(state, pg.SimConfig(gravity="simple_astro", e=e)) as sim:
        sim.set_plan(symmetric=symmetric, **plan)
        return sim.accelerations()


def _state(n, seed):
    from physim_gb300 import ics
    s = ics.cube_with_stars(max(n - 2, 0), seed=seed, stars=ics.STARS_2[: min(n, 2)])
    if n > 9:
        s["fixed"][n // 3] = 1
        s["mass"][n // 7] = 0.0  # massless: the reference's 0/0
        for k in range(n // 2, n // 2 + 3):  # coincident bodies skip each other
            s[k]["x"], s[k]["y"], s[k]["z"] = 0.125, -0.25, 0.375
    return s


@pytest.mark.parametrize("n", [1, 2, 3, 33, 1000, 1024, 1025, 2049, 4098, 12345])
def test_symmetric_matches_oracle(oracle_mod, n):
    s = _state(n, seed=n + 3)
    got = _sim_acc(s, 0.01)
    want = oracle_mod.simple_astro(s, 0.01)
    bad = np.isnan(_vec(want)).any(axis=1)
    assert np.array_equal(np.isnan(_vec(got)).any(axis=1), bad)
    ok = ~bad
    err = rel_err(got[ok], want[ok])
    assert np.all(err < RTOL), err.max()


@pytest.mark.parametrize("n", [5000, 40_000])
def test_symmetric_matches_one_pair_kernels(n):
    from physim_gb300 import ics
    s = ics.plummer(n, seed=n, a=0.1)
    a = _sim_acc(s, 1e-3)
    b = _sim_acc(s, 1e-3, symmetric=False, block=256, ipt=4, splits=2)
    assert np.all(rel_err(a, b) < 2e-6), rel_err(a, b).max()
    # deterministic: a second pass is bit-identical
    assert _vec(_sim_acc(s, 1e-3)).tobytes() == _vec(a).tobytes()


def test_symmetric_precision_vs_fp64(oracle_mod):
    """RMS relative error against the f64 direct sum, 65,536-body Plummer."""
    from physim_gb300 import ics
    s = ics.plummer(65536, seed=7, a=0.1)
    idx = np.random.default_rng(0).choice(len(s), 256, replace=False)
    want = oracle_mod.simple_astro_sample(s, 1e-3, idx)
    got = _sim_acc(s, 1e-3)[idx]
    rms = float(np.sqrt(np.mean(rel_err(got, want) ** 2)))
    assert rms < 1e-6, rms


def test_symmetric_pipeline_matches_oracle(oracle_mod):
    """4,096 cube bodies + 2 stars, e=0.01, dt=1e-5, 100 verlet steps on the
    symmetric plan against the oracle's pipeline."""
    import physim_gb300 as pg
    from physim_gb300 import ics
    from test_verlet_gpu import _trajectory_check
    s = ics.workload_direct_small()
    with pg.Simulation(s, pg.SimConfig(gravity="simple_astro", e=0.01, dt=1e-5)) as sim:
        sim.set_plan(symmetric=True)
        sim.step(100)
        got = sim.download()
    want = oracle_mod.run_pipeline(s, "simple_astro", 100, 1e-5, 0.01)
    _trajectory_check(got, want, s)


def test_plugin_large_state_uses_symmetric_plan(oracle_mod):
    """The plugin's transform at 140,000 bodies (the symmetric plan by
    default from 20,480 bodies) against the one-pair kernels and a sample of
    the f64 oracle."""
    import physim_gb300 as pg
    from physim_gb300 import ics
    s = ics.cube_with_stars(140_000 - 4, seed=9, stars=ics.STARS_4)
    acc = pg.accelerations(len(s))
    with pg.TransformElementHandler("simple_astro", {"e": 0.01}) as el:
        el.transform(s, acc)
    one = _sim_acc(s, 0.01, symmetric=False, block=128, ipt=4, splits=1)
    assert np.all(rel_err(acc, one) < 2e-6)
    idx = np.random.default_rng(2).choice(len(s), 64, replace=False)
    want = oracle_mod.simple_astro_sample(s, 0.01, idx)
    assert np.all(rel_err(acc[idx], want) < RTOL)


def test_set_plan_validation():
    import physim_gb300 as pg
    from physim_gb300 import ics
    s = ics.cube_with_stars(2000, seed=1)
    with pg.Simulation(s, pg.SimConfig(gravity="simple_astro", compensated=False)) as sim:
        with pytest.raises(pg.PhysimError):
            sim.set_plan(symmetric=True)
        with pytest.raises(pg.PhysimError):
            sim.set_plan(block=96, ipt=3)
        sim.set_plan(block=128, ipt=2, splits=3)
        sim.step(1)
    with pg.Simulation(s, pg.SimConfig(gravity="astro2")) as sim:
        with pytest.raises(pg.PhysimError):
            sim.set_plan(symmetric=True)


def test_symmetric_cap_falls_back_to_one_pair_plans(oracle_mod):
    """The heuristic plan gives 30,000 bodies the each-pair-once plan; with
    its slot buffer capped below its size it takes a one-pair plan instead,
    for simulations and for the simple_astro element, with the same results
    (within the one-pair tolerance)."""
    import physim_gb300 as pg
    s = _state(30_000, seed=77)
    cfg = pg.SimConfig(gravity="simple_astro", e=0.01)
    try:
        with pg.Simulation(s, cfg) as sim:
            assert sim.plan()["symmetric"]
            sym = sim.accelerations()
        pg.set_symmetric_cap(1 << 20)
        with pg.Simulation(s, cfg) as sim:
            plan = sim.plan()
            assert not plan["symmetric"] and plan["splits"] >= 1
            one = sim.accelerations()
        acc = pg.accelerations(len(s))
        with pg.TransformElementHandler("simple_astro", {"e": 0.01}) as el:
            el.transform(s, acc)
    finally:
        pg.set_symmetric_cap(0)
    idx = np.arange(0, len(s), 97)
    ref = oracle_mod.simple_astro_sample(s, 0.01, idx)
    live = ~np.isnan(_vec(ref)).any(axis=1) & (s["fixed"][idx] == 0)
    for got in (sym, one, acc):
        assert rel_err(got[idx][live], ref[live]).max() < RTOL
    keep = ~np.isnan(_vec(sym)).any(axis=1) & (s["fixed"] == 0)
    assert rel_err(one[keep], sym[keep]).max() < 2e-6


def test_schedules_agree():
    """The two schedules on the same state: within FP32 rounding of each other
    (2e-6 per body), each deterministic."""
    import physim_gb300 as pg
    from physim_gb300 import ics
    s = ics.plummer(30_000, seed=12, a=0.1)
    out = {}
    try:
        for name, limit in (("pairs", 0), ("clusters", 1)):
            pg.set_symmetric_pairs_limit(limit)
            out[name] = _sim_acc(s, 1e-3)
    finally:
        pg.set_symmetric_pairs_limit(0)
    assert np.all(rel_err(out["pairs"], out["clusters"]) < 2e-6)
