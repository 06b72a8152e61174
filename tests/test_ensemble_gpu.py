"""Batched ensembles (physim_gpu_ensemble_*): every member's trajectory equals
its solo run (the same pair arithmetic, partial sums split differently: FP32
rounding only, relative L2 error below 1e-6 after 20 steps) and the oracle's
(below 1e-5), with per-member parameters and step budgets."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _members():
    from physim_gb300 import ics
    sizes = [256, 300, 1000, 1025, 4096, 5000, 700, 2048, 257, 12345]
    out = []
    for k, n in enumerate(sizes):
        if k % 2:
            out.append(ics.plummer(n, seed=100 + k, a=0.1))
        else:
            out.append(ics.cube_with_stars(n, seed=100 + k))
    return out


def _solo(state, steps, e=0.01, dt=1e-5):
    import physim_gb300 as pg
    with pg.Simulation(state, pg.SimConfig(gravity="simple_astro", e=e, dt=dt)) as sim:
        sim.step(steps)
        return sim.download()


def test_members_match_solo_runs():
    import physim_gb300 as pg
    from test_verlet_gpu import trajectory_errors
    members = _members()
    with pg.Ensemble(members, pg.SimConfig(gravity="simple_astro", e=0.01, dt=1e-5)) as ens:
        ens.step(20)
        got = [ens.download(k) for k in range(len(members))]
        done, _ = ens.progress()
    assert np.all(done == 20)
    for k, s in enumerate(members):
        err = trajectory_errors(s, got[k], _solo(s, 20))
        assert err["pos_rel_l2"] < 1e-6 and err["vel_rel_l2"] < 1e-6, (k, err)


def test_member_matches_oracle(oracle_mod):
    import physim_gb300 as pg
    from test_verlet_gpu import trajectory_errors
    members = _members()[:4]
    with pg.Ensemble(members, pg.SimConfig(gravity="simple_astro", e=0.01, dt=1e-5)) as ens:
        ens.step(5)
        got = ens.download(2)
    want = oracle_mod.run_pipeline(members[2], "simple_astro", 5, 1e-5, 0.01)
    err = trajectory_errors(members[2], got, want)
    assert err["pos_rel_l2"] < 1e-5 and err["vel_rel_l2"] < 1e-5, err


def test_budgets_and_parameters():
    import physim_gb300 as pg
    from test_verlet_gpu import trajectory_errors
    members = _members()[:6]
    params = [(0.01, 1e-5), (0.02, 2e-5), (0.01, 1e-5), (0.05, 1e-5), (0.01, 3e-5), (0.01, 1e-5)]
    budgets = [5, 10, 3, 10, 0, 7]
    cfg = pg.SimConfig(gravity="simple_astro", e=0.01, dt=1e-5)
    with pg.Ensemble(members, cfg, steps=budgets, params=params) as ens:
        ens.step(4)
        ens.step(6)
        done, rem = ens.progress()
        got = [ens.download(k) for k in range(len(members))]
    assert list(done) == [5, 10, 3, 10, 0, 7]
    assert np.all(rem == 0)
    for k, s in enumerate(members):
        if budgets[k] == 0:
            assert got[k]["x"].tobytes() == s["x"].tobytes()
            continue
        e, dt = params[k]
        err = trajectory_errors(s, got[k], _solo(s, budgets[k], e=e, dt=dt))
        assert err["pos_rel_l2"] < 1e-6 and err["vel_rel_l2"] < 1e-6, (k, err)


def test_autotune_keeps_results():
    import physim_gb300 as pg
    from test_verlet_gpu import trajectory_errors
    members = _members()
    cfg = pg.SimConfig(gravity="simple_astro", e=0.01, dt=1e-5)
    with pg.Ensemble(members, cfg) as ens:
        plan = ens.autotune()
        ens.step(10)
        got = [ens.download(k) for k in range(len(members))]
    assert plan["candidates"] >= 8 and plan["force_ms"] > 0
    for k in (0, 5, 9):
        err = trajectory_errors(members[k], got[k], _solo(members[k], 10))
        assert err["pos_rel_l2"] < 1e-6, (k, err)


def test_upload_resets_member():
    import physim_gb300 as pg
    from test_verlet_gpu import trajectory_errors
    members = _members()[:3]
    cfg = pg.SimConfig(gravity="simple_astro", e=0.01, dt=1e-5)
    with pg.Ensemble(members, cfg) as ens:
        ens.step(3)
        ens.upload(1, members[1])
        ens.step(2)
        got1 = ens.download(1)
        done, _ = ens.progress()
    assert list(done) == [5, 2, 5]
    err = trajectory_errors(members[1], got1, _solo(members[1], 2))
    assert err["pos_rel_l2"] < 1e-6, err


def test_resized_slots_match_solo_runs():
    """Continuous batching: empty slots take new members of any size up to
    their capacity, mid-run, while other members keep stepping; each equals
    its solo run, and a slot shrunk to a smaller member leaves no stale
    bodies behind (the larger previous occupant's bodies would add force)."""
    import physim_gb300 as pg
    from physim_gb300 import ics
    from test_verlet_gpu import trajectory_errors
    cfg = pg.SimConfig(gravity="simple_astro", e=0.01, dt=1e-5)
    big = ics.cube_with_stars(3000, seed=900)
    small = ics.plummer(700, seed=901, a=0.1)
    other = ics.cube_with_stars(1500, seed=902)
    ens = pg.Ensemble.slots([4096, 4096], cfg)
    try:
        ens.resize_member(0, len(big))
        ens.upload(0, big)
        ens.set_member(0, 0.01, 1e-5, 6)
        ens.resize_member(1, len(other))
        ens.upload(1, other)
        ens.set_member(1, 0.01, 1e-5, 12)
        ens.step(6)
        got_big = ens.download(0)
        ens.resize_member(0, len(small))  # slot 0 now holds a smaller job
        ens.upload(0, small)
        ens.set_member(0, 0.01, 1e-5, 5)
        ens.step(6)
        got_small = ens.download(0)
        got_other = ens.download(1)
        done, rem = ens.progress()
    finally:
        ens.close()
    assert list(done) == [5, 12] and list(rem) == [0, 0]
    for s, g, k in ((big, got_big, 6), (small, got_small, 5), (other, got_other, 12)):
        err = trajectory_errors(s, g, _solo(s, k))
        assert err["pos_rel_l2"] < 1e-6 and err["vel_rel_l2"] < 1e-6, err


def _big_members():
    """Members on both sides of the default symmetric threshold (16,384
    bodies), one with a fixed body."""
    from physim_gb300 import ics
    out = [ics.cube_with_stars(20000, seed=301), ics.plummer(1000, seed=302, a=0.1),
           ics.plummer(40000, seed=303, a=0.1), ics.cube_with_stars(16384, seed=304),
           ics.cube_with_stars(5000, seed=305)]
    out[0]["fixed"][7] = 1
    return out


def test_symmetric_members_match_solo_runs():
    """Members from 16,384 bodies evaluate each unordered pair once (slot
    sums added in the verlet kernel); every member still equals its solo run
    and the oracle."""
    import physim_gb300 as pg
    from test_verlet_gpu import trajectory_errors
    members = _big_members()
    with pg.Ensemble(members, pg.SimConfig(gravity="simple_astro", e=0.01, dt=1e-5)) as ens:
        assert ens.launches_per_step == 4  # symmetric + one-pair pair kernels, verlet, count
        ens.step(10)
        got = [ens.download(k) for k in range(len(members))]
    for k, s in enumerate(members):
        err = trajectory_errors(s, got[k], _solo(s, 10))
        assert err["pos_rel_l2"] < 1e-6 and err["vel_rel_l2"] < 1e-6, (k, err)


def test_symmetric_member_matches_oracle(oracle_mod):
    import physim_gb300 as pg
    from test_verlet_gpu import trajectory_errors
    members = _big_members()[:1]
    with pg.Ensemble(members, pg.SimConfig(gravity="simple_astro", e=0.01, dt=1e-5)) as ens:
        ens.step(3)
        got = ens.download(0)
    want = oracle_mod.run_pipeline(members[0], "simple_astro", 3, 1e-5, 0.01)
    err = trajectory_errors(members[0], got, want)
    assert err["pos_rel_l2"] < 1e-5 and err["vel_rel_l2"] < 1e-5, err


def test_autotune_with_symmetric_members():
    import physim_gb300 as pg
    from test_verlet_gpu import trajectory_errors
    members = _big_members()
    with pg.Ensemble(members, pg.SimConfig(gravity="simple_astro", e=0.01, dt=1e-5)) as ens:
        plan = ens.autotune()
        ens.step(5)
        got = [ens.download(k) for k in range(len(members))]
    assert plan["candidates"] >= 20 and plan["symmetric_from"] in (0, 8192, 16384, 32768)
    for k, s in enumerate(members):
        err = trajectory_errors(s, got[k], _solo(s, 5))
        assert err["pos_rel_l2"] < 1e-6, (k, plan, err)


def test_resized_slot_crosses_symmetric_threshold():
    """A slot of 40,000 bodies holds a symmetric member, then a smaller
    symmetric one, then a one-pair one: each equals its solo run."""
    import physim_gb300 as pg
    from physim_gb300 import ics
    from test_verlet_gpu import trajectory_errors
    cfg = pg.SimConfig(gravity="simple_astro", e=0.01, dt=1e-5)
    jobs = [ics.plummer(40000, seed=310, a=0.1), ics.cube_with_stars(18000, seed=311),
            ics.plummer(3000, seed=312, a=0.1)]
    other = ics.cube_with_stars(17000, seed=313)
    ens = pg.Ensemble.slots([40000, 17000], cfg)
    try:
        ens.resize_member(1, len(other))
        ens.upload(1, other)
        ens.set_member(1, 0.01, 1e-5, 9)
        for job in jobs:
            ens.resize_member(0, len(job))
            ens.upload(0, job)
            ens.set_member(0, 0.01, 1e-5, 3)
            ens.step(3)
            got = ens.download(0)
            err = trajectory_errors(job, got, _solo(job, 3))
            assert err["pos_rel_l2"] < 1e-6 and err["vel_rel_l2"] < 1e-6, (len(job), err)
        got_other = ens.download(1)
    finally:
        ens.close()
    err = trajectory_errors(other, got_other, _solo(other, 9))
    assert err["pos_rel_l2"] < 1e-6, err
