"""The request loop on the GPU: a staggered mix of direct-sum and Barnes-Hut
jobs is admitted while others run, their work overlaps, and every job's final
state equals the same job run alone -- bit for bit for Barnes-Hut jobs (each
is its own device-resident simulation), and within relative L2 1e-6 for
direct-sum jobs (an ensemble member splits its pair sums differently from a
solo run: FP32 rounding only)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _alone(spec):
    import physim_gb300 as pg
    from physim_gb300.server import initial_state
    cfg = pg.SimConfig(gravity=spec.gravity, theta=spec.theta, e=spec.e, dt=spec.dt,
                       leaf_size=spec.leaf_size, traversal="warp")
    with pg.Simulation(initial_state(spec), cfg) as sim:
        sim.step(spec.steps)
        return sim.download()


@pytest.mark.parametrize("policy", [{}, {"async_admission": True},
                                    {"async_admission": True, "scheduling": "srpt",
                                     "inflight_seconds": 0.01},
                                    {"async_admission": True, "queue_seconds": 0.005}])
def test_mix_equals_alone(policy):
    """Also with units built on a worker thread while others run, with
    shortest-remaining-work tick scheduling, and with a cap on the work
    queued under 'all' scheduling."""
    from physim_gb300.server import GpuExecutor, JobSpec, Server
    from test_verlet_gpu import trajectory_errors
    from physim_gb300.server import initial_state
    jobs = []
    sizes = [1000, 2500, 4096, 6000, 1500, 3000]
    for i, n in enumerate(sizes):
        jobs.append(JobSpec(arrival=0.002 * i, id=i, n=n, steps=30 + 10 * i, seed=500 + i,
                            ic="cube" if i % 2 else "plummer"))
    jobs.append(JobSpec(arrival=0.001, id=10, n=40_000, steps=20, gravity="astro2", theta=0.5,
                        seed=510))
    jobs.append(JobSpec(arrival=0.004, id=11, n=60_000, steps=15, gravity="astro2", theta=1.0,
                        seed=511, ic="plummer"))
    srv = Server(GpuExecutor(tick_ms=2.0), hbm_budget=8 << 30, keep_states=True, **policy)
    srv.submit(jobs)
    res = srv.run(until=300.0)
    srv.close()
    assert not srv.failed and srv.unfinished() == 0
    assert sorted(r.spec.id for r in res) == sorted(j.id for j in jobs)
    if policy.get("scheduling", "all") == "all":
        assert srv.max_running >= 2  # units overlapping on the device
    for r in res:
        alone = _alone(r.spec)
        if r.spec.gravity == "astro2":
            for f in ("x", "y", "z", "vx", "vy", "vz"):
                assert r.state[f].tobytes() == alone[f].tobytes(), (r.spec.id, f)
        else:
            err = trajectory_errors(initial_state(r.spec), r.state, alone)
            assert err["pos_rel_l2"] < 1e-6 and err["vel_rel_l2"] < 1e-6, (r.spec.id, err)


def test_budget_limits_concurrency():
    from physim_gb300.server import GpuExecutor, JobSpec, Server
    jobs = [JobSpec(arrival=0.0, id=i, n=50_000, steps=10, gravity="astro2", seed=600 + i)
            for i in range(6)]
    one = jobs[0].device_bytes()
    srv = Server(GpuExecutor(tick_ms=2.0, download=False), hbm_budget=2 * one + 1)
    srv.submit(jobs)
    res = srv.run(until=300.0)
    assert len(res) == 6 and not srv.failed
    assert max(in_use for _, _, _, in_use in srv.queue_depth) <= 2 * one + 1


@pytest.mark.parametrize("admission", ["fifo", "shortest"])
def test_pool_mix_equals_alone(admission):
    """Continuous batching of direct-sum jobs in a slot pool: more jobs than
    slots arrive over time, finished jobs free their slots for waiting ones
    (slots are resized in place), and every result still equals the job run
    alone (relative L2 1e-6); Barnes-Hut jobs overlap with the pool."""
    from physim_gb300.server import GpuExecutor, JobSpec, Server, initial_state
    from test_verlet_gpu import trajectory_errors
    jobs = [JobSpec(arrival=0.001 * i, id=i, n=n, steps=20 + 7 * (i % 5), seed=700 + i,
                    ic="cube" if i % 2 else "plummer")
            for i, n in enumerate([1200, 3000, 500, 2048, 4096, 700, 2500, 1800, 3500, 900])]
    jobs.append(JobSpec(arrival=0.002, id=20, n=40_000, steps=12, gravity="astro2", theta=0.5,
                        seed=720))
    ex = GpuExecutor(tick_ms=2.0, pool_slots=4, pool_bodies=4096)
    srv = Server(ex, hbm_budget=8 << 30, keep_states=True, admission=admission)
    srv.submit(jobs)
    res = srv.run(until=300.0)
    assert not srv.failed and srv.unfinished() == 0
    assert sorted(r.spec.id for r in res) == sorted(j.id for j in jobs)
    for r in res:
        alone = _alone(r.spec)
        if r.spec.gravity == "astro2":
            for f in ("x", "y", "z", "vx", "vy", "vz"):
                assert r.state[f].tobytes() == alone[f].tobytes(), (r.spec.id, f)
        else:
            err = trajectory_errors(initial_state(r.spec), r.state, alone)
            assert err["pos_rel_l2"] < 1e-6 and err["vel_rel_l2"] < 1e-6, (r.spec.id, err)
