"""The continuous-batching request loop (physim_gb300/server.py) with a fake
executor: admission within the memory budget, first-fit ordering, arrival
times, cutoff accounting and isolation of a failing unit.  CPU only; the
failure is made on the host (an exception from a fake unit)."""
from __future__ import annotations

import pytest

from physim_gb300.server import (BYTES_FIXED, BYTES_PER_BODY_DIRECT, Executor, JobSpec, Server,
                                 Unit, latency_summary, served_mix)


class FakeUnit(Unit):
    def __init__(self, jobs, ex):
        self.jobs = list(jobs)
        self.ex = ex
        self.left = {j.id: j.steps for j in jobs}
        self.reported = set()

    def launch_tick(self):
        if any(j.id in self.ex.fail_ids for j in self.jobs):
            raise RuntimeError("injected device failure")
        self.tick_steps = 0
        for j in self.jobs:
            t = min(self.ex.k, self.left[j.id])
            self.left[j.id] -= t
            self.tick_steps += t

    def tick_done(self):
        return True

    def finished_jobs(self):
        out = []
        for j in self.jobs:
            if self.left[j.id] == 0 and j.id not in self.reported:
                self.reported.add(j.id)
                out.append((j, None))
        return out

    def alive(self):
        return len(self.reported) < len(self.jobs)

    def close(self):
        self.ex.closed += 1


class FakeExecutor(Executor):
    def __init__(self, k=10, fail_ids=()):
        self.k = k
        self.fail_ids = set(fail_ids)
        self.batches = []
        self.closed = 0
        self.max_in_use = 0
        self.server = None

    def make_units(self, jobs):
        self.batches.append([j.id for j in jobs])
        if self.server is not None:
            self.max_in_use = max(self.max_in_use, self.server.in_use)
        return [FakeUnit([j], self) for j in jobs]


def job(i, n, steps, t=0.0, gravity="simple_astro"):
    return JobSpec(arrival=t, id=i, n=n, steps=steps, gravity=gravity)


def test_all_jobs_complete_once():
    ex = FakeExecutor()
    srv = Server(ex, hbm_budget=1 << 40)
    ex.server = srv
    jobs = [job(i, 1000 + i, 5 + 3 * i, t=0.001 * i) for i in range(30)]
    srv.submit(jobs)
    res = srv.run(until=30.0)
    assert sorted(r.spec.id for r in res) == list(range(30))
    assert srv.unfinished() == 0 and srv.in_use == 0
    assert srv.steps_done == sum(j.steps for j in jobs)
    assert srv.steps_executed == sum(j.steps for j in jobs)
    for r in res:
        assert r.admitted >= r.spec.arrival and r.finished >= r.admitted
    s = latency_summary(res)
    assert s["completed"] == 30 and s["p99_s"] >= s["p50_s"]


def test_budget_is_respected_and_first_fit():
    ex = FakeExecutor(k=1)
    big = job(0, 10_000, 50)
    blocked = job(1, 15_000, 5, t=0.0001)   # does not fit beside `big`
    small = job(2, 5_000, 5, t=0.0002)      # fits: overtakes the waiting job
    budget = big.device_bytes() + small.device_bytes() + BYTES_PER_BODY_DIRECT
    assert big.device_bytes() + blocked.device_bytes() > budget
    srv = Server(ex, hbm_budget=budget)
    ex.server = srv
    srv.submit([big, blocked, small])
    srv.run(until=30.0)
    assert ex.max_in_use <= budget
    order = [i for b in ex.batches for i in b]
    assert order.index(2) < order.index(1)
    assert srv.unfinished() == 0


def test_unit_and_batch_caps():
    ex = FakeExecutor(k=1)
    srv = Server(ex, hbm_budget=1 << 40, max_units=5, max_batch=2)
    ex.server = srv
    srv.submit([job(i, 100, 30) for i in range(12)])
    srv.run(until=30.0)
    assert max(len(b) for b in ex.batches) <= 2
    assert srv.max_running <= 5
    assert len(srv.results) == 12


def test_oversized_job_is_rejected():
    ex = FakeExecutor()
    srv = Server(ex, hbm_budget=BYTES_FIXED + 10)
    srv.submit([job(0, 1_000_000, 10)])
    srv.run(until=5.0)
    assert [j.id for j in srv.rejected] == [0]
    assert not srv.results


def test_arrivals_wait_for_their_time():
    ex = FakeExecutor()
    srv = Server(ex, hbm_budget=1 << 40)
    srv.submit([job(0, 100, 1, t=0.0), job(1, 100, 1, t=0.15)])
    res = srv.run(until=10.0)
    by_id = {r.spec.id: r for r in res}
    assert by_id[1].admitted >= 0.15


def test_cutoff_leaves_jobs_unfinished():
    ex = FakeExecutor(k=1)
    srv = Server(ex, hbm_budget=1 << 40)
    srv.submit([job(i, 100, 10**9, t=0.0) for i in range(3)] + [job(9, 100, 1, t=100.0)])
    srv.run(until=0.05)
    assert srv.unfinished() == 4
    srv.close()


def test_failing_unit_is_isolated():
    ex = FakeExecutor(fail_ids={3})
    srv = Server(ex, hbm_budget=1 << 40)
    srv.submit([job(i, 100 * (i + 1), 20) for i in range(6)])
    res = srv.run(until=30.0)
    assert sorted(r.spec.id for r in res) == [0, 1, 2, 4, 5]
    assert [f.spec.id for f in srv.failed] == [3]
    assert "injected" in srv.failed[0].error
    assert srv.in_use == 0


def test_served_mix_distribution():
    jobs = served_mix(rate=50.0, seconds=20.0, seed=5)
    assert 800 < len(jobs) < 1200
    ns = [j.n for j in jobs]
    assert min(ns) >= 1024 and max(ns) <= 2_097_152
    assert all((j.gravity == "simple_astro") == (j.n < 32768) for j in jobs)
    assert {j.theta for j in jobs if j.gravity == "astro2"} <= {0.5, 1.0}
    assert all(100 <= j.steps <= 5000 for j in jobs)
    arr = [j.arrival for j in jobs]
    assert arr == sorted(arr) and arr[-1] < 20.0


def test_one_at_a_time_baseline():
    """max_units=1 / max_batch=1 runs the jobs strictly one after another in
    arrival order (the plain baseline of the served mix)."""
    ex = FakeExecutor(k=1000)
    jobs = [job(i, 1000 + i, 50, t=0.0) for i in range(6)]
    srv = Server(ex, hbm_budget=1 << 40, max_units=1, max_batch=1)
    ex.server = srv
    srv.submit(jobs)
    res = srv.run(poll=0.0)
    assert [r.spec.id for r in res] == list(range(6))
    assert ex.batches == [[i] for i in range(6)]
    assert srv.max_running == 1


def test_shortest_job_first_admission():
    """admission="shortest" admits pending jobs in order of estimated device
    work; "fifo" in arrival order."""
    jobs = [job(0, 30000, 4000), job(1, 2000, 100), job(2, 8000, 500), job(3, 1000, 50)]
    for policy, want in (("fifo", [0, 1, 2, 3]), ("shortest", [3, 1, 2, 0])):
        ex = FakeExecutor(k=10_000)
        srv = Server(ex, hbm_budget=1 << 40, max_units=1, max_batch=1, admission=policy)
        ex.server = srv
        srv.submit(jobs)
        srv.run(poll=0.0)
        assert [b[0] for b in ex.batches] == want, policy
    with pytest.raises(ValueError):
        Server(FakeExecutor(), admission="random")


class TimedUnit(FakeUnit):
    """A fake unit whose tick takes three polls and whose work is estimated
    at 1 ms per job-step."""

    def __init__(self, jobs, ex):
        super().__init__(jobs, ex)
        self.polls = 0

    def launch_tick(self):
        super().launch_tick()
        self.tick_seconds = self.tick_steps * 1e-3
        self.polls = 0
        self.ex.launches.append(self.jobs[0].id)

    def tick_done(self):
        self.polls += 1
        return self.polls >= 3

    def remaining_seconds(self):
        return sum(self.left.values()) * 1e-3


class TimedExecutor(FakeExecutor):
    def __init__(self, k=10):
        super().__init__(k=k)
        self.launches = []

    def make_units(self, jobs):
        return [TimedUnit([j], self) for j in jobs]


@pytest.mark.parametrize("scheduling", ["all", "srpt"])
def test_shortest_remaining_work_scheduling(scheduling):
    """Under "srpt" a short job that arrives while a long one runs gets the
    GPU at the long job's next tick boundary, and the two never have ticks in
    flight together (each tick's estimated work fills the in-flight budget);
    under "all" both keep a tick in flight."""
    ex = TimedExecutor(k=10)
    srv = Server(ex, hbm_budget=1 << 40, scheduling=scheduling, inflight_seconds=0.005,
                 admission="shortest")
    long_job, short_job = job(0, 1000, 400, t=0.0), job(1, 1000, 30, t=0.02)
    srv.submit([long_job, short_job])
    res = srv.run(until=60.0)
    done = {r.spec.id: r.finished for r in res}
    assert set(done) == {0, 1} and done[1] < done[0]
    assert srv.steps_executed == 430
    if scheduling == "srpt":
        assert srv.max_running == 1
        # once the short job is admitted, its 3 ticks run back to back
        first = ex.launches.index(1)
        assert ex.launches[first:first + 3] == [1, 1, 1]
    else:
        assert srv.max_running == 2


def test_unknown_scheduling_policy():
    with pytest.raises(ValueError):
        Server(FakeExecutor(), scheduling="lifo")


class SlowBuildExecutor(TimedExecutor):
    """Builds units slowly (as large initial states do) and fails one job's
    build."""

    def make_units(self, jobs):
        import time
        time.sleep(0.02)
        if any(j.id == 3 for j in jobs):
            raise RuntimeError("injected build failure")
        return super().make_units(jobs)


@pytest.mark.parametrize("scheduling", ["all", "srpt"])
def test_async_admission(scheduling):
    """Units built on a worker thread: every job completes or fails once, the
    memory budget returns to zero, and a failed build fails only its batch."""
    ex = SlowBuildExecutor(k=10)
    srv = Server(ex, hbm_budget=1 << 40, scheduling=scheduling, async_admission=True,
                 max_batch=1)
    jobs = [job(i, 1000 + i, 20 + 10 * i, t=0.005 * i) for i in range(8)]
    srv.submit(jobs)
    res = srv.run(until=60.0)
    srv.close()
    assert sorted(r.spec.id for r in res) == [0, 1, 2, 4, 5, 6, 7]
    assert [f.spec.id for f in srv.failed] == [3]
    assert srv.unfinished() == 0 and srv.in_use == 0
    assert srv.steps_executed == sum(j.steps for j in jobs if j.id != 3)


def test_device_bytes_estimates():
    """Direct-sum jobs from the symmetric size up also hold one f32 slot sum
    per 1,024-body tile and body (while those fit 4 GiB); Barnes-Hut jobs hold
    the tree workspace."""
    from physim_gb300.server import BYTES_PER_BODY_TREE, SYMMETRIC_FROM
    small = job(0, SYMMETRIC_FROM - 1, 10)
    big = job(1, 32768, 10)
    assert small.device_bytes() == BYTES_FIXED + BYTES_PER_BODY_DIRECT * small.n
    assert big.device_bytes() == BYTES_FIXED + (BYTES_PER_BODY_DIRECT + 12 * 32) * big.n
    tree = job(2, 100_000, 10, gravity="astro2")
    assert tree.device_bytes() == BYTES_FIXED + BYTES_PER_BODY_TREE * tree.n


def test_device_bytes_in_an_ensemble_mirror_plan_ensemble():
    """GpuExecutor runs direct sums in ensembles, whose each-pair-once members
    keep one [3][n] f32 slot per 1,024-body tile at any size
    (csrc/ensemble.cu, plan_ensemble) while the slots fit the library's cap (a
    quarter of a GB300's memory: up to about 2.4M bodies for one job)."""
    from physim_gb300.server import SYMMETRIC_CAP_BYTES
    for n in (500_000, 1_048_580, 2_000_000):
        j = job(0, n, 10)
        slots = 12 * -(-n // 1024) * n
        assert slots <= SYMMETRIC_CAP_BYTES
        assert j.device_bytes() == BYTES_FIXED + BYTES_PER_BODY_DIRECT * n + slots
    over = job(1, 3_000_000, 10)
    assert 12 * -(-over.n // 1024) * over.n > SYMMETRIC_CAP_BYTES
    assert over.device_bytes() == BYTES_FIXED + BYTES_PER_BODY_DIRECT * over.n


def test_device_bytes_as_a_simulation_mirror_the_symmetric_plan():
    """A direct sum run as its own simulation (PlainExecutor) counts the slot
    sums of the schedule the library picks: one [3][n] slot per tile while
    those stay within 4 GiB, the cluster schedule's triangular layout above
    (1,234,722,816 bytes at 1,048,580 bodies, the figure of the layout test),
    and none once the f64 sums and slots pass the library's cap (above about
    8.2M bodies), where a one-pair plan keeps no slot sums."""
    from physim_gb300.server import (SYM_PAIRS_SLOT_BYTES, SYMMETRIC_CAP_BYTES,
                                     symmetric_slot_bytes)
    pairs = job(0, 500_000, 10)
    t = -(-pairs.n // 1024)
    assert 12 * t * pairs.n <= SYM_PAIRS_SLOT_BYTES
    assert pairs.device_bytes("simulation") == (BYTES_FIXED
                                                + (BYTES_PER_BODY_DIRECT + 12 * t) * pairs.n)
    million = job(1, 1_048_580, 10)
    assert symmetric_slot_bytes(million.n) == 1_234_722_816
    assert million.device_bytes("simulation") == (BYTES_FIXED + BYTES_PER_BODY_DIRECT * million.n
                                                  + 1_234_722_816)
    three = job(2, 3_000_000, 10)  # a cluster plan: counted
    slots3 = symmetric_slot_bytes(three.n)
    assert 24 * three.n + slots3 <= SYMMETRIC_CAP_BYTES
    assert three.device_bytes("simulation") == (BYTES_FIXED + BYTES_PER_BODY_DIRECT * three.n
                                                + slots3)
    over = job(3, 9_000_000, 10)
    assert 24 * over.n + symmetric_slot_bytes(over.n) > SYMMETRIC_CAP_BYTES
    assert over.device_bytes("simulation") == BYTES_FIXED + BYTES_PER_BODY_DIRECT * over.n
    # the slot count grows with the square of the tiles in the cluster layout
    # (3 T^2 / 32 slots), linearly in T per body below the 4 GiB bound
    t3 = -(-three.n // 1024)
    assert abs(slots3 / (3 * t3 * t3 / 32 * 3 * 1024 * 4) - 1) < 0.02


def test_admission_uses_the_executors_estimate():
    """The server admits and releases a job with the bytes of the executor
    that runs it: ensembles for GpuExecutor, simulations for PlainExecutor
    (constructing either touches no GPU)."""
    from physim_gb300.server import GpuExecutor, PlainExecutor, Server
    big = job(0, 1_048_580, 10)
    assert GpuExecutor().job_bytes(big) == big.device_bytes()
    assert PlainExecutor().job_bytes(big) == big.device_bytes("simulation")
    assert big.device_bytes("simulation") < big.device_bytes()
    assert Server(PlainExecutor())._job_bytes(big) == big.device_bytes("simulation")
    assert Server(GpuExecutor())._job_bytes(big) == big.device_bytes()


def test_async_admission_cutoff_while_building():
    """A run cut off while units are still being built counts their jobs as
    unfinished, and close() waits for the builds and closes their units."""
    import time

    class VerySlow(TimedExecutor):
        def make_units(self, jobs):
            time.sleep(0.3)
            return super().make_units(jobs)

    ex = VerySlow(k=10)
    srv = Server(ex, hbm_budget=1 << 40, async_admission=True, max_batch=1)
    srv.submit([job(i, 1000, 50) for i in range(3)])
    res = srv.run(until=0.1)
    assert res == [] and srv.unfinished() == 3
    srv.close()
    assert ex.closed >= 1  # the unit built after the cut-off was closed


def test_all_scheduling_queue_cap_round_robin():
    """Under 'all' scheduling with queue_seconds, ticks go out least recently
    ticked unit first while the estimated work in flight is below the cap
    (at least one tick is always handed out)."""

    class SlowUnit(FakeUnit):
        def __init__(self, jobs, ex):
            super().__init__(jobs, ex)
            self.flight = 0

        def launch_tick(self):
            super().launch_tick()
            self.tick_seconds = 0.004
            self.flight = 2  # done after two polls
            self.ex.order.append(self.jobs[0].id)

        def tick_done(self):
            self.flight -= 1
            return self.flight <= 0

    class SlowExecutor(FakeExecutor):
        def __init__(self):
            super().__init__(k=5)
            self.order = []

        def make_units(self, jobs):
            return [SlowUnit([j], self) for j in jobs]

    ex = SlowExecutor()
    srv = Server(ex, hbm_budget=1 << 40, max_units=64, max_batch=64, queue_seconds=0.01)
    srv.submit([JobSpec(arrival=0.0, id=i, n=1000, steps=20) for i in range(6)])
    res = srv.run(until=30.0)
    assert len(res) == 6 and not srv.failed
    assert srv.max_running <= 3  # 3 x 4 ms reaches the 10 ms cap
    # round robin: the first six ticks go to six different units
    assert sorted(ex.order[:6]) == list(range(6))
