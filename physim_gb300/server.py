"""A continuous-batching request loop for gravity simulations.

Jobs (a physim pipeline: one gravity element + verlet, a body count, a step
count) arrive over time.  The server admits them while their device memory
fits an HBM budget, keeps every job's state on the device until it
finishes, and overlaps the work of all admitted jobs on the GPU:

  * direct-sum jobs admitted in the same admission round become the members
    of one batched ensemble (one persistent pair kernel per step for all of
    them, each member stopping at its own step count on the device);
  * Barnes-Hut jobs (astro2) run as device-resident simulations;
  * every running unit has its own CUDA stream and at most one "tick" of
    steps in flight; when a tick completes the unit gets the next one, jobs
    that finished are downloaded and their memory returns to the budget,
    and waiting jobs are admitted into the freed room.

Admission order is arrival order or shortest estimated device work first.
Ticks go either to every admitted unit at once ("all") or, under "srpt",
to the units with the least remaining estimated work while the estimated
work in flight is below a budget.  With `async_admission` the units of
admitted jobs (initial states, device allocations, uploads) are built on a
worker thread, so handing out ticks never waits for them.

Latency is measured per job from its arrival to the download of its final
state.  The device work goes through the `Executor` interface so the
scheduling logic can be exercised without a GPU (tests use a fake executor).
"""
from __future__ import annotations

import collections
import concurrent.futures
import heapq
import math
import threading
import time
from dataclasses import dataclass, field
from typing import Callable, Iterable

import numpy as np

# Device bytes per body, by how a job runs (state, f32 copy, partial sums and,
# for Barnes-Hut, the key/sort/tree workspace); used for admission.
BYTES_PER_BODY_DIRECT = 200
BYTES_PER_BODY_TREE = 700
BYTES_FIXED = 4 << 20
# Smallest direct-sum job that may evaluate each unordered pair once (the
# lowest size threshold the ensemble autotuner picks), and the largest slot
# buffer the library gives that evaluation (a quarter of a GB300's 284,208
# MiB; above it the library takes one-pair kernels, which keep no slot sums)
SYMMETRIC_FROM = 8192
SYMMETRIC_CAP_BYTES = 284_208 * (1 << 20) // 4
# The slot sums, by where a direct-sum job runs:
#   * in an ensemble (GpuExecutor): one [3][n] f32 slot per 1,024-body tile
#     for each member from the threshold up (csrc/ensemble.cu, plan_ensemble);
#   * as its own simulation (PlainExecutor): the same while those stay within
#     4 GiB (one block per tile pair), else thread-block clusters of 8 I tiles
#     over runs of 16 J tiles with [3][1,024] slots in a triangular layout
#     (csrc/direct_sym.cu, make_symmetric_plan and direct_partial_doubles)
SYM_TILE = 1024
SYM_PAIRS_SLOT_BYTES = 4 << 30
SYM_CLUSTER, SYM_RUN = 8, 16


def tile_slot_bytes(n: int) -> int:
    """Slot bytes of one [3][n] f32 slot per 1,024-body tile."""
    return 12 * (-(-n // SYM_TILE)) * n


def symmetric_slot_bytes(n: int) -> int:
    """Bytes of f32 slot sums a simulation's each-pair-once plan allocates
    for n bodies (sym_slot_floats and make_symmetric_plan in
    csrc/direct_sym.cu)."""
    t = -(-n // SYM_TILE)
    if tile_slot_bytes(n) <= SYM_PAIRS_SLOT_BYTES:
        return tile_slot_bytes(n)
    runs = -(-t // SYM_RUN)
    q, rem = divmod(t, SYM_RUN)
    iside = t * runs - (SYM_RUN * q * (q - 1) // 2 + q * rem)
    q, rem = divmod(t, SYM_CLUSTER)
    jside = t + SYM_CLUSTER * q * (q - 1) // 2 + q * rem
    return (iside + jside) * 3 * SYM_TILE * 4


@dataclass(order=True)
class JobSpec:
    arrival: float
    id: int = field(compare=False)
    n: int = field(compare=False)
    steps: int = field(compare=False)
    gravity: str = field(default="simple_astro", compare=False)  # or "astro2"
    theta: float = field(default=0.5, compare=False)
    e: float = field(default=0.01, compare=False)
    dt: float = field(default=1e-5, compare=False)
    ic: str = field(default="cube", compare=False)  # "cube" or "plummer"
    seed: int = field(default=0, compare=False)
    leaf_size: int = field(default=16, compare=False)

    def device_bytes(self, runs_as: str = "ensemble") -> int:
        """Device bytes the job holds while it runs: in an ensemble (how
        GpuExecutor runs direct sums) or as its own simulation
        (`runs_as="simulation"`, PlainExecutor and Barnes-Hut jobs)."""
        per = BYTES_PER_BODY_DIRECT if self.gravity == "simple_astro" else BYTES_PER_BODY_TREE
        slots = 0
        if self.gravity == "simple_astro" and self.n >= SYMMETRIC_FROM:
            # evaluating each unordered pair once adds the slot sums, while
            # they fit the library's cap
            if runs_as == "simulation":
                slots = symmetric_slot_bytes(self.n)
                if 24 * self.n + slots > SYMMETRIC_CAP_BYTES:
                    slots = 0
            else:
                slots = tile_slot_bytes(self.n)
                if slots > SYMMETRIC_CAP_BYTES:
                    slots = 0
        return BYTES_FIXED + per * self.n + slots

    def step_seconds(self) -> float:
        """Rough device seconds per step on one GB300 (scheduling estimates
        only): N^2 pairs at 2.3e12 pairs/s for the direct sum, 1.4 us per
        1,000 bodies plus launch latency for Barnes-Hut."""
        if self.gravity == "simple_astro":
            return self.n * self.n / 2.3e12 + 5e-6
        return self.n * 1.4e-9 + 6e-5

    def work_seconds(self) -> float:
        return self.steps * self.step_seconds()


@dataclass
class JobResult:
    spec: JobSpec
    admitted: float
    finished: float
    state: np.ndarray | None = None
    error: str | None = None

    @property
    def latency(self) -> float:
        return self.finished - self.spec.arrival


def job_initialiser(spec: JobSpec) -> tuple[str, dict]:
    """The device initialiser and its properties for a Barnes-Hut job's
    bodies: the seeded cube (x, y in [-0.5, 0.5), z in [0, 0.5)) or Plummer
    sphere (a = 0.1) of physim_gb300.initialisers, total mass 1, generated on
    the GPU where the job's state lives (no host generation or upload when
    its unit is built)."""
    if spec.ic == "plummer":
        return "plummer", {"n": spec.n, "seed": spec.seed, "a": 0.1}
    return "cube", {"n": spec.n, "seed": spec.seed, "size": 0.5}


def initial_state(spec: JobSpec) -> np.ndarray:
    """A job's initial bodies on the host: for Barnes-Hut jobs the bodies
    their units generate on the device (job_initialiser), for direct-sum jobs
    the seeded host generators of physim_gb300.ics."""
    if spec.gravity != "simple_astro":
        from . import initialisers
        kind, props = job_initialiser(spec)
        return getattr(initialisers, kind)(props)
    from . import ics
    if spec.ic == "plummer":
        return ics.plummer(spec.n, seed=spec.seed, a=0.1)
    return ics.cube_with_stars(spec.n, seed=spec.seed)


def served_mix(rate: float = 50.0, seconds: float = 120.0, seed: int = 5,
               n_lo: int = 1024, n_hi: int = 2_097_152, steps_lo: int = 100,
               steps_hi: int = 5000, direct_below: int = 32768) -> list[JobSpec]:
    """Poisson arrivals at `rate` jobs/s for `seconds`; N log-uniform in
    [n_lo, n_hi], steps uniform in [steps_lo, steps_hi]; N < direct_below runs
    the direct sum, larger N Barnes-Hut with theta drawn from {0.5, 1.0};
    cube or Plummer initial conditions with equal odds; e = 0.01, dt = 1e-5."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t, jobs, k = 0.0, [], 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            break
        n = int(math.floor(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        steps = int(rng.integers(steps_lo, steps_hi + 1))
        direct = n < direct_below
        theta = float(rng.choice([0.5, 1.0]))
        ic = "cube" if rng.random() < 0.5 else "plummer"
        jobs.append(JobSpec(arrival=t, id=k, n=n, steps=steps,
                            gravity="simple_astro" if direct else "astro2", theta=theta,
                            ic=ic, seed=1000 + k))
        k += 1
    return jobs


# ---------------------------------------------------------------------------
# device execution
# ---------------------------------------------------------------------------
class Unit:
    """A group of jobs that advances together on one stream."""

    jobs: list[JobSpec]
    tick_steps: int = 0  # job-steps enqueued by the last launch_tick
    tick_seconds: float = 0.0  # estimated device seconds of the last launched tick
    in_flight: bool = False  # a launched tick has not completed yet
    last_tick: int = -1  # order of its last tick ("all" with a queue cap: least recent first)

    def remaining_seconds(self) -> float:
        """Estimated device seconds of the unit's unfinished steps (used to
        order ticks under shortest-remaining-work scheduling)."""
        return 0.0

    def launch_tick(self) -> None: ...

    def tick_done(self) -> bool: ...

    def finished_jobs(self) -> list[tuple[JobSpec, np.ndarray | None]]:
        """Jobs that reached their step count since the last call (with states)."""
        ...

    def alive(self) -> bool: ...

    def close(self) -> None: ...


class Executor:
    def make_units(self, jobs: list[JobSpec]) -> list[Unit]: ...

    def job_bytes(self, job: JobSpec) -> int:
        """Device bytes `job` holds in this executor's units (admission)."""
        return job.device_bytes()

    def unit_cost(self, job: JobSpec) -> int:
        """Units a job adds when admitted (0: it joins an existing unit)."""
        return 1


class GpuExecutor(Executor):
    """Runs direct-sum jobs of one admission round as one ensemble and each
    Barnes-Hut job as one device-resident simulation, each on its own stream;
    a tick is about `tick_ms` of device work.  With `priorities`, a unit's
    stream gets a CUDA stream priority by its per-step cost (cheap steps run
    first when the GPU is contended), so short jobs are not held behind the
    kernels of long ones."""

    def __init__(self, device: int = 0, tick_ms: float = 20.0, download: bool = True,
                 priorities: bool = False, pool_slots: int = 0, pool_bodies: int = 32768):
        self.device = device
        self.tick_ms = tick_ms
        self.download = download
        self.priorities = priorities
        # pool_slots > 0: direct-sum jobs join one long-lived ensemble of
        # pool_slots member slots (up to pool_bodies bodies each) as slots
        # free up, instead of forming one ensemble per admission round
        self.pool_slots = pool_slots
        self.pool_bodies = pool_bodies
        self.pool: _PoolUnit | None = None

    def _pooled(self, job: JobSpec) -> bool:
        return (self.pool_slots > 0 and job.gravity == "simple_astro"
                and job.n <= self.pool_bodies)

    def unit_cost(self, job: JobSpec) -> int:
        if self._pooled(job):
            return 0 if (self.pool is not None and self.pool.alive()) else 1
        return 1

    def stream_for(self, step_seconds: float):
        """A torch stream for a unit (None: the unit makes its own)."""
        if not self.priorities:
            return None
        import torch
        # lower number = higher priority; torch clamps to the device's range
        prio = -3 if step_seconds < 1e-4 else (-2 if step_seconds < 3e-4 else
                                                 (-1 if step_seconds < 1e-3 else 0))
        return torch.cuda.Stream(device=torch.device("cuda", self.device), priority=prio)

    def make_units(self, jobs: list[JobSpec]) -> list[Unit]:
        pooled = [j for j in jobs if self._pooled(j)]
        direct = [j for j in jobs if j.gravity == "simple_astro" and not self._pooled(j)]
        tree = [j for j in jobs if j.gravity != "simple_astro"]
        units: list[Unit] = []
        if pooled:
            if self.pool is None or not self.pool.alive():
                self.pool = _PoolUnit(self)
                units.append(self.pool)
            self.pool.add(pooled)
        if direct:
            units.append(_EnsembleUnit(direct, self))
        for j in tree:
            units.append(_SimUnit(j, self))
        return units


class PlainExecutor(Executor):
    """The baseline the served mix is compared with: every job, direct sum or
    Barnes-Hut, as a plain device-resident simulation, in ticks of about
    `tick_ms` (long enough that the host's polling leaves the GPU idle for
    about 1% of the time; short enough that a job cut off by the end of a
    run gets credit for the steps it took).  Run it under a Server with
    max_units=1 and max_batch=1 to execute the jobs one at a time in arrival
    order."""

    def __init__(self, device: int = 0, download: bool = True, tick_ms: float = 100.0):
        self.device = device
        self.download = download
        self.tick_ms = tick_ms

    def make_units(self, jobs: list[JobSpec]) -> list[Unit]:
        return [_SimUnit(j, self) for j in jobs]

    def job_bytes(self, job: JobSpec) -> int:
        return job.device_bytes("simulation")


class _CudaTick:
    def __init__(self, stream_ptr: int, device: int):
        import torch
        self.torch = torch
        self.stream = torch.cuda.ExternalStream(stream_ptr, device=torch.device("cuda", device))
        self.event = None

    def record(self):
        self.event = self.torch.cuda.Event()
        self.event.record(self.stream)

    def done(self) -> bool:
        return self.event is None or self.event.query()


class _EnsembleUnit(Unit):
    def __init__(self, jobs: list[JobSpec], ex: GpuExecutor):
        from . import Ensemble, SimConfig
        self.jobs = list(jobs)
        self.ex = ex
        states = [initial_state(j) for j in jobs]
        self.torch_stream = ex.stream_for(max(j.step_seconds() for j in jobs)) \
            if hasattr(ex, "stream_for") else None
        cfg = SimConfig(gravity="simple_astro", e=0.01, dt=1e-5, device=ex.device,
                        stream=self.torch_stream.cuda_stream if self.torch_stream else None)
        self.ens = Ensemble(states, cfg, steps=[j.steps for j in jobs],
                            params=[(j.e, j.dt) for j in jobs])
        self.tick = _CudaTick(self.ens.stream, ex.device)
        pairs = sum(j.n * j.n for j in jobs)
        est_ms = max(pairs / 2.0e12 * 1e3, 0.02)
        self.k = int(max(1, min(max(j.steps for j in jobs), ex.tick_ms / est_ms)))
        self.reported: set[int] = set()
        self.left = len(jobs)
        self.host_left = [j.steps for j in jobs]  # host-side count for step accounting
        self.tick_steps = 0

    def remaining_seconds(self) -> float:
        return sum(r * j.step_seconds() for r, j in zip(self.host_left, self.jobs))

    def launch_tick(self) -> None:
        self.ens.step(self.k)
        self.tick_steps = 0
        self.tick_seconds = 0.0
        for i, r in enumerate(self.host_left):
            t = min(self.k, r)
            self.host_left[i] = r - t
            self.tick_steps += t
            self.tick_seconds += t * self.jobs[i].step_seconds()
        self.tick.record()

    def tick_done(self) -> bool:
        return self.tick.done()

    def finished_jobs(self):
        done, rem = self.ens.progress()
        out = []
        for i, j in enumerate(self.jobs):
            if i not in self.reported and rem[i] == 0:
                self.reported.add(i)
                self.left -= 1
                out.append((j, self.ens.download(i) if self.ex.download else None))
        return out

    def alive(self) -> bool:
        return self.left > 0

    def close(self) -> None:
        self.ens.close()


class _PoolUnit(Unit):
    """Continuous batching of direct-sum jobs: one ensemble of fixed member
    slots; before every tick, jobs waiting for the pool take the free slots
    (resize + upload + step budget), and after it, finished jobs are
    downloaded and their slots freed.  Each job starts with the Taylor step
    and stops at its own step count on the device, so its result is the same
    as alone."""

    def __init__(self, ex: GpuExecutor):
        from . import Ensemble, SimConfig
        self.ex = ex
        self.jobs: list[JobSpec] = []
        self.torch_stream = ex.stream_for(0.0)
        cfg = SimConfig(gravity="simple_astro", e=0.01, dt=1e-5, device=ex.device,
                        stream=self.torch_stream.cuda_stream if self.torch_stream else None)
        self.ens = Ensemble.slots([ex.pool_bodies] * ex.pool_slots, cfg)
        self.tick = _CudaTick(self.ens.stream, ex.device)
        self.slot_job: list[JobSpec | None] = [None] * ex.pool_slots
        self.slot_left = [0] * ex.pool_slots
        self.waiting: collections.deque[JobSpec] = collections.deque()
        self.tick_steps = 0
        self.closed = False

    def add(self, jobs: list[JobSpec]) -> None:
        self.waiting.extend(jobs)
        self.jobs.extend(jobs)

    def _fill(self) -> None:
        for k in range(len(self.slot_job)):
            if not self.waiting:
                break
            if self.slot_job[k] is not None:
                continue
            j = self.waiting.popleft()
            self.ens.resize_member(k, j.n)
            self.ens.upload(k, initial_state(j))
            self.ens.set_member(k, j.e, j.dt, j.steps)
            self.slot_job[k] = j
            self.slot_left[k] = j.steps

    def remaining_seconds(self) -> float:
        return (sum(self.slot_left[k] * j.step_seconds()
                    for k, j in enumerate(self.slot_job) if j is not None) +
                sum(j.work_seconds() for j in self.waiting))

    def launch_tick(self) -> None:
        self._fill()
        active = [k for k, j in enumerate(self.slot_job) if j is not None and self.slot_left[k]]
        self.tick_steps = 0
        self.tick_seconds = 0.0
        if active:
            est_ms = sum(self.slot_job[k].n ** 2 for k in active) / 2.0e12 * 1e3 + 0.02
            steps = int(max(1, min(max(self.slot_left[k] for k in active),
                                   self.ex.tick_ms / est_ms)))
            self.ens.step(steps)
            for k in active:
                t = min(steps, self.slot_left[k])
                self.slot_left[k] -= t
                self.tick_steps += t
                self.tick_seconds += t * self.slot_job[k].step_seconds()
        self.tick.record()

    def tick_done(self) -> bool:
        return self.tick.done()

    def finished_jobs(self):
        out = []
        if not any(j is not None for j in self.slot_job):
            return out
        _, rem = self.ens.progress()
        for k, j in enumerate(self.slot_job):
            if j is not None and rem[k] == 0:
                out.append((j, self.ens.download(k) if self.ex.download else None))
                self.slot_job[k] = None
                self.slot_left[k] = 0
        return out

    def alive(self) -> bool:
        return not self.closed and (bool(self.waiting) or
                                    any(j is not None for j in self.slot_job))

    def close(self) -> None:
        if not self.closed:
            self.closed = True
            self.ens.close()


class _SimUnit(Unit):
    def __init__(self, job: JobSpec, ex: GpuExecutor):
        from . import SimConfig, Simulation
        self.jobs = [job]
        self.ex = ex
        self.torch_stream = ex.stream_for(job.step_seconds()) \
            if hasattr(ex, "stream_for") else None
        kind, props = job_initialiser(job)
        self.sim = Simulation.generated(
            kind, props,
            SimConfig(gravity=job.gravity, theta=job.theta, e=job.e, dt=job.dt,
                      leaf_size=job.leaf_size, traversal="warp", device=ex.device,
                      stream=self.torch_stream.cuda_stream if self.torch_stream else None))
        self.tick = _CudaTick(self.sim.stream, ex.device)
        est_ms = max(job.n * 1.6e-6, 0.05) if job.gravity != "simple_astro" else \
            max(job.n * job.n / 2.0e12 * 1e3, 0.02)
        self.k_full = int(max(1, ex.tick_ms / est_ms))
        self.left = job.steps
        self.reported = False
        self.tick_steps = 0

    def remaining_seconds(self) -> float:
        return self.left * self.jobs[0].step_seconds()

    def launch_tick(self) -> None:
        k = min(self.k_full, self.left)
        if k > 0:
            self.sim.step(k)
            self.left -= k
        self.tick_steps = k
        self.tick_seconds = k * self.jobs[0].step_seconds()
        self.tick.record()

    def tick_done(self) -> bool:
        return self.tick.done()

    def finished_jobs(self):
        if self.left == 0 and not self.reported:
            self.reported = True
            return [(self.jobs[0], self.sim.download() if self.ex.download else None)]
        return []

    def alive(self) -> bool:
        return not self.reported

    def close(self) -> None:
        self.sim.close()


# ---------------------------------------------------------------------------
# the request loop
# ---------------------------------------------------------------------------
class Server:
    """Continuous batching: admission by memory budget, overlapping units."""

    def __init__(self, executor: Executor, hbm_budget: int = 150 << 30,
                 clock: Callable[[], float] = time.perf_counter,
                 max_units: int = 64, max_batch: int = 16, keep_states: bool = False,
                 admission: str = "fifo", scheduling: str = "all",
                 inflight_seconds: float = 0.03, async_admission: bool = False,
                 queue_seconds: float | None = None):
        if admission not in ("fifo", "shortest"):
            raise ValueError(f"unknown admission policy {admission!r}")
        if scheduling not in ("all", "srpt"):
            raise ValueError(f"unknown scheduling policy {scheduling!r}")
        self.admission = admission
        # "all": every admitted unit keeps one tick in flight, so all of them
        # share the GPU.  "srpt": ticks are handed out in order of the units'
        # estimated remaining device work, only while the estimated device
        # work already in flight is below `inflight_seconds` (at least one
        # tick is always in flight): a long job's next tick waits while
        # shorter ones run, small launch-bound units still overlap, and the
        # preemption point is the end of a tick.
        self.scheduling = scheduling
        self.inflight_seconds = inflight_seconds
        # queue_seconds (scheduling "all"): hand out ticks, least recently
        # ticked unit first, only while the estimated device work in flight
        # is below this; None hands every idle unit a tick at once.  Under a
        # saturated GPU an unbounded round enqueues seconds of work, the host
        # blocks in the launch calls and admission stalls with it.
        self.queue_seconds = queue_seconds
        self._ticks = 0
        # async_admission: admitted jobs' units (initial states, device
        # allocations, uploads) are built on a worker thread, so the loop
        # that hands out ticks never waits for them
        self._builder = (concurrent.futures.ThreadPoolExecutor(max_workers=1)
                         if async_admission else None)
        self._building: list[tuple[concurrent.futures.Future, list[JobSpec], int]] = []
        self.executor = executor
        # device bytes of a job in this executor's units (admission and release)
        self._job_bytes = getattr(executor, "job_bytes", None) or (lambda j: j.device_bytes())
        self.max_batch = max_batch
        self.keep_states = keep_states
        self.budget = hbm_budget
        self.clock = clock
        self.max_units = max_units
        self.pending: collections.deque[JobSpec] = collections.deque()
        self.arrivals: list[tuple[float, int, JobSpec]] = []  # heap: not yet arrived
        self.units: list[Unit] = []
        self.in_use = 0
        self.results: list[JobResult] = []
        self.admitted_at: dict[int, float] = {}
        self.queue_depth: list[tuple[float, int, int, int]] = []  # (t, waiting, running, in_use)
        self.rejected: list[JobSpec] = []
        self.failed: list[JobResult] = []
        self.steps_done = 0      # steps of completed jobs
        self.steps_executed = 0  # all job-steps the device finished
        self.max_running = 0  # most units with work on the device at one time
        self._lock = threading.Lock()
        self.t0 = 0.0

    def submit(self, jobs: Iterable[JobSpec]) -> None:
        with self._lock:
            for j in jobs:
                # (arrival, id): jobs arriving at the same time keep their order
                heapq.heappush(self.arrivals, (j.arrival, j.id, j))

    def _admit(self, now: float) -> None:
        while self.arrivals and self.arrivals[0][0] <= now:
            j = heapq.heappop(self.arrivals)[2]
            if self._job_bytes(j) > self.budget:
                self.rejected.append(j)  # can never fit
            else:
                self.pending.append(j)
        batch = []
        # first fit in arrival order ("fifo") or in order of estimated device
        # work ("shortest": shortest job first, ties by arrival); a job that
        # does not fit now keeps its place and later (smaller) jobs may go
        # ahead of it
        if self.admission == "shortest" and len(self.pending) > 1:
            self.pending = collections.deque(
                sorted(self.pending, key=lambda j: (j.work_seconds(), j.arrival, j.id)))
        keep = collections.deque()
        room = self.budget - self.in_use
        new_units = sum(c for _, _, c in self._building)
        cost = getattr(self.executor, "unit_cost", lambda job: 1)
        while self.pending:
            j = self.pending.popleft()
            need = self._job_bytes(j)
            c = cost(j)
            if (need <= room and len(self.units) + new_units + c <= self.max_units
                    and len(batch) < self.max_batch):
                batch.append(j)
                room -= need
                new_units += c
            else:
                keep.append(j)
        self.pending = keep
        if batch:
            for j in batch:
                self.admitted_at[j.id] = now
                self.in_use += self._job_bytes(j)
            if self._builder is not None:
                cost_new = new_units - sum(c for _, _, c in self._building)
                self._building.append((self._builder.submit(self.executor.make_units, batch),
                                       batch, cost_new))
                return
            try:
                units = self.executor.make_units(batch)
            except Exception as err:  # noqa: BLE001 -- e.g. device out of memory
                self._fail_batch(batch, err)
                return
            for u in units:
                u.in_flight = False
                self.units.append(u)
            self._dispatch()

    def _fail_batch(self, batch: list[JobSpec], err: BaseException) -> None:
        t = self.clock() - self.t0
        for j in batch:
            self.failed.append(JobResult(j, self.admitted_at.get(j.id, t), t, None, repr(err)))
            self.in_use -= self._job_bytes(j)

    def _collect_built(self) -> None:
        """Units whose building finished join the running set."""
        still = []
        for fut, batch, c in self._building:
            if not fut.done():
                still.append((fut, batch, c))
                continue
            try:
                units = fut.result()
            except Exception as err:  # noqa: BLE001 -- e.g. device out of memory
                self._fail_batch(batch, err)
                continue
            for u in units:
                u.in_flight = False
                self.units.append(u)
        self._building = still

    def _fail_unit(self, u: Unit, err: BaseException) -> None:
        """A unit whose device work raised: its unfinished jobs fail, their
        memory returns to the budget, the other units keep running."""
        done_ids = {r.spec.id for r in self.results}
        t = self.clock() - self.t0
        for j in u.jobs:
            if j.id not in done_ids:
                self.failed.append(JobResult(j, self.admitted_at.get(j.id, t), t, None, repr(err)))
                self.in_use -= self._job_bytes(j)
        try:
            u.close()
        except Exception:
            pass

    def _launch(self, u: Unit) -> bool:
        try:
            u.launch_tick()
            u.in_flight = True
            return True
        except Exception as err:  # noqa: BLE001 -- isolate the failing unit
            self._fail_unit(u, err)
            self.units.remove(u)
            return False

    def _dispatch(self) -> None:
        """Hands out ticks to the units that have none in flight."""
        idle = [u for u in self.units if not u.in_flight]
        if self.scheduling == "all" and self.queue_seconds is None:
            for u in idle:
                self._launch(u)
        elif self.scheduling == "all":
            inflight = sum(u.tick_seconds for u in self.units if u.in_flight)
            for u in sorted(idle, key=lambda v: v.last_tick):
                if inflight >= self.queue_seconds:
                    break
                if self._launch(u):
                    self._ticks += 1
                    u.last_tick = self._ticks
                    inflight += u.tick_seconds
        else:
            busy = [u for u in self.units if u.in_flight]
            inflight = sum(u.tick_seconds for u in busy)
            for u in sorted(idle, key=lambda v: v.remaining_seconds()):
                if busy and inflight >= self.inflight_seconds:
                    break
                if self._launch(u):
                    busy.append(u)
                    inflight += u.tick_seconds
        self.max_running = max(self.max_running, sum(1 for u in self.units if u.in_flight))

    def _service(self, now: float) -> None:
        if self._building:
            self._collect_built()
        still = []
        for u in self.units:
            try:
                if u.in_flight:
                    if not u.tick_done():
                        still.append(u)
                        continue
                    u.in_flight = False
                    self.steps_executed += u.tick_steps
                    u.tick_steps = 0
                    for j, state in u.finished_jobs():
                        t = self.clock() - self.t0
                        self.results.append(JobResult(j, self.admitted_at[j.id], t,
                                                      state if self.keep_states else None))
                        self.in_use -= self._job_bytes(j)
                        self.steps_done += j.steps
                if u.alive():
                    still.append(u)
                else:
                    u.close()
            except Exception as err:  # noqa: BLE001 -- isolate the failing unit
                self._fail_unit(u, err)
        self.units = still
        self._dispatch()

    def run(self, until: float | None = None, poll: float = 0.001,
            sample_every: float = 0.25) -> list[JobResult]:
        """Serves until every submitted job finished, or until `until` seconds
        after the start (jobs still running then are left unfinished)."""
        self.t0 = self.clock()
        next_sample = 0.0
        while True:
            now = self.clock() - self.t0
            if until is not None and now >= until:
                break
            with self._lock:
                self._admit(now)
            self._service(now)
            if now >= next_sample:
                self.queue_depth.append((now, len(self.pending), len(self.units), self.in_use))
                next_sample = now + sample_every
            if not self.units and not self.pending and not self.arrivals and not self._building:
                break
            time.sleep(poll)
        return self.results

    def unfinished(self) -> int:
        done_ids = {r.spec.id for r in self.results} | {f.spec.id for f in self.failed}
        running = sum(1 for u in self.units for j in u.jobs if j.id not in done_ids)
        building = sum(len(b) for _, b, _ in self._building)
        return running + building + len(self.pending) + len(self.arrivals)

    def close(self) -> None:
        if self._builder is not None:
            self._builder.shutdown(wait=True)
            for fut, _, _ in self._building:
                try:
                    for u in fut.result():
                        u.close()
                except Exception:  # noqa: BLE001 -- its jobs are already unfinished
                    pass
            self._building = []
        for u in self.units:
            u.close()
        self.units = []


def latency_summary(results: list[JobResult]) -> dict:
    if not results:
        return {"completed": 0}
    lat = np.array([r.latency for r in results])
    return {"completed": len(results), "p50_s": float(np.percentile(lat, 50)),
            "p99_s": float(np.percentile(lat, 99)), "mean_s": float(lat.mean()),
            "max_s": float(lat.max())}
