"""Benchmark: direct-sum gravity + verlet at N = 1,048,580 on GB300.

One step = one pipeline step of physim with the simple_astro element and the
verlet integrator over 1,048,576 cube bodies + 4 stars (e = 0.01, dt = 1e-5):
N(N-1) pair interactions plus the f64 kick-drift.  Prints one JSON line.

  value     Gpair-interactions/s of the device-resident path (state in HBM;
            CUDA events on the simulation's stream around each step, L2
            flushed between timed steps).
  e2e       the same metric through the plugin C ABI with host Entity arrays:
            simple_astro_transform + physim_gpu_verlet_integrate per step,
            host<->device transfers inside the timed region (wall clock).  On a
            device that reaches pageable host memory (Grace over NVLink-C2C)
            the kernels read and write the host arrays in place ("transfer":
            "direct"); value_with_copies is the same run with cudaMemcpyAsync.
  roofline  the pair kernel against the FP32 peak: 20 flop per ordered pair
            (Nyland, Harris & Prins, GPU Gems 3 ch. 31), or 27 per unordered
            pair when the autotuner picks the symmetric kernel (each pair
            evaluated once, both bodies updated), over the kernel's event
            time; peak = SMs x 128 FP32 lanes x 2 x max SM clock.
  cpu_baseline  the C restatement of the reference (single thread, as physim's
            transform runs) on a bounded sample of bodies.

--impl reference times the reference algorithm's CPU implementation (the C
restatement, the Rust reference cannot be built here) on all host cores: each
step is a bounded sample of one full step (a fixed number of bodies against
all their partners), ms_per_step is the time that sample took, and the line
also carries a single-thread figure (physim's transform runs on one thread).
That arm imports only numpy modules of the package and the oracle, so the
CUDA library is never loaded into it.
Under torchrun every rank runs an independent replica (the path has no
exchange step); value is the sum of the ranks' pairs over the slowest rank.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_CUBE = 1_048_576
E = 0.01
DT = 1e-5
FLOP_PER_PAIR = 20
# one unordered pair of the symmetric kernel: 3 FADD (d), FMUL + 2 FFMA (r^2),
# FADD + FMUL + FFMA (the argument), rsqrt, FMUL + 3 FFMA (a_i), FMUL + 3 FFMA
# (a_j), counting an FFMA as 2 flop and the rsqrt as 1
FLOP_PER_SYM_PAIR = 27
FP32_LANES_PER_SM = 128
METRIC = "Gpair-interactions/s at N=1M (direct-sum simple_astro + verlet)"
WORKLOAD = "direct-sum N=1,048,580 (1,048,576 cube U[-0.5,0.5]^3 seed 1 + 4 stars m=1e5), e=0.01, verlet dt=1e-5"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--cpu-seconds", type=float, default=12.0,
                   help="target seconds of CPU work for the CPU-baseline sample")
    p.add_argument("--e2e-steps", type=int, default=None)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--skip-e2e", action="store_true", help="profiling runs: device path only")
    p.add_argument("--only", default="",
                   help="comma list of parts: direct, bh, ensemble, served, precision; tour "
                        "(every kernel once, for launch lists)")
    p.add_argument("--precision-steps", type=int, default=200)
    p.add_argument("--precision-bodies", type=int, default=262_144)
    p.add_argument("--precision-variants", default="",
                   help="comma list of precision-study variants (default: all)")
    p.add_argument("--serve-seconds", type=float, default=120.0,
                   help="seconds of Poisson arrivals of the served mix (the configured 120 s)")
    p.add_argument("--serve-admission", choices=["shortest", "fifo"], default="shortest",
                   help="admission order of the served run (the one-at-a-time baselines run "
                        "both orders)")
    p.add_argument("--serve-drain", type=float, default=30.0)
    p.add_argument("--serve-scheduling", choices=["srpt", "all"], default="all",
                   help="tick scheduling of the served run: shortest remaining work first "
                        "within an in-flight budget, or every admitted unit at once")
    p.add_argument("--serve-inflight-ms", type=float, default=30.0,
                   help="estimated device work kept in flight under srpt scheduling")
    p.add_argument("--serve-queue-ms", type=float, default=0.0,
                   help="under 'all' scheduling, estimated device work queued at most (units "
                        "ticked least recently first); 0 hands every idle unit a tick at once")
    p.add_argument("--serve-max-units", type=int, default=2048,
                   help="most units (ensembles, simulations) admitted at one time; the default "
                        "is high enough that the 150 GB HBM budget is what limits admission")
    p.add_argument("--serve-fifo-baseline", action="store_true",
                   help="also run the one-at-a-time baseline in arrival order")
    p.add_argument("--serve-async-admission", type=int, default=1,
                   help="build admitted jobs' units on a worker thread (1) or inline (0)")
    p.add_argument("--ens-steps", type=int, default=200)
    p.add_argument("--ens-members", type=int, default=512)
    p.add_argument("--bh-steps", type=int, default=1000)
    p.add_argument("--bh-e2e-steps", type=int, default=5)
    p.add_argument("--bh-default-steps", type=int, default=3,
                   help="pipeline steps of the drop-in default astro2 (leaf 1, exact traversal) "
                        "through the plugin on host arrays, per theta")
    p.add_argument("--bh-sample", type=int, default=16384,
                   help="bodies whose accelerations are checked against the f64 reference law")
    p.add_argument("--sym-pairs-limit", type=int, default=0,
                   help="slot bytes up to which the each-pair-once plan runs one block per tile "
                        "pair (0: the library's 4 GiB; 1: thread-block clusters at any size)")
    p.add_argument("--bodies", type=int, default=N_CUBE,
                   help="cube bodies (profiling of smaller cases; the reported workload is "
                        "the default 1,048,576)")
    return p.parse_args()


# ---------------------------------------------------------------------------
# distributed plumbing (replicas only)
# ---------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            backend = "nccl" if _cuda_ok() else "gloo"
            dist.init_process_group(backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        return self._reduce(v, "max")

    def sum(self, v: float) -> float:
        return self._reduce(v, "sum")

    def _reduce(self, v, op):
        if not self.pg:
            return v
        import torch
        dev = torch.device("cuda", self.local) if _cuda_ok() else torch.device("cpu")
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX if op == "max" else self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def _cuda_ok() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except FileNotFoundError:
            self.proc = None

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        rows = []
        for ln in out.strip().splitlines():
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append({"sm": float(parts[1]), "max": float(parts[2]),
                             "power": float(parts[3]) if parts[3] not in ("[N/A]", "") else 0.0,
                             "hw": parts[5], "hwt": parts[6], "swt": parts[7], "cap": parts[8]})
            except ValueError:
                continue
        if not rows:
            return None
        sm_max = max(r["max"] for r in rows)
        loaded = [r for r in rows if r["power"] > 200.0] or rows
        reasons = set()
        for r in rows:
            for key, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"),
                              ("swt", "sw_thermal_slowdown"), ("cap", "sw_power_cap")):
                if r[key].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r["sm"] for r in loaded), "sm_max_mhz": sm_max,
                "samples": len(rows), "reasons": sorted(reasons)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            pass
    return {}


# ---------------------------------------------------------------------------
# CPU baseline: the C restatement on a bounded sample
# ---------------------------------------------------------------------------
def _sample_rows(n: int, k: int, seed: int) -> np.ndarray:
    return np.sort(np.random.default_rng(seed).choice(n, k, replace=False))


def cpu_rows_per_second(state, threads: int, probe_s: float = 0.3) -> float:
    """Rows (bodies x all their partners) of the f64 simple_astro restatement
    one call on `threads` threads finishes per second, from growing probes."""
    import oracle
    n = len(state)
    k = max(8, threads)
    while True:
        idx = _sample_rows(n, min(n, k), 99)
        t0 = time.perf_counter()
        oracle.simple_astro_sample(state, E, idx, threads=threads)
        dt = time.perf_counter() - t0
        if dt > probe_s or k >= n:
            return len(idx) / max(dt, 1e-9)
        k *= 4


def cpu_sample_step(state, threads: int, rows: int, seed: int) -> dict:
    """One bounded CPU step: the reference's simple_astro accelerations
    (f64 C restatement, transformers.rs:219-244) of `rows` bodies against
    all n-1 partners, on `threads` threads.  Returns its seconds and pairs."""
    import oracle
    n = len(state)
    idx = _sample_rows(n, rows, seed)
    t0 = time.perf_counter()
    oracle.simple_astro_sample(state, E, idx, threads=threads)
    dt = time.perf_counter() - t0
    return {"seconds": dt, "pairs": len(idx) * (n - 1), "rows": len(idx)}


def cpu_sample_rate(state, threads: int, target_s: float) -> dict:
    """The CPU baseline of our arm: one sample of about target_s seconds."""
    n = len(state)
    rows = int(min(n, max(threads, cpu_rows_per_second(state, threads) * target_s)))
    r = cpu_sample_step(state, threads, rows, 123)
    return {"value": r["pairs"] / r["seconds"] / 1e9, "unit": "Gpair-interactions/s",
            "cores": threads, "seconds": r["seconds"],
            "sample": f"{rows} of the {n} bodies x their {n - 1} partners, {r['seconds']:.1f} s "
                      f"(f64 C restatement of simple_astro, transformers.rs:219-244, "
                      f"{threads} thread{'s' if threads > 1 else ''})"}


def bench_config(bodies: int, gpus: int) -> dict:
    """The workload both arms report (our arm's plan details are kept outside)."""
    return {"workload": WORKLOAD, "bodies": bodies + 4, "pairs_per_step": (bodies + 4) * (bodies + 3),
            "parallelism": f"replicas x{gpus}" if gpus > 1 else "single GPU",
            "l2": "flushed between timed steps (256 MiB write, outside the events)"}


def workload_state(bodies: int):
    from physim_gb300 import ics  # numpy only: the CUDA library stays unloaded
    return ics.workload_large(bodies)


def run_reference(args, dist: Dist):
    """The reference algorithm on the host cores: each step is a bounded
    sample of one full simple_astro step (a fixed number of bodies against
    all their partners), timed as it runs; value = sampled pairs / seconds."""
    if dist.rank != 0:
        return
    import oracle
    state = workload_state(args.bodies)
    n = len(state)
    threads = oracle.load().oracle_max_threads()
    per_step_s = max(0.5, args.cpu_seconds / 4.0)
    rows = int(min(n, max(threads, cpu_rows_per_second(state, threads) * per_step_s)))
    for w in range(args.warmup):
        cpu_sample_step(state, threads, max(threads, rows // 4), 1000 + w)
    steps = [cpu_sample_step(state, threads, rows, 2000 + k) for k in range(args.steps)]
    seconds = sum(r["seconds"] for r in steps)
    pairs = sum(r["pairs"] for r in steps)
    value = pairs / seconds / 1e9
    single = cpu_sample_rate(state, 1, max(1.0, args.cpu_seconds / 4.0))
    sample = (f"each step: {rows} of the {n} bodies x their {n - 1} partners "
              f"({rows / n:.2%} of one full step's {n * (n - 1):.4g} pairs), "
              f"{args.steps} steps in {seconds:.1f} s")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Gpair-interactions/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": seconds / max(args.steps, 1) * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(args.bodies, args.gpus),
        "implementation": "C restatement of physim's simple_astro (oracle/, f64, OpenMP over "
                          "bodies); the Rust reference needs cargo, absent here",
        "sampling": {"rows_per_step": rows, "total_rows": n, "partners_per_row": n - 1,
                     "seconds_timed": seconds, "full_step_seconds_estimate":
                         n * (n - 1) / (value * 1e9)},
        "cpu_baseline": {"value": value, "unit": "Gpair-interactions/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "single_thread": {"value": single["value"], "unit": "Gpair-interactions/s", "cores": 1,
                          "sample": single["sample"],
                          "note": "physim's transform runs on one thread"},
        "e2e": {"value": value, "unit": "Gpair-interactions/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def _device_context(dist: Dist):
    import torch
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    device = dist.local
    torch.cuda.set_device(device)
    props = torch.cuda.get_device_properties(device)
    return device, props.multi_processor_count


def host_array_steps(pg, element, props, state, steps, device, mode):
    """Wall-clock seconds of `steps` plugin pipeline steps on host Entity
    arrays with host access `mode`, the transfers inside the timed region;
    returns (seconds, the mode the calls used).  Each step is physim's
    pipeline step (pipeline.rs:137-173, verlet.rs:85-106): fresh zeroed
    accelerations, the element's transform into them, the verlet update into
    the reused new_state array, which becomes the next state."""
    pg.set_host_access(mode)
    try:
        used = pg.host_access(device)
        el = pg.TransformElementHandler(element, props)
        verlet = pg.GpuVerlet(device)
        cur = state.copy()
        nxt = np.empty_like(cur)
        # one untimed pipeline step first: the element's and the integrator's
        # device buffers, module loads and the integrator's initial (Taylor)
        # step, so the timed steps are the regular ones
        acc = pg.accelerations(len(cur))
        el.transform(cur, acc)
        verlet.integrate(cur, acc, DT, out=nxt)
        cur, nxt = nxt, cur
        t0 = time.perf_counter()
        for _ in range(steps):
            acc = np.zeros(len(cur), dtype=pg.ACCELERATION)
            el.transform(cur, acc)
            verlet.integrate(cur, acc, DT, out=nxt)
            cur, nxt = nxt, cur
        seconds = time.perf_counter() - t0
        el.destroy()
        verlet.close()
    finally:
        pg.set_host_access("auto")
    return seconds, used


def _timed_steps(sim, stream, steps: int, flush, pair=False):
    """Per-step CUDA-event times on the simulation's stream, L2 flushed between
    steps outside the events.  Returns (step ms, gravity-kernel ms) and, with
    `pair`, the pair kernel's ms as a third list."""
    import torch
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    grav, pairs = [], []
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            starts[k].record(stream)
            sim.step(1)
            ends[k].record(stream)
        grav.append(sim.last_step_ms()[0])
        if pair:
            pairs.append(sim.last_pair_ms())
    torch.cuda.synchronize()
    times = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    return (times, grav, pairs) if pair else (times, grav)


def measure_direct(args, dist: Dist, device: int, sms: int, peaks: dict) -> dict:
    import torch

    import physim_gb300 as pg
    state = workload_state(args.bodies)
    n = len(state)
    pairs_step = n * (n - 1)  # no fixed bodies in this workload
    stream = torch.cuda.Stream(device=device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    sim = pg.Simulation(state, pg.SimConfig(gravity="simple_astro", e=E, dt=DT, device=device,
                                            stream=stream.cuda_stream))
    plan = sim.autotune()
    sim.set_profiling(True)
    with torch.cuda.stream(stream):
        sim.step(args.warmup)
    sim.synchronize()
    clocks = Clocks(device)
    dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_wall = time.perf_counter()
    step_ms, grav_ms, pair_ms = _timed_steps(sim, stream, args.steps, flush, pair=True)
    wall = time.perf_counter() - t_wall
    dist.barrier()
    clk = clocks.stop()
    total_ms = dist.max(sum(step_ms))
    all_pairs = dist.sum(float(pairs_step * args.steps))
    launches = sim.launches_per_step * args.steps
    sim.close()

    # the other each-pair-once schedule at this size, for the record: one block
    # per tile pair (faster, but one [3][n] f32 slot per tile: 12.9 GB at 1M
    # bodies), same state, same steps
    alt = None
    if plan.get("symmetric") and args.bodies == N_CUBE and not args.sym_pairs_limit:
        slot_bytes = 12 * plan["tiles"] * n
        pg.set_symmetric_pairs_limit(slot_bytes)
        try:
            sim = pg.Simulation(state, pg.SimConfig(gravity="simple_astro", e=E, dt=DT,
                                                    device=device, stream=stream.cuda_stream))
            sim.set_plan(symmetric=True)
            sim.set_profiling(True)
            with torch.cuda.stream(stream):
                sim.step(args.warmup)
            sim.synchronize()
            alt_ms, _, alt_pair = _timed_steps(sim, stream, args.steps, flush, pair=True)
            sim.close()
            alt = {"value": dist.sum(float(pairs_step * args.steps)) / (dist.max(sum(alt_ms)) / 1e3)
                   / 1e9, "unit": "Gpair-interactions/s",
                   "ms_per_step": dist.max(sum(alt_ms)) / args.steps,
                   "kernel_ms": statistics.mean(alt_pair), "slot_gb": slot_bytes / 1e9,
                   "schedule": "one block per pair of 1,024-body tiles, one slot per tile "
                               "(physim_gpu_set_symmetric_pairs_limit above its slot bytes)"}
        finally:
            pg.set_symmetric_pairs_limit(0)

    kern_ms = statistics.mean(pair_ms)
    if plan.get("symmetric"):
        # each unordered pair evaluated once: 27 flop (FFMA = 2) per pair
        kernel, flop_note = "direct_sym_kernel", FLOP_PER_SYM_PAIR
        flops_step = FLOP_PER_SYM_PAIR * pairs_step / 2
    else:
        kernel, flop_note = "direct_forces_kernel", FLOP_PER_PAIR
        flops_step = FLOP_PER_PAIR * pairs_step
    achieved = flops_step / (kern_ms / 1e3) / 1e12
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    peak = sms * FP32_LANES_PER_SM * 2 * sm_max * 1e6 / 1e12
    # DRAM bytes per launch from a committed ncu capture of a smaller case,
    # scaled to this workload (not measured in this run)
    traffic, traffic_source = None, None
    tfile = ROOT / "profiles" / "direct_forces_traffic.json"
    if tfile.exists() and args.bodies == N_CUBE:
        try:
            rec = json.loads(tfile.read_text()).get(kernel, {})
            traffic = rec.get("bytes_per_launch")
            traffic_source = "committed capture, not this run: " + rec.get("basis", "")
        except (ValueError, AttributeError):
            traffic = None
    out = {"value": all_pairs / (total_ms / 1e3) / 1e9, "ms_per_step": total_ms / args.steps,
           "bodies": n, "pairs_per_step": pairs_step, "wall_s": wall, "gpu_launches": launches,
           "plan": plan, "tile_pair_schedule": alt,
           "roofline": {"bound": "fp32", "kernel": kernel, "achieved": achieved,
                        "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                        "traffic": traffic, "traffic_source": traffic_source,
                        "peak_basis": f"{sms} SMs x {FP32_LANES_PER_SM} FP32 lanes x 2 x "
                                      f"{sm_max:.0f} MHz (max SM clock, measured-peaks file)",
                        "flop_per_pair": flop_note,
                        "pairs_per_launch": pairs_step // 2 if plan.get("symmetric")
                        else pairs_step,
                        "kernel_ms": kern_ms,
                        "reduce_ms": statistics.mean(grav_ms) - kern_ms}}
    if clk:
        out["clocks"] = clk
        if clk.get("sm_mhz"):
            out["roofline"]["frac_at_observed_clock"] = achieved / (
                sms * FP32_LANES_PER_SM * 2 * clk["sm_mhz"] * 1e6 / 1e12)

    if not args.skip_e2e:
        e2e_steps = args.e2e_steps or max(3, min(args.steps, 5))
        props = {"e": E, "device": device}
        runs = {m: host_array_steps(pg, "simple_astro", props, state, e2e_steps, device, m)
                for m in ("copy", "auto")}
        rate = {m: dist.sum(float(pairs_step * e2e_steps)) / dist.max(t) / 1e9
                for m, (t, _) in runs.items()}
        out["e2e"] = {"value": rate["auto"], "unit": "Gpair-interactions/s",
                      "h2d_bytes_per_step": n * (80 + 24) + n * (80 + 24),
                      "d2h_bytes_per_step": n * 24 + n * 80, "steps": e2e_steps,
                      "transfer": runs["auto"][1], "value_with_copies": rate["copy"],
                      "path": "simple_astro_transform + physim_gpu_verlet_integrate on host "
                              "Entity arrays (pipeline.rs:137-173)"}
    if dist.rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_sample_rate(state, 1, args.cpu_seconds)
        cpu.pop("seconds", None)
        cpu["kind"] = "port"
        out["cpu_baseline"] = cpu
    return out


# Algorithmic HBM bytes per body per Barnes-Hut step (f64 state, f32 bodies,
# 63-bit keys, 32-bit body indices, 8 radix passes), by kernel:
BH_BYTES_PER_BODY = {
    "extent": 24,                 # read x, y, z (f64)
    "keys": 24 + 12,              # read x, y, z; write key + index
    "sort": 8 * (8 + 12 + 12),    # per pass: histogram read, scatter read + write
    "gather": 4 + 16 + 32 + 16 + 24 + 8,  # order, f32 body, f64 x,y,z,m -> sorted copies
    "moments": 32 + 32 + 32,      # partial sums read, scan read + prefix write
    "traversal": 16 + 4 + 24,     # own body, order, acceleration partial
    "verlet": 24 + 8 + 1 + 72 + 16 + 72 + 16,  # partial, m, fixed, state in, body4, state out
}


def cpu_bh_step_time(state, theta: float, target_s: float) -> dict:
    """The reference astro2 restated (single thread): full tree build plus the
    traversal/force of a sample of bodies, scaled to all bodies."""
    import oracle
    n = len(state)
    rng = np.random.default_rng(11)
    k = 64
    t0 = time.perf_counter()
    oracle.barnes_hut(state, theta, E, nchild=8, idx=np.array([0]), threads=1)
    t_build = time.perf_counter() - t0  # build + one body
    while True:
        idx = rng.choice(n, k, replace=False)
        t0 = time.perf_counter()
        oracle.barnes_hut(state, theta, E, nchild=8, idx=idx, threads=1)
        t = time.perf_counter() - t0
        if t - t_build > target_s / 2 or k >= n:
            break
        k = min(n, k * 4)
    per_body = max(t - t_build, 1e-9) / k
    step_s = t_build + per_body * n
    return {"value": 1.0 / step_s, "unit": "steps/s", "cores": 1, "kind": "port",
            "sample": f"astro2 restatement (transformers.rs:122-160), theta {theta}: tree build "
                      f"of all {n} bodies ({t_build:.2f} s) + traversal/force of {k} bodies, "
                      f"scaled to {n} bodies"}


def measure_bh(args, dist: Dist, device: int, sms: int, peaks: dict) -> dict:
    import torch

    import physim_gb300 as pg
    from physim_gb300 import ics

    state = ics.workload_large(args.bodies)
    n = len(state)
    stream = torch.cuda.Stream(device=device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    results = {}
    # accuracy sample: RMS relative error of the initial accelerations against
    # the reference law in f64 (physim_gpu_sim_accelerations_f64) on 16,384 bodies
    sample = np.sort(np.random.default_rng(5).choice(n, min(n, args.bh_sample), replace=False))
    exact = None
    runs = [("0.5", 0.5, args.bh_steps, {}), ("1.0", 1.0, args.bh_steps, {}),
            ("1.5", 1.5, args.bh_steps, {}),
            ("0.5 quadrupole com_theta 0.6", 0.5, max(args.bh_steps // 4, 10),
             {"quadrupole": True, "com_theta": 0.6})]
    for name, theta, steps, extra in runs:
        sim = pg.Simulation(state, pg.SimConfig(gravity="astro2", theta=theta, e=E, dt=DT,
                                                leaf_size=16, traversal="warp", device=device,
                                                stream=stream.cuda_stream, **extra))
        err = None
        if exact is None:  # every run starts from the same state
            ex = sim.accelerations_f64(sample)
            exact = np.stack([ex["x"], ex["y"], ex["z"]], 1)
        a = sim.accelerations()[sample]
        got = np.stack([a["x"], a["y"], a["z"]], 1)
        rel = np.linalg.norm(got - exact, axis=1) / np.linalg.norm(exact, axis=1)
        err = {"rms_rel": float(np.sqrt(np.mean(rel ** 2))), "max_rel": float(rel.max()),
               "sample_bodies": len(sample), "reference": "physim_gpu_sim_accelerations_f64"}
        sim.set_profiling(True)
        with torch.cuda.stream(stream):
            sim.step(max(args.warmup, 3))
        sim.synchronize()
        dist.barrier()
        clocks = Clocks(device)
        clocks.start()
        step_ms, grav_ms = _timed_steps(sim, stream, steps, flush)
        clk = clocks.stop()
        total = dist.max(sum(step_ms))
        st = sim.bh_stats()
        results[name] = {"steps_per_s": dist.sum(float(steps)) / (total / 1e3),
                         "ms_per_step": total / steps, "steps": steps,
                         "gravity_ms": statistics.mean(grav_ms),
                         "traversal_ms_last_step": st["traversal_ms"],
                         "interactions_per_step": st["interactions"],
                         "node_visits_per_step": st["node_visits"],
                         "gpu_launches": sim.launches_per_step * steps,
                         "acc_error_vs_f64": err, "clocks": clk}
        sim.close()
        if not extra:
            # the same steps as one sim.step(steps) call, as a simulation runs
            # them: a fresh simulation from the same state, the same warm-up,
            # one L2 flush before the timed region and none between steps (the
            # step's working set, ~250 MB at 1M bodies, exceeds the 129 MB L2)
            sim = pg.Simulation(state, pg.SimConfig(gravity="astro2", theta=theta, e=E, dt=DT,
                                                    leaf_size=16, traversal="warp",
                                                    device=device, stream=stream.cuda_stream))
            with torch.cuda.stream(stream):
                sim.step(max(args.warmup, 3))
            sim.synchronize()
            dist.barrier()
            e0, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
            with torch.cuda.stream(stream):
                flush.zero_()
                e0.record(stream)
                sim.step(steps)
                e1.record(stream)
            torch.cuda.synchronize()
            b2b = dist.max(e0.elapsed_time(e1))
            results[name]["back_to_back"] = {
                "steps_per_s": dist.sum(float(steps)) / (b2b / 1e3), "ms_per_step": b2b / steps,
                "steps": steps, "path": "one physim_gpu_sim_step(steps) call, CUDA events on the "
                                        "simulation's stream, no L2 flush between steps"}
            sim.close()
    main = results["0.5"]
    bytes_step = sum(BH_BYTES_PER_BODY.values()) * n
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    achieved = bytes_step / (main["ms_per_step"] / 1e3) / 1e9
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    fp32_peak = sms * FP32_LANES_PER_SM * 2 * sm_max * 1e6 / 1e12
    trav_ms = main["traversal_ms_last_step"]
    trav_tflops = (FLOP_PER_PAIR * main["interactions_per_step"] / (trav_ms / 1e3) / 1e12
                   if trav_ms and trav_ms > 0 else None)
    out = {"metric": "BH steps/s at N=1M (astro2, theta 0.5, leaf 16, warp traversal)",
           "value": main["steps_per_s"], "unit": "steps/s", "ms_per_step": main["ms_per_step"],
           "bodies": n, "theta": results,
           "roofline": {"bound": "hbm", "kernel": "whole step", "achieved": achieved,
                        "peak": hbm, "unit": "GB/s", "frac": achieved / hbm, "traffic": None,
                        "algorithmic_bytes_per_body": BH_BYTES_PER_BODY,
                        "note": "interaction-list node reads (L2-resident tree) excluded",
                        "frac_by_theta": {
                            k: bytes_step / (v["ms_per_step"] / 1e3) / 1e9 / hbm
                            for k, v in results.items() if "quadrupole" not in k}},
           "traversal_roofline": {"bound": "fp32", "kernel": "traverse_warp_kernel",
                                  "achieved": trav_tflops, "peak": fp32_peak, "unit": "TFLOP/s",
                                  "frac": trav_tflops / fp32_peak if trav_tflops else None,
                                  "flop_per_interaction": FLOP_PER_PAIR,
                                  "kernel_ms": trav_ms}}
    if not args.skip_e2e:
        props = {"theta": 0.5, "e": E, "leaf_size": 16, "traversal": "warp", "device": device}
        runs = {m: host_array_steps(pg, "astro2", props, state, args.bh_e2e_steps, device, m)
                for m in ("copy", "auto")}
        rate = {m: dist.sum(float(args.bh_e2e_steps)) / dist.max(t) for m, (t, _) in runs.items()}
        out["e2e"] = {"value": rate["auto"], "unit": "steps/s",
                      "h2d_bytes_per_step": n * (80 + 24) * 2, "d2h_bytes_per_step": n * 104,
                      "steps": args.bh_e2e_steps, "transfer": runs["auto"][1],
                      "value_with_copies": rate["copy"],
                      "path": "astro2_transform (leaf_size 16, warp) + physim_gpu_verlet_integrate "
                              "on host Entity arrays"}
        # what unchanged TOML runs: `astro2 theta=.. e=..` with no other
        # properties (leaf 1, exact traversal: the reference's interaction
        # lists, transformers.rs:162-180), e.g. energysink.toml:37-39
        out["e2e_default"] = {}
        for theta in (0.5, 1.0):
            t, used = host_array_steps(pg, "astro2", {"theta": theta, "e": E, "device": device},
                                       state, args.bh_default_steps, device, "auto")
            out["e2e_default"][str(theta)] = {
                "value": dist.sum(float(args.bh_default_steps)) / dist.max(t), "unit": "steps/s",
                "steps": args.bh_default_steps, "transfer": used,
                "path": f"astro2_transform {{theta: {theta}, e: {E}}} (leaf 1, exact traversal) "
                        "+ physim_gpu_verlet_integrate on host Entity arrays"}
    if dist.rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_bh_step_time(state, 0.5, args.cpu_seconds)
    return out


def ensemble_states(count: int = 512, seed: int = 3):
    """The batched uneven workload: N_k log-uniform in [256, 65536] (seed 3);
    even members a uniform cube U[-0.5,0.5]^3, odd members a Plummer sphere."""
    from physim_gb300 import ics
    sizes = ics.ensemble_sizes(count, seed=seed)
    states = []
    for k, n in enumerate(sizes):
        if k % 2 == 0:
            states.append(ics.cube_with_stars(int(n), seed=10_000 + k))
        else:
            states.append(ics.plummer(int(n), seed=20_000 + k, a=0.1))
    return states


def measure_ensemble(args, dist: Dist, device: int) -> dict:
    import torch

    import physim_gb300 as pg

    states = ensemble_states(args.ens_members)
    sizes = [len(s) for s in states]
    pairs = sum(n * (n - 1) for n in sizes)
    stream = torch.cuda.Stream(device=device)
    cfg = pg.SimConfig(gravity="simple_astro", e=E, dt=DT, device=device,
                       stream=stream.cuda_stream)
    ens = pg.Ensemble(states, cfg)
    t0 = time.perf_counter()
    plan = ens.autotune()
    tune_s = time.perf_counter() - t0
    with torch.cuda.stream(stream):
        ens.step(max(args.warmup, 3))
    ens.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist.barrier()
    with torch.cuda.stream(stream):
        a.record(stream)
        ens.step(args.ens_steps)
        b.record(stream)
    torch.cuda.synchronize()
    ens_ms = dist.max(a.elapsed_time(b))
    launches = ens.launches_per_step * args.ens_steps
    ens.close()

    def one_at_a_time(one_pair: bool) -> float:
        """The same members one at a time through the per-simulation path:
        its heuristic plans, or (one_pair) the plain one-pair kernels only
        (each ordered pair evaluated, no each-pair-once plan)."""
        if one_pair:
            pg.set_symmetric_cap(1)
        try:
            sims = [pg.Simulation(s, pg.SimConfig(gravity="simple_astro", e=E, dt=DT,
                                                  device=device)) for s in states]
        finally:
            pg.set_symmetric_cap(0)
        for sim in sims:
            sim.step(1)
            sim.synchronize()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for sim in sims:
            sim.step(args.ens_steps)
            sim.synchronize()
        sec = dist.max(time.perf_counter() - t0)
        for sim in sims:
            sim.close()
        return sec

    plain_s = one_at_a_time(False)
    one_pair_s = one_at_a_time(True)
    member_steps = len(states) * args.ens_steps
    ens_rate = dist.sum(float(member_steps)) / (ens_ms / 1e3)
    plain_rate = dist.sum(float(member_steps)) / plain_s
    one_pair_rate = dist.sum(float(member_steps)) / one_pair_s
    return {"metric": "aggregate member-steps/s, 512-member uneven ensemble (direct sum)",
            "value": ens_rate, "unit": "member-steps/s", "members": len(states),
            "bodies_total": int(sum(sizes)), "pairs_per_step": pairs,
            "steps": args.ens_steps, "ms_per_step": ens_ms / args.ens_steps,
            "gpair_per_s": pairs * args.ens_steps / (ens_ms / 1e3) / 1e9,
            "plan": plan, "autotune_s": tune_s, "gpu_launches": launches,
            "plain_one_at_a_time": {"value": plain_rate, "unit": "member-steps/s",
                                    "seconds": plain_s,
                                    "path": "physim_gpu_sim_step per member, members in turn, "
                                            "each with its heuristic plan (each pair once "
                                            "from 20,480 bodies)"},
            "plain_one_pair_kernels": {"value": one_pair_rate, "unit": "member-steps/s",
                                       "seconds": one_pair_s,
                                       "path": "the same, one-pair kernels only (every ordered "
                                               "pair evaluated)"},
            "speedup_vs_plain": ens_rate / plain_rate,
            "speedup_vs_plain_one_pair": ens_rate / one_pair_rate}


def _acc_errors(sim, idx) -> dict:
    """RMS / max relative acceleration error of the GPU forces of the
    simulation's current state against the reference law in f64
    (physim_gpu_sim_accelerations_f64) on the bodies idx."""
    exact = sim.accelerations_f64(idx)
    ex = np.stack([exact["x"], exact["y"], exact["z"]], 1)
    a = sim.accelerations()[idx]
    got = np.stack([a["x"], a["y"], a["z"]], 1)
    rel = np.linalg.norm(got - ex, axis=1) / np.linalg.norm(ex, axis=1)
    return {"rms": float(np.sqrt(np.mean(rel ** 2))), "max": float(rel.max())}


def measure_precision(args, dist: Dist, device: int) -> dict:
    """Precision study: 262,144-body Plummer sphere (a = 0.1, M = 1, seed 7,
    isotropic distribution-function velocities), e = 1e-3, dt = 1e-4.  Per
    variant (plain FP32 sums; compensated FP32 sums per j tile; each unordered
    pair once with TwoSum-added slot sums): RMS/max relative acceleration
    error against the reference law in f64 evaluated on the GPU
    (physim_gpu_sim_accelerations_f64) on a 1,024-body sample of the initial
    and of the final state, and the relative
    energy and momentum drift (f64 on the device) every steps/10 steps over
    --precision-steps steps."""
    import physim_gb300 as pg
    from physim_gb300 import ics

    n = args.precision_bodies
    steps = args.precision_steps
    state = ics.plummer(n, seed=7, a=0.1, total_mass=1.0)
    e, dt = 1e-3, 1e-4
    idx = np.sort(np.random.default_rng(7).choice(n, min(n, 1024), replace=False))
    every = max(1, steps // 10)
    # momentum scale: sum of |m v| of the initial state
    pscale = float(np.sum(state["mass"] * np.sqrt(state["vx"] ** 2 + state["vy"] ** 2 +
                                                  state["vz"] ** 2)))
    out = {"bodies": n, "e": e, "dt": dt, "steps": steps, "sample_bodies": len(idx),
           "potential": "V = -m_a m_b atan(sqrt(e)/r)/sqrt(e) (gradient = the reference force)",
           "variants": {}}
    variants = (("fp32_plain", False, None),
                ("fp32_compensated", True, {"symmetric": False, "block": 128, "ipt": 4,
                                            "splits": 4}),
                ("fp32_each_pair_once", True, {"symmetric": True}))
    chosen = set(filter(None, args.precision_variants.split(",")))
    for name, comp, plan in variants:
        if chosen and name not in chosen:
            continue
        sim = pg.Simulation(state, pg.SimConfig(gravity="simple_astro", e=e, dt=dt,
                                                compensated=comp, device=device))
        if plan:
            sim.set_plan(**plan)
        err0 = _acc_errors(sim, idx)
        d0 = sim.diagnostics(potential=True)
        p0 = np.array(d0["momentum"])
        series = []
        t0 = time.perf_counter()
        done = 0
        while done < steps:
            k = min(every, steps - done)
            sim.step(k)
            done += k
            d = sim.diagnostics(potential=True)
            series.append({"step": done,
                           "energy_drift": (d["energy"] - d0["energy"]) / abs(d0["energy"]),
                           "momentum_drift": float(np.linalg.norm(np.array(d["momentum"]) - p0))
                           / pscale})
        run_s = time.perf_counter() - t0
        err1 = _acc_errors(sim, idx)
        sim.close()
        out["variants"][name] = {
            "acc_rms_rel_error": err0["rms"], "acc_max_rel_error": err0["max"],
            "acc_rms_rel_error_final": err1["rms"], "acc_max_rel_error_final": err1["max"],
            "energy_start": d0["energy"], "kinetic_start": d0["kinetic"],
            "potential_start": d0["potential"],
            "max_abs_relative_energy_drift": max(abs(r["energy_drift"]) for r in series),
            "max_momentum_drift_over_sum_mv": max(r["momentum_drift"] for r in series),
            "series": series, "run_s": run_s}
    return out


def _serve_once(jobs, executor, until: float, **server_kw) -> dict:
    from physim_gb300.server import Server, latency_summary
    srv = Server(executor, hbm_budget=150 << 30, **server_kw)
    srv.submit(jobs)
    t0 = time.perf_counter()
    res = srv.run(until=until)
    wall = time.perf_counter() - t0
    unfinished = srv.unfinished()
    srv.close()
    lat = latency_summary(res)
    depth = srv.queue_depth
    return {"p50_s": lat.get("p50_s"), "p99_s": lat.get("p99_s"), "latency": lat,
            "completed": len(res), "unfinished_at_cutoff": unfinished,
            "failed": len(srv.failed), "rejected": len(srv.rejected),
            "steps_of_completed_jobs": srv.steps_done, "steps_executed": srv.steps_executed,
            "aggregate_steps_per_s": srv.steps_executed / wall, "wall_s": wall,
            "max_waiting": max((d[1] for d in depth), default=0),
            "max_running_units": srv.max_running,
            "max_hbm_in_use_gb": max((d[3] for d in depth), default=0) / 2**30,
            "queue_depth_samples": [(round(t, 2), w, r) for t, w, r, _ in depth[::16]]}


def measure_served(args, dist: Dist, device: int) -> dict:
    """The served mix: Poisson arrivals (50 jobs/s) of direct-sum and
    Barnes-Hut jobs with log-uniform N in [1,024, 2,097,152] and 100-5,000
    steps, admitted by a 150 GB HBM budget (the unit cap is set high enough
    that the budget is what binds) and run with continuous batching
    (shortest job first).  Arrivals for --serve-seconds (120 s), then up to
    --serve-drain seconds to finish; jobs still queued or running at the
    cut-off are reported as unfinished.  The same arrivals are then run one
    job at a time through the plain per-simulation path in the same
    admission order (and, with --serve-fifo-baseline, in arrival order) over
    the same window."""
    from physim_gb300.server import GpuExecutor, PlainExecutor, served_mix

    until = args.serve_seconds + args.serve_drain
    jobs = served_mix(rate=50.0, seconds=args.serve_seconds, seed=5)
    served = _serve_once(jobs, GpuExecutor(device=device, tick_ms=25.0, download=True), until,
                         admission=args.serve_admission, scheduling=args.serve_scheduling,
                         inflight_seconds=args.serve_inflight_ms / 1e3,
                         async_admission=bool(args.serve_async_admission),
                         max_units=args.serve_max_units,
                         queue_seconds=(args.serve_queue_ms / 1e3 if args.serve_queue_ms > 0
                                        else None))
    plain_same = _serve_once(served_mix(rate=50.0, seconds=args.serve_seconds, seed=5),
                             PlainExecutor(device=device, download=True), until, max_units=1,
                             max_batch=1, admission=args.serve_admission)
    plain_fifo = (_serve_once(served_mix(rate=50.0, seconds=args.serve_seconds, seed=5),
                              PlainExecutor(device=device, download=True), until, max_units=1,
                              max_batch=1, admission="fifo")
                  if args.serve_fifo_baseline and args.serve_admission != "fifo" else None)
    offered_direct = sum(j.n * j.n * j.steps for j in jobs if j.gravity == "simple_astro")
    rate = served["aggregate_steps_per_s"]
    out = {"metric": "served-mix job latency (arrival to final state on the host)",
           "admission": ("shortest job first (estimated device work)"
                         if args.serve_admission == "shortest" else "arrival order")
                        + f", HBM budget 150 GB, at most {args.serve_max_units} units (one "
                          "ensemble per admission round of direct-sum jobs, one simulation per "
                          "Barnes-Hut job, each on its own stream)"
                        + (", units built on a worker thread" if args.serve_async_admission
                           else ""),
           "scheduling": args.serve_scheduling
                         + (f" (at most {args.serve_queue_ms:.0f} ms of estimated device work "
                            "queued, units ticked least recently first)"
                            if args.serve_scheduling == "all" and args.serve_queue_ms > 0
                            else f" (in flight {args.serve_inflight_ms:.0f} ms)"
                            if args.serve_scheduling == "srpt" else ""),
           "jobs_arrived": len(jobs), "arrival_seconds": args.serve_seconds,
           "drain_seconds": args.serve_drain, "offered_direct_pairs": offered_direct}
    out.update(served)
    out["plain_one_at_a_time"] = {
        "same_order": plain_same, "order": args.serve_admission,
        "path": "each job alone as a device-resident simulation (direct or Barnes-Hut), "
                "100 ms ticks, admitted in the served run's order"}
    out["speedup_vs_plain_same_order"] = rate / max(plain_same["aggregate_steps_per_s"], 1e-9)
    out["p50_ratio_plain_over_served"] = ((plain_same["p50_s"] or 0.0) / served["p50_s"]
                                          if served.get("p50_s") else None)
    out["hbm_budget_gb"] = 150.0
    if plain_fifo is not None:
        out["plain_one_at_a_time"]["arrival_order"] = plain_fifo
        out["speedup_vs_plain_arrival_order"] = rate / max(
            plain_fifo["aggregate_steps_per_s"], 1e-9)
    out["note"] = ("offered load far exceeds one GPU (the direct-sum jobs alone are "
                   f"{offered_direct / 2.3e12:.0f} GPU-seconds at 2.3e12 pairs/s), so latency "
                   "is dominated by backlog and steps/s by which jobs run first")
    return out


def measure_tour(args, dist: Dist, device: int) -> dict:
    """Runs every kernel of the library at least once on small and mid-size
    states (profiling runs: `--only tour` under an ncu launch list shows each
    kernel's device time).  Returns the paths run."""
    import physim_gb300 as pg
    from physim_gb300 import ics, initialisers

    paths = []
    cube = ics.cube_with_stars(65536, seed=1, stars=ics.STARS_4)
    small = ics.cube_with_stars(4096, seed=2, stars=ics.STARS_2)
    # direct sums: each pair once + verlet; one-pair kernels with euler and rk4
    with pg.Simulation(cube, pg.SimConfig(gravity="simple_astro", e=E, dt=DT,
                                          device=device)) as sim:
        sim.step(2)
        sim.diagnostics(potential=True)
        sim.accelerations()
        sim.accelerations_f64(np.arange(64))
        sim.download()
    paths.append("simple_astro 65,536 each pair once + verlet, diagnostics, f64 sample")
    # the same sum in thread-block clusters (the schedule of large states)
    pg.set_symmetric_pairs_limit(1)
    try:
        with pg.Simulation(cube, pg.SimConfig(gravity="simple_astro", e=E, dt=DT,
                                              device=device)) as sim:
            sim.step(2)
    finally:
        pg.set_symmetric_pairs_limit(0)
    paths.append("simple_astro 65,536 each pair once in thread-block clusters")
    for integ in ("euler", "rk4"):
        with pg.Simulation(small, pg.SimConfig(gravity="simple_astro", e=E, dt=DT,
                                               integrator=integ, device=device)) as sim:
            sim.step(1)
    paths.append("simple_astro 4,098 one-pair kernels + euler, rk4")
    # Barnes-Hut: warp traversal (monopole, quadrupole), exact traversal, quadtree
    big = ics.workload_large(262_144)
    for cfg in (dict(gravity="astro2", theta=0.5, leaf_size=16, traversal="warp"),
                dict(gravity="astro2", theta=0.5, leaf_size=16, traversal="warp",
                     quadrupole=True, com_theta=0.6),
                dict(gravity="astro2", theta=0.5, leaf_size=1, traversal="exact"),
                dict(gravity="astro", theta=0.5, leaf_size=16, traversal="warp")):
        with pg.Simulation(big, pg.SimConfig(e=E, dt=DT, device=device, **cfg)) as sim:
            sim.step(2)
        paths.append(" ".join(f"{k}={v}" for k, v in cfg.items()))
    # the radix sort as one launch per pass (the form without cooperative launches)
    pg.lib.physim_gpu_set_sort_single_launch(0)
    try:
        with pg.Simulation(big, pg.SimConfig(gravity="astro2", theta=0.5, leaf_size=16,
                                             traversal="warp", e=E, dt=DT,
                                             device=device)) as sim:
            sim.step(1)
    finally:
        pg.lib.physim_gpu_set_sort_single_launch(1)
    paths.append("astro2 with the radix sort as one launch per pass")
    # host arrays: the plugin transform + verlet, in place and with copies
    try:
        for mode in ("direct", "copy"):
            if mode == "direct" and pg.host_access(device) != "direct":
                continue
            pg.set_host_access(mode)
            el = pg.TransformElementHandler("simple_astro", {"e": E, "device": device})
            acc = pg.accelerations(len(small))
            el.transform(small, acc)
            pg.GpuVerlet(device).integrate(small, acc, DT)
            el.destroy()
            paths.append(f"plugin simple_astro + verlet, host access {mode}")
    finally:
        pg.set_host_access("auto")
    for kind in ("euler", "rk4"):
        el = pg.TransformElementHandler("astro2", {"e": E, "theta": 0.5, "device": device})
        pg.GpuIntegrator(kind, device).integrate(small, lambda st, ac: el.transform(st, ac), DT)
        el.destroy()
    paths.append("host-array euler, rk4 with an astro2 acc_fn")
    # ensemble with members on both kinds of units
    members = [ics.plummer(n, seed=n, a=0.1) for n in (300, 2048, 9000, 20000)]
    with pg.Ensemble(members, pg.SimConfig(gravity="simple_astro", e=E, dt=DT,
                                           device=device)) as ens:
        ens.step(2)
        ens.download(0)
    paths.append("ensemble of 4 members (one-pair and each-pair-once units)")
    # device initialisers
    initialisers.cube({"n": 10_000, "seed": 3}, device)
    initialisers.plummer({"n": 10_000, "seed": 4}, device)
    paths.append("cube and plummer initialisers")
    return {"metric": "kernel tour", "value": len(paths), "unit": "paths", "paths": paths}


def bench_parts(only: str, world: int) -> list[str]:
    """The parts a run measures: --only's list, else every part on one GPU and,
    under torchrun (replicas), the headline direct sum and Barnes-Hut only -- the
    ensemble, the served mix and the precision study are single-GPU studies,
    measured in the N = 1 run."""
    if only:
        return only.split(",")
    if world == 1:
        return ["direct", "bh", "ensemble", "served", "precision"]
    return ["direct", "bh"]


def run_ours(args, dist: Dist):
    device, sms = _device_context(dist)
    if args.sym_pairs_limit:
        import physim_gb300 as pg
        pg.set_symmetric_pairs_limit(args.sym_pairs_limit)
    peaks = measured_peaks()
    parts = bench_parts(args.only, dist.world)
    direct = measure_direct(args, dist, device, sms, peaks) if "direct" in parts else None
    bh = measure_bh(args, dist, device, sms, peaks) if "bh" in parts else None
    ens = measure_ensemble(args, dist, device) if "ensemble" in parts else None
    served = measure_served(args, dist, device) if "served" in parts else None
    precision = measure_precision(args, dist, device) if "precision" in parts else None
    tour = measure_tour(args, dist, device) if "tour" in parts else None
    if dist.rank != 0:
        return
    if tour and not (direct or bh or ens or served or precision):
        print(json.dumps({**tour, "higher_is_better": True}), flush=True)
        return
    if precision and not (direct or bh or ens or served):
        print(json.dumps({"metric": "precision study (RMS relative acceleration error)",
                          "value": min(v["acc_rms_rel_error"]
                                       for v in precision["variants"].values()),
                          "unit": "relative", "higher_is_better": False,
                          "precision": precision}), flush=True)
        return
    if served and not (direct or bh or ens):
        print(json.dumps({"metric": served["metric"], "value": served["p50_s"], "unit": "s",
                          "higher_is_better": False, "served": served}), flush=True)
        return
    base = direct if direct else (bh if bh else ens)
    line = {
        "metric": METRIC if direct else base["metric"],
        "value": base["value"],
        "unit": "Gpair-interactions/s" if direct else base["unit"],
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": base["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 pairs, f64 integration", "data": "synthetic",
        "config": {"workload": WORKLOAD if direct else ("astro2 " + WORKLOAD if bh else
                                                        "512-member uneven ensemble"),
                   "bodies": base.get("bodies", base.get("bodies_total")),
                   "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "single GPU",
                   "l2": "flushed between timed steps (256 MiB write, outside the events)",
                   "compensated_sums": True},
    }
    if direct:
        line["config"] = bench_config(args.bodies, args.gpus)
        line["pair_kernel_plan"] = direct["plan"]
        line["compensated_sums"] = True
        for k in ("roofline", "e2e", "gpu_launches", "cpu_baseline", "clocks",
                  "tile_pair_schedule"):
            if k in direct:
                line[k] = direct[k]
    if served:
        line["served"] = served
    if precision:
        line["precision"] = precision
    if ens:
        line["ensemble"] = ens
        if not direct and not bh:
            line["metric"] = ens["metric"]
            line["unit"] = ens["unit"]
            line["gpu_launches"] = ens["gpu_launches"]
    if bh:
        line["bh"] = bh
        if not direct:
            for k in ("roofline", "e2e", "cpu_baseline"):
                if k in bh:
                    line[k] = bh[k]
            line["gpu_launches"] = bh["theta"]["0.5"]["gpu_launches"]
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
