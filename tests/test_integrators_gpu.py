"""The euler and rk4 integrators on the GPU (integrators/src/euler.rs:17-49,
integrators/src/rk4.rs:24-178), and verlet through the same acc_fn-shaped
entry point.

Given the same acc_fn, the host-array integrators are bit-identical to the
oracle: their stage states and updates are f64 in the reference's operation
order, and acc_fn runs on the host for exactly those stage states.  The
device-resident simulations evaluate gravity with FP32 pair forces, so whole
trajectories are compared within the tolerance of the verlet tests: relative
L2 1e-5 of positions (against the distance travelled) and velocities."""
from __future__ import annotations

import numpy as np
import pytest

from test_verlet_gpu import FIELDS, _same, _trajectory_check

pytestmark = pytest.mark.gpu


def _state(n=800, seed=31):
    from physim_gb300 import ics
    s = ics.cube_with_stars(n, seed=seed, stars=ics.STARS_2)
    s["fixed"][3] = 1
    s["vx"][3] = 0.25  # a fixed body with a velocity: euler drifts it, rk4 pins it
    return s


@pytest.mark.parametrize("kind", ["euler", "rk4", "verlet"])
def test_host_integrators_bit_identical(oracle_mod, kind):
    import physim_gb300 as pg
    s = _state()
    calls = []

    def acc_fn(state, acc):
        calls.append(state.copy())
        oracle_mod.simple_astro(state, 0.01, acc)

    it = pg.GpuIntegrator(kind)
    dt = 1e-4
    got = s
    for _ in range(3):
        got = it.integrate(got, acc_fn, dt)
    it.close()
    assert len(calls) == (12 if kind == "rk4" else 3)
    want = s
    ov = oracle_mod.Verlet()
    for _ in range(3):
        if kind == "euler":
            acc = oracle_mod.simple_astro(want, 0.01)
            want = oracle_mod.euler_step(want, acc, dt)
        elif kind == "rk4":
            want = oracle_mod.rk4_step(want, lambda st, ac: oracle_mod.simple_astro(st, 0.01, ac),
                                       dt)
        else:
            acc = oracle_mod.simple_astro(want, 0.01)
            want = ov.step(want, acc, dt)
    _same(got, want)
    if kind == "euler":
        assert got["x"][3] != s["x"][3]  # euler.rs ignores `fixed`
    if kind == "rk4":
        assert got["x"][3] == s["x"][3] and got["vx"][3] == 0.0  # rk4.rs:165-171


def test_rk4_stage_states_handed_to_acc_fn(oracle_mod):
    """acc_fn sees the entity state, then state + k1/2, state + k2/2 and
    state + k3 (rk4.rs:50-62, 76-87, 101-112), with zeroed accelerations."""
    import physim_gb300 as pg
    s = _state(200, seed=5)
    seen = []

    def rec(state, acc):
        assert not np.any(acc["x"]) and not np.any(acc["y"]) and not np.any(acc["z"])
        seen.append(state.copy())
        oracle_mod.simple_astro(state, 0.01, acc)

    with_gpu = pg.GpuIntegrator("rk4")
    with_gpu.integrate(s, rec, 1e-3)
    with_gpu.close()
    ref = []

    def rec_ref(state, acc):
        ref.append(state.copy())
        oracle_mod.simple_astro(state, 0.01, acc)

    oracle_mod.rk4_step(s, rec_ref, 1e-3)
    assert len(seen) == len(ref) == 4
    for a, b in zip(seen, ref):
        _same(a, b)


@pytest.mark.parametrize("integrator", ["euler", "rk4"])
@pytest.mark.parametrize("gravity", ["simple_astro", "astro2"])
def test_device_resident_integrators(oracle_mod, integrator, gravity):
    """Device-resident simulation (state in HBM, gravity on the GPU) against
    the oracle pipeline with the same integrator: 4,098-body cube + stars,
    e = 0.01; simple_astro 40 steps of dt = 1e-5; astro2 (the reference's
    leaf-1 tree and per-body interaction lists, theta 0.5) 5 steps of
    dt = 1e-6, so that no body's interaction list changes between the two
    runs (a flipped opening decision is a discrete jump in its force)."""
    import physim_gb300 as pg
    from physim_gb300 import ics
    s = ics.workload_direct_small()
    s["fixed"][10] = 1
    steps, dt = (40, 1e-5) if gravity == "simple_astro" else (5, 1e-6)
    cfg = pg.SimConfig(gravity=gravity, e=0.01, dt=dt, theta=0.5, integrator=integrator)
    with pg.Simulation(s, cfg) as sim:
        sim.step(steps)
        got = sim.download()
        lps = sim.launches_per_step
    want = oracle_mod.run_pipeline(s, gravity, steps, dt, 0.01, theta=0.5,
                                   integrator=integrator)
    _trajectory_check(got, want, s)
    if integrator == "rk4":
        assert got["x"][10] == s["x"][10] and got["vx"][10] == 0.0
        assert lps % 4 == 0


def test_plugin_pipeline_rk4(oracle_mod):
    """pipeline.rs:137-173 with the simple_astro plugin transform as
    transform_fn and the rk4 integrator over host arrays, 5 steps."""
    import physim_gb300 as pg
    from physim_gb300 import ics
    s = ics.cube_with_stars(1500, seed=23, stars=ics.STARS_2)
    s["fixed"][1] = 1
    el = pg.TransformElementHandler("simple_astro", {"e": 0.01})
    it = pg.GpuIntegrator("rk4")
    got = pg.Pipeline([el], it, 1e-5).run(s, 5)
    el.destroy()
    it.close()
    want = oracle_mod.run_pipeline(s, "simple_astro", 5, 1e-5, 0.01, integrator="rk4")
    _trajectory_check(got, want, s)


def test_integrator_rejects_unknown_kind():
    import ctypes as C

    import physim_gb300 as pg
    h = C.c_void_p()
    assert pg.lib.physim_gpu_integrator_create(7, 0, C.byref(h)) == 1
    cfg = pg.SimConfig(gravity="simple_astro").to_c()
    cfg.integrator = 9
    assert pg.lib.physim_gpu_sim_create(C.byref(cfg), 10, C.byref(h)) == 1
    assert FIELDS
