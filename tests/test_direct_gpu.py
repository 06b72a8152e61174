"""simple_astro on the GPU against the oracle (astro/src/transformers.rs:219-244).

Tolerance: the pair arithmetic is FP32 with compensated per-body sums, the
oracle f64, so each body's acceleration must agree to a relative error
(|a_gpu - a_ref| / |a_ref|) of 1e-5; NaN, fixed and untouched entries must
agree exactly."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def _vec(acc):
    return np.stack([acc["x"], acc["y"], acc["z"]], axis=1)


def rel_err(got, want):
    g, w = _vec(got), _vec(want)
    return np.linalg.norm(g - w, axis=1) / np.maximum(np.linalg.norm(w, axis=1), 1e-300)


def run_plugin(state, e, prefill=None, name="simple_astro", props=None):
    import physim_gb300 as pg
    acc = pg.accelerations(len(state)) if prefill is None else prefill.copy()
    with pg.TransformElementHandler(name, {"e": e, **(props or {})}) as el:
        el.transform(state, acc)
    return acc


def test_smoke_entry():
    import __graft_entry__
    __graft_entry__.smoke()


@pytest.mark.parametrize("n", [1, 2, 3, 31, 257, 1000, 1025, 4098, 12345])
def test_plugin_matches_oracle(oracle_mod, n):
    from physim_gb300 import ics
    s = ics.cube_with_stars(max(n - 2, 0), seed=n, stars=ics.STARS_2[: min(n, 2)])
    assert len(s) == n
    if n > 5:
        s["fixed"][n // 3] = 1
    import physim_gb300 as pg
    acc0 = pg.accelerations(n)
    acc0["x"] = np.linspace(-1.0, 1.0, n)
    acc0["z"] = -0.0
    got = run_plugin(s, 0.01, acc0)
    want = oracle_mod.simple_astro(s, 0.01, acc0.copy())
    fixed = s["fixed"].astype(bool)
    assert _vec(got)[fixed].tobytes() == _vec(want)[fixed].tobytes()
    err = rel_err(got[~fixed], want[~fixed])
    assert np.all(err < RTOL), err.max()


def test_coincident_bodies_skip_each_other(oracle_mod):
    """transformers.rs:230: equal centres contribute nothing."""
    from physim_gb300 import ics
    s = ics.cube_with_stars(300, seed=4)
    for k in range(10):
        s[k]["x"], s[k]["y"], s[k]["z"] = 0.125, -0.25, 0.375
    got = run_plugin(s, 0.05)
    want = oracle_mod.simple_astro(s, 0.05)
    assert np.all(rel_err(got, want) < RTOL)


def test_massless_body_is_nan(oracle_mod):
    from physim_gb300 import ics
    s = ics.cube_with_stars(100, seed=5)
    s["mass"][[3, 40]] = 0.0
    got = run_plugin(s, 0.01)
    want = oracle_mod.simple_astro(s, 0.01)
    assert np.array_equal(np.isnan(_vec(got)), np.isnan(_vec(want)))
    ok = ~np.isnan(_vec(want)).any(axis=1)
    assert np.all(rel_err(got[ok], want[ok]) < RTOL)


def test_zero_easing(oracle_mod):
    from physim_gb300 import ics
    s = ics.cube_with_stars(500, seed=6)
    got = run_plugin(s, 0.0)
    want = oracle_mod.simple_astro(s, 0.0)
    assert np.all(rel_err(got, want) < 1e-4)


def test_negative_easing_is_absolute(oracle_mod):
    from physim_gb300 import ics
    s = ics.cube_with_stars(200, seed=7)
    got = run_plugin(s, -0.3)
    want = oracle_mod.simple_astro(s, 0.3)
    assert np.all(rel_err(got, want) < RTOL)


def test_longer_acceleration_buffer_untouched_tail(oracle_mod):
    import physim_gb300 as pg
    from physim_gb300 import ics
    s = ics.cube_with_stars(64, seed=8)
    acc = pg.accelerations(70)
    acc["y"][64:] = 3.0
    with pg.TransformElementHandler("simple_astro", {"e": 0.01}) as el:
        el.api.transform(el.instance, s.ctypes.data, 64, acc.ctypes.data, 70)
    assert np.all(acc["y"][64:] == 3.0)
    want = oracle_mod.simple_astro(s, 0.01)
    assert np.all(rel_err(acc[:64], want) < RTOL)


def test_empty_state_is_noop():
    import physim_gb300 as pg
    acc = pg.accelerations(0)
    run_plugin(pg.entities(0), 0.01, acc)


def test_repeated_calls_and_resizing(oracle_mod):
    """The element keeps device buffers between calls and grows them."""
    import physim_gb300 as pg
    from physim_gb300 import ics
    with pg.TransformElementHandler("simple_astro", {"e": 0.02}) as el:
        for n in (100, 3000, 50, 3000):
            s = ics.cube_with_stars(n, seed=n + 1)
            acc = pg.accelerations(n)
            el.transform(s, acc)
            assert np.all(rel_err(acc, oracle_mod.simple_astro(s, 0.02)) < RTOL)


def test_sim_accelerations_match_plugin():
    import physim_gb300 as pg
    from physim_gb300 import ics
    s = ics.cube_with_stars(5000, seed=12, stars=ics.STARS_4)
    plug = run_plugin(s, 0.01)
    with pg.Simulation(s, pg.SimConfig(gravity="simple_astro", e=0.01)) as sim:
        a = sim.accelerations()
    assert np.all(rel_err(a, plug) < 1e-12)


@pytest.mark.parametrize("compensated,tol", [(True, 1e-6), (False, 1e-4)])
def test_precision_vs_fp64(oracle_mod, compensated, tol):
    """RMS relative error against the f64 direct sum on a sample of bodies."""
    import physim_gb300 as pg
    from physim_gb300 import ics
    s = ics.plummer(65536, seed=7, a=0.1)
    idx = np.random.default_rng(0).choice(len(s), 256, replace=False)
    want = oracle_mod.simple_astro_sample(s, 1e-3, idx)
    with pg.Simulation(s, pg.SimConfig(gravity="simple_astro", e=1e-3,
                                       compensated=compensated)) as sim:
        got = sim.accelerations()[idx]
    rms = float(np.sqrt(np.mean(rel_err(got, want) ** 2)))
    assert rms < tol, rms


def test_full_size_workload_sample_and_momentum(oracle_mod):
    """1,048,580 bodies: a 128-body sample against the f64 oracle (RMS <= 1e-5)
    and net force sum_i m_i a_i ~ 0 (Newton's third law of the pair law)."""
    import physim_gb300 as pg
    from physim_gb300 import ics
    s = ics.workload_large()
    with pg.Simulation(s, pg.SimConfig(gravity="simple_astro", e=0.01)) as sim:
        a = sim.accelerations()
    idx = np.concatenate([np.arange(len(s) - 4, len(s)),
                          np.random.default_rng(1).choice(len(s) - 4, 124, replace=False)])
    want = oracle_mod.simple_astro_sample(s, 0.01, idx)
    err = rel_err(a[idx], want)
    assert float(np.sqrt(np.mean(err ** 2))) < 1e-5, err.max()
    f = _vec(a) * s["mass"][:, None]
    scale = np.abs(f).sum(axis=0)
    assert np.all(np.abs(f.sum(axis=0)) < 1e-6 * scale)
