"""physim_gpu_sim_accelerations_f64, the f64 accuracy reference on the GPU,
against the oracle (astro/src/lib.rs:84-113, transformers.rs:219-244): each
pair term is the reference's operation for operation, only the order of the
per-body sum differs, so the results agree to f64 rounding (relative 1e-12);
NaN for massless bodies, 0 for fixed ones, coincident bodies skipped."""
from __future__ import annotations

import numpy as np
import pytest

from test_direct_gpu import _vec

pytestmark = pytest.mark.gpu


def _state(n, seed):
    from physim_gb300 import ics
    s = ics.cube_with_stars(max(n - 2, 0), seed=seed, stars=ics.STARS_2[: min(n, 2)])
    if n > 9:
        s["fixed"][n // 3] = 1
        s["mass"][n // 7] = 0.0
        for k in range(n // 2, n // 2 + 3):
            s[k]["x"], s[k]["y"], s[k]["z"] = 0.125, -0.25, 0.375
    return s


@pytest.mark.parametrize("gravity", ["simple_astro", "astro2", "astro"])
@pytest.mark.parametrize("n", [1, 3, 257, 3001, 20000])
def test_f64_sample_matches_oracle(oracle_mod, gravity, n):
    import physim_gb300 as pg
    s = _state(n, seed=n)
    idx = np.unique(np.concatenate([np.arange(min(n, 5)), np.arange(n - min(n, 5), n),
                                    np.random.default_rng(n).integers(0, n, 40)]))
    with pg.Simulation(s, pg.SimConfig(gravity=gravity, e=0.01)) as sim:
        got = sim.accelerations_f64(idx)
    want = oracle_mod.simple_astro_sample(s, 0.01, idx)
    g, w = _vec(got), _vec(want)
    nan = np.isnan(w).any(axis=1)
    assert np.array_equal(np.isnan(g).any(axis=1), nan)
    g, w = g[~nan], w[~nan]
    err = np.linalg.norm(g - w, axis=1) / np.maximum(np.linalg.norm(w, axis=1), 1e-300)
    assert np.all(err < 1e-12), err.max()


def test_f64_sample_after_steps_and_bad_index(oracle_mod):
    """The sample reads the current state; indices outside [0, n) are refused."""
    import physim_gb300 as pg
    s = _state(2000, seed=4)
    s["mass"][2000 // 7] = 1.0  # a massless body's NaN would spread through the steps
    with pg.Simulation(s, pg.SimConfig(gravity="simple_astro", e=0.01, dt=1e-5)) as sim:
        sim.step(3)
        cur = sim.download()
        got = sim.accelerations_f64([0, 1999, 1000])
        with pytest.raises(pg.PhysimError):
            sim.accelerations_f64([2000])
        with pytest.raises(pg.PhysimError):
            sim.accelerations_f64([-1])
    want = oracle_mod.simple_astro_sample(cur, 0.01, np.array([0, 1999, 1000]))
    assert np.allclose(_vec(got), _vec(want), rtol=1e-12, atol=0)
